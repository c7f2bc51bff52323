"""GPU parity: the CUDA path through the C-ABI against the CPU oracle and the golden fixtures.

Bit-exact where the reference's arithmetic is integer or FP64 in a fixed order (Morton keys,
sort order, node table, the FP64 walk, direct sum, potential terms, KDK); tolerances stated per
test for the FP32 walks.
"""
import os

import numpy as np
import pytest

from gravitas_gb300 import abi, ics
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
P = abi.ptr


@pytest.fixture(scope="module")
def ctx():
    c = abi.Context(0)
    yield c
    c.close()


def gpu_acc(ctx, s, theta, leaf, eps, walk, monopole=False, dm_off=False, acc=None):
    n = len(s["px"])
    ax, ay, az = (np.zeros(n) for _ in range(3)) if acc is None else (a.copy() for a in acc)
    par = abi.make_params(theta, eps, leaf, monopole, dm_off, walk)
    ctx.call("gbh_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]),
             P(s.get("kind")), P(s.get("alive")), P(ax), P(ay), P(az))
    return np.stack([ax, ay, az], axis=1)


def oracle_tree(s, theta, leaf, dm_off=False):
    return O.Tree(s["px"], s["py"], s["pz"], s["mass"], s.get("kind"), s.get("alive"), theta=theta, leaf=leaf,
                  dm_off=dm_off, workers=1)


def rel_err(got, want):
    return np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)


def random_state(n, seed, spread=1.0, kinds=False, dead=False):
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(n, 3)) * spread
    s = dict(px=p[:, 0].copy(), py=p[:, 1].copy(), pz=p[:, 2].copy(), mass=rng.uniform(0.5, 1.5, n))
    s["kind"] = rng.choice([0, 2, 3], n).astype(np.uint8) if kinds else np.zeros(n, np.uint8)
    s["alive"] = (rng.random(n) > 0.1).astype(np.uint8) if dead else np.ones(n, np.uint8)
    return s


def assert_tree_equal(ctx, s, theta, leaf, dm_off=False):
    t = oracle_tree(s, theta, leaf, dm_off)
    e = t.export()
    g = ctx.tree_export()
    assert np.array_equal(g["keys"], e["keys"]), "Morton keys differ"
    assert np.array_equal(g["order"], e["order"]), "sort order differs"
    assert len(g["nodes"]) == len(e["nodes"]), "node count differs"
    for f in abi.NODE_DTYPE.names:
        assert np.array_equal(g["nodes"][f], e["nodes"][f]), f"node field {f} differs"
    return t


# ---------------------------------------------------------------- known answer

@pytest.mark.parametrize("walk", ["fp64", "plain", "mixed"])
def test_known_answer(ctx, walk):  # bh_test.go:137-147
    g = np.load(os.path.join(GOLDEN, "kat.npz"))
    s = {k: g[k] for k in ("px", "py", "pz", "mass", "kind", "alive")}
    a = gpu_acc(ctx, s, 0.0, 0, 0.0, walk)
    if walk == "fp64":
        assert np.array_equal(a, g["acc"])
    else:
        assert np.allclose(a, g["acc"], rtol=1e-6, atol=0)


# ---------------------------------------------------------------- tree, bit exact

@pytest.mark.parametrize("name", ["plummer", "disk"])
def test_tree_and_fp64_walk_match_golden(ctx, name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s = {k: g[k] for k in ("px", "py", "pz", "mass", "kind", "alive")}
    a = gpu_acc(ctx, s, float(g["theta"]), int(g["leaf"]), float(g["eps"]), "fp64")
    t = ctx.tree_export()
    assert np.array_equal(t["keys"], g["keys"])
    assert np.array_equal(t["order"], g["order"])
    assert np.array_equal(t["nodes"], g["nodes"])
    assert np.array_equal(a, g["acc"])


@pytest.mark.parametrize("n,leaf,seed,theta", [
    (1, 8, 0, 0.5), (2, 1, 1, 0.5), (7, 1, 2, 0.3), (100, 4, 3, 0.5), (1000, 8, 4, 0.5),
    (5000, 24, 5, 0.9), (33_000, 32, 6, 0.7), (50_000, 8, 7, 0.5)])
def test_tree_bit_exact_random(ctx, n, leaf, seed, theta):
    s = random_state(n, seed)
    a = gpu_acc(ctx, s, theta, leaf, 0.01, "fp64")
    t = assert_tree_equal(ctx, s, theta, leaf)
    assert np.array_equal(a, t.accelerations(0.01))


@pytest.mark.parametrize("n,leaf,seed", [(700_000, 16, 12), (1_000_000, 32, 13)])
def test_tree_bit_exact_both_sort_paths(ctx, n, leaf, seed):
    """Keys, order and the node table against the oracle at sizes on both sides of the switch
    between the one-sweep radix passes (capacity up to 786,432 bodies: 700k) and the three-launch
    passes (1M), in a fresh context so that the capacity is the state's own."""
    s = random_state(n, seed, kinds=True, dead=True)
    c = abi.Context(0)
    try:
        gpu_acc(c, s, 0.5, leaf, 0.01, "fp64")
        assert_tree_equal(c, s, 0.5, leaf)
    finally:
        c.close()


def test_tree_bit_exact_kinds_dead_dm_off(ctx):
    s = random_state(20_000, 11, kinds=True, dead=True)
    s["kind"][::97] = O.BLACK_HOLE
    rng = np.random.default_rng(3)
    init = [rng.normal(size=len(s["px"])) for _ in range(3)]
    a = gpu_acc(ctx, s, 0.6, 12, 0.02, "fp64", dm_off=True, acc=init)
    t = assert_tree_equal(ctx, s, 0.6, 12, dm_off=True)
    want = t.accelerations(0.02, acc=[x.copy() for x in init])
    assert np.array_equal(a, want)
    dead = s["alive"] == 0
    assert np.array_equal(a[dead], np.stack(init, axis=1)[dead])  # dead bodies untouched
    holes = (s["alive"] == 1) & (s["kind"] == O.BLACK_HOLE)
    assert np.all(a[holes] == 0)


def test_coincident_stars(ctx):  # bh_test.go:149-163
    n = 101
    s = dict(px=np.full(n, 1.0), py=np.full(n, 2.0), pz=np.full(n, 3.0), mass=np.ones(n))
    s["px"][-1] = s["py"][-1] = s["pz"][-1] = 0.0
    for walk in ("plain", "mixed", "fp64"):
        a = gpu_acc(ctx, s, 0.0, 0, 0.01, walk)
        assert not np.isnan(a).any()
    assert_tree_equal(ctx, s, 0.9, 24)
    nodes = ctx.tree_export()["nodes"]
    assert (nodes["hi"] - nodes["lo"])[nodes["first"] < 0].max() == 100


def test_clustered_and_far_apart(ctx):
    """Extreme dynamic range: two tight clumps 1e6 apart (deep trees, large coordinates)."""
    rng = np.random.default_rng(9)
    p = np.concatenate([rng.normal(size=(3000, 3)) * 1e-3, rng.normal(size=(3000, 3)) * 1e-3 + 1e6])
    s = dict(px=p[:, 0].copy(), py=p[:, 1].copy(), pz=p[:, 2].copy(), mass=np.ones(6000))
    a = gpu_acc(ctx, s, 0.5, 8, 1e-4, "fp64")
    t = assert_tree_equal(ctx, s, 0.5, 8)
    assert np.array_equal(a, t.accelerations(1e-4))
    # the mixed walk stays accurate far from the origin (group-relative coordinates)
    am = gpu_acc(ctx, s, 0.5, 8, 1e-4, "mixed")
    scale = np.linalg.norm(a, axis=1).mean()
    e = np.linalg.norm(am - a, axis=1) / scale
    assert np.median(e) < 1e-5 and e.max() < 1e-3


# ---------------------------------------------------------------- FP32 walks

@pytest.mark.parametrize("name,theta,leaf", [("plummer", 0.5, 8), ("disk", 0.9, 24)])
def test_fast_moments_agree_with_exact(ctx, name, theta, leaf):
    """The FP32 walks run on node moments formed in FP32 about a point inside each node; same
    node set and links, values within FP32 rounding of the reference's FP64 moments."""
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    s = {k: g[k] for k in ("px", "py", "pz", "mass", "kind", "alive")}
    gpu_acc(ctx, s, theta, leaf, float(g["eps"]), "mixed")
    fast = ctx.tree_export()["nodes"]
    ex = g["nodes"]
    for f in ("first", "next", "lo", "hi"):
        assert np.array_equal(fast[f], ex[f]), f
    side = max(np.ptp(s[k][(s["alive"] == 1) & (s["kind"] != O.BLACK_HOLE)]) for k in ("px", "py", "pz"))
    for f in ("x", "y", "z"):
        assert np.abs(fast[f] - ex[f]).max() <= 1e-6 * side, f
    assert np.allclose(fast["m"], ex["m"], rtol=1e-6, atol=0)
    assert np.allclose(fast["crit2"], ex["crit2"], rtol=1e-5, atol=0)
    qs = ("qxx", "qyy", "qzz", "qxy", "qxz", "qyz")
    qmax = np.max(np.abs(np.stack([ex[q] for q in qs])), axis=0)
    for q in qs:
        assert np.all(np.abs(fast[q] - ex[q]) <= 1e-5 * qmax + 1e-30), q


def test_plain_walk_matches_cpu_walk(ctx):  # gpu_test.go:8-21
    s = ics.test_disk(20000)
    stars = s["kind"] == O.STAR
    want = oracle_tree(s, 0.9, 24).accelerations(0.06)
    got = gpu_acc(ctx, s, 0.0, 0, 0.06, "plain")
    e = rel_err(got[stars], want[stars])
    assert np.median(e) <= 1e-5 and e.max() <= 1e-3


def test_mixed_walk_accuracy_vs_direct(ctx):
    """The warp walk opens a node wherever any star of its group would, so against the FP64
    direct sum it is at least as accurate as the reference's per-star walk."""
    s = ics.plummer(16384, seed=0)
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], eps=0.01)
    ref = oracle_tree(s, 0.5, 8).accelerations(0.01)
    e_ref = rel_err(ref, want)
    for walk in ("mixed", "plain"):
        got = gpu_acc(ctx, s, 0.5, 8, 0.01, walk)
        e = rel_err(got, want)
        rms, rms_ref = np.sqrt(np.mean(e ** 2)), np.sqrt(np.mean(e_ref ** 2))
        p99, p99_ref = np.percentile(e, 99), np.percentile(e_ref, 99)
        if walk == "mixed":
            assert rms <= rms_ref * 1.001 + 1e-7 and p99 <= p99_ref * 1.001 + 1e-7
        assert rms <= 2e-3
        # against the reference walk itself: within its own approximation error
        d = rel_err(got, ref)
        assert np.median(d) <= np.median(e_ref) and d.max() <= 5 * e_ref.max()


def test_mixed_walk_monopole_and_no_softening(ctx):
    s = random_state(3000, 21)
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], eps=0.0)
    for mono in (False, True):
        ref = oracle_tree(s, 0.5, 8).accelerations(0.0, monopole_only=mono)
        got = gpu_acc(ctx, s, 0.5, 8, 0.0, "mixed", monopole=mono)
        assert np.isfinite(got).all()
        e, e_ref = rel_err(got, want), rel_err(ref, want)
        assert np.sqrt(np.mean(e ** 2)) <= np.sqrt(np.mean(e_ref ** 2)) * 1.01 + 1e-6


@pytest.mark.parametrize("walk", ["fp64", "plain", "mixed"])
def test_walks_are_deterministic(ctx, walk):
    s = ics.plummer(30000, seed=2)
    a = gpu_acc(ctx, s, 0.5, 8, 0.01, walk)
    b = gpu_acc(ctx, s, 0.5, 8, 0.01, walk)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("paired", [False, True])
@pytest.mark.parametrize("n,group,scene", [(20000, 64, "galaxy"), (100000, 64, "galaxy"), (700, 64, "galaxy"),
                                           (20000, 64, "disk"), (20000, 32, "galaxy")])
def test_split_walk_adds_the_same_interactions(n, group, scene, paired):
    """With few groups each group's walk is split over several warps by source-star range (the
    list walk's split mode; the paired walk's with GBH_CFG_PAIRED, 64-star groups). The parts
    together add exactly the unsplit walk's interactions, in another order: the split forces
    equal the unsplit ones to FP32 summation rounding (global relative norm <= 1e-6, every star
    <= 1e-4), are as accurate against the FP64 direct sum, and repeat bit for bit."""
    if paired and group != 64:
        pytest.skip("the paired walk takes 64-star groups")
    ctx = abi.Context(0, abi.CFG_PAIRED if paired else 0)
    if scene == "galaxy":
        s = ics.galaxy(n, seed=3)
    else:  # two black holes, dead bodies, dark matter that pulls nothing
        s = ics.test_disk(n, seed=3)
        s["kind"][5::50] = 2
        s["alive"][7::97] = 0
    n = len(s["px"])
    dm_off = scene == "disk"
    whole = abi.Context(0, abi.CFG_NO_SPLIT | (abi.CFG_PAIRED if paired else 0))  # the same walk, unsplit
    try:
        par = abi.make_params(0.5, 0.02, 16, False, dm_off, "mixed", group_size=group)
        got = []
        for c in (ctx, whole):
            c.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None,
                   None, P(s["mass"]), P(s["kind"]), P(s["alive"]))
            c.call("gbh_state_accelerations", par)
            a = [np.zeros(n) for _ in range(3)]
            c.call("gbh_state_download", None, None, None, None, None, None, P(a[0]), P(a[1]), P(a[2]))
            got.append(np.stack(a, axis=1))
        split, unsplit = got
        assert not np.array_equal(split, unsplit)  # the split path ran
        assert np.linalg.norm(split - unsplit) <= 1e-6 * np.linalg.norm(unsplit)
        live = np.linalg.norm(unsplit, axis=1) > 0  # holes and dead bodies get 0 in both
        assert np.array_equal(split[~live], unsplit[~live]) and live.sum() > 0.9 * n
        assert (rel_err(split[live], unsplit[live]) <= 1e-4).all()
        if n <= 20000 and scene == "galaxy":
            want = O.direct(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.02)
            e_s, e_u = rel_err(split, want), rel_err(unsplit, want)
            assert abs(np.sqrt(np.mean(e_s ** 2)) - np.sqrt(np.mean(e_u ** 2))) <= 1e-3 * np.sqrt(np.mean(e_u ** 2))
        again = gpu_acc(ctx, s, 0.5, 16, 0.02, "mixed", dm_off=dm_off)
        first = gpu_acc(ctx, s, 0.5, 16, 0.02, "mixed", dm_off=dm_off)
        assert np.array_equal(again, first)
    finally:
        whole.close()
        ctx.close()


# ---------------------------------------------------------------- direct, potential, KDK

def test_direct_sum_bit_exact(ctx):
    s = random_state(3000, 5, kinds=True)
    s["kind"][::50] = O.BLACK_HOLE
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.02, dm_off=True)
    n = len(s["px"])
    out = np.zeros((3, n))
    par = abi.make_params(0, 0.02, 0, False, True, "fp64")
    ctx.call("gbh_direct_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s["kind"]),
             None, 0, P(out[0]), P(out[1]), P(out[2]))
    assert np.array_equal(out.T, want)
    tg = np.array([0, 17, 2999, 50], np.int64)
    sub = np.zeros((3, 4))
    ctx.call("gbh_direct_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s["kind"]),
             P(tg), 4, P(sub[0]), P(sub[1]), P(sub[2]))
    assert np.array_equal(sub.T, want[tg])


def test_potential_matches_oracle(ctx):
    g = np.load(os.path.join(GOLDEN, "disk.npz"))
    s = {k: g[k] for k in ("px", "py", "pz", "mass", "kind", "alive")}
    u = np.zeros(1)
    par = abi.make_params(float(g["theta"]), float(g["eps"]), int(g["leaf"]), False, False, "fp64")
    ctx.call("gbh_potential_energy", par, len(s["px"]), P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]),
             P(s["kind"]), P(s["alive"]), float(g["c"]), P(u))
    assert abs((u[0] - float(g["potential"])) / float(g["potential"])) <= 1e-12


@pytest.mark.parametrize("dm_off", [False, True])
def test_mixed_potential_matches_fp64_tree_potential(ctx, dm_off):
    """The mixed walk's potential (FP32 node terms, compensated sums, 64-star groups that open a
    node wherever any star would): against the exact pair sum at least as accurate as the
    reference's per-star tree estimate (the FP64 walk, bit for bit the oracle's), holes and the
    pair model included."""
    s = ics.test_disk(40000)
    s["kind"][3::11] = O.DARK_MATTER
    n = len(s["px"])
    u = {}
    for walk in ("fp64", "mixed"):
        out = np.zeros(1)
        par = abi.make_params(0.5, 0.06, 16, False, dm_off, walk)
        ctx.call("gbh_potential_energy", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s["kind"]),
                 P(s["alive"]), 10.0, P(out))
        u[walk] = out[0]
        ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                 P(s["mass"]), P(s["kind"]), P(s["alive"]))
        d = ctx.diagnostics(par, c=10.0)
        assert d["quality"] == 1 and d["potential"] == out[0], walk
    t = O.Tree(s["px"], s["py"], s["pz"], s["mass"], s["kind"], s["alive"], theta=0.5, leaf=16, dm_off=dm_off)
    assert abs(u["fp64"] - t.potential(0.06, c=10.0)) <= 1e-12 * abs(u["fp64"])
    exact = O.potential_exact(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.06, c=10.0, dm_off=dm_off)
    assert abs(u["mixed"] - exact) <= abs(u["fp64"] - exact) + 1e-7 * abs(exact), (u["mixed"], u["fp64"], exact)
    assert abs(u["mixed"] - exact) <= 2e-5 * abs(exact)


def test_kdk_fp64_bit_exact(ctx):
    g = np.load(os.path.join(GOLDEN, "kdk.npz"))
    st = {k: g[f"in_{k}"].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
    n = len(st["px"])
    acc = [np.zeros(n) for _ in range(3)]
    par = abi.make_params(float(g["theta"]), float(g["eps"]), int(g["leaf"]), False, False, "fp64")
    ctx.call("gbh_step_kdk", par, float(g["dt"]), int(g["nsteps"]), 0, n, P(st["px"]), P(st["py"]), P(st["pz"]),
             P(st["vx"]), P(st["vy"]), P(st["vz"]), P(acc[0]), P(acc[1]), P(acc[2]), P(st["mass"]), None, None)
    for k in ("px", "py", "pz", "vx", "vy", "vz"):
        assert np.array_equal(st[k], g[f"out_{k}"]), k
    for k, a in zip(("ax", "ay", "az"), acc):
        assert np.array_equal(a, g[f"out_{k}"]), k


def test_resident_steps_match_host_steps(ctx):
    s = ics.plummer(20000, seed=7)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, "mixed")
    host = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")}
    ctx.call("gbh_step_kdk", par, 1e-3, 3, 0, n, *[P(host[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax",
                                                                         "ay", "az")], P(s["mass"]), None, None)
    ctx.call("gbh_state_upload", n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["vx"]), P(s["vy"]), P(s["vz"]), None,
             None, None, P(s["mass"]), None, None)
    ctx.call("gbh_state_step", par, 1e-3, 3)
    dev = {k: np.zeros(n) for k in host}
    ctx.call("gbh_state_download", *[P(dev[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")])
    for k in host:
        assert np.array_equal(host[k], dev[k]), k


@pytest.mark.parametrize("walk", ["mixed", "plain", "fp64"])
def test_graph_replay_matches_plain_launches(ctx, walk):
    """Steps replayed from a captured CUDA graph equal steps launched kernel by kernel."""
    s = ics.plummer(30000, seed=11)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, walk)
    out = []
    for c in (ctx, abi.Context(0, abi.CFG_NO_GRAPHS)):
        c.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
               P(s["mass"]), None, None)
        c.call("gbh_state_step", par, 1e-3, 2)
        c.call("gbh_state_step", par, 1e-3, 1)
        t = c.timings()
        assert t["walk_ms"] > 0 and t["build_ms"] > 0
        st = {k: np.zeros(n) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")}
        c.call("gbh_state_download", *[P(st[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")])
        out.append(st)
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


def test_diagnostics_match_oracle_and_sums(ctx):  # diag.go:31-135, potential.go:12-42
    """1,502 bodies (two holes, c = 10): TotalEnergy's exact pair sum (n <= 30,000), bit for
    bit against the oracle's restatement; the other sums against numpy."""
    g = np.load(os.path.join(GOLDEN, "disk.npz"))
    s = {k: g[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass", "kind", "alive")}
    n = len(s["px"])
    ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
             P(s["mass"]), P(s["kind"]), P(s["alive"]))
    par = abi.make_params(float(g["theta"]), float(g["eps"]), int(g["leaf"]), False, False, "fp64")
    d = ctx.diagnostics(par, c=float(g["c"]))
    m, v = s["mass"], np.stack([s["vx"], s["vy"], s["vz"]], 1)
    x = np.stack([s["px"], s["py"], s["pz"]], 1)
    c = float(g["c"])
    u2 = (v * v).sum(1)
    kin = (m * u2 / (np.sqrt(1 + u2 / c ** 2) + 1)).sum()
    assert abs(d["kinetic"] - kin) <= 1e-12 * abs(kin)
    assert d["quality"] == 2
    assert d["potential"] == O.potential_exact(s["px"], s["py"], s["pz"], m, s["kind"], eps=float(g["eps"]), c=c)
    # the exact sum and the tree estimate agree to the tree's accuracy
    assert abs((d["potential"] - float(g["potential"])) / float(g["potential"])) <= 1e-3
    assert abs(d["total"] - (d["kinetic"] + d["potential"])) <= 1e-15 * abs(d["total"]) + 1e-300
    assert np.allclose(d["momentum"], (m[:, None] * v).sum(0), rtol=1e-12, atol=1e-14)
    assert np.allclose(d["angular_momentum"], (m[:, None] * np.cross(x, v)).sum(0), rtol=1e-12, atol=1e-14)
    assert np.allclose(d["center_of_mass"], (m[:, None] * x).sum(0) / m.sum(), rtol=1e-12, atol=1e-14)
    assert abs(d["mass"] - m.sum()) <= 1e-12 * m.sum()


BLOCK_FIELDS = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")


def upload_state(ctx, s):
    ctx.call("gbh_state_upload", len(s["px"]), *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None,
             None, P(s["mass"]), None, None)


def download_state(ctx, n):
    st = {k: np.zeros(n) for k in BLOCK_FIELDS}
    ctx.call("gbh_state_download", *[P(st[k]) for k in BLOCK_FIELDS])
    return st


@pytest.mark.parametrize("walk", ["fp64", "mixed"])
def test_block_steps_one_level_is_global_step(ctx, walk):
    s = ics.plummer(20000, seed=12)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, walk)
    upload_state(ctx, s)
    ctx.call("gbh_state_step", par, 1e-2, 3)
    want = download_state(ctx, n)
    upload_state(ctx, s)
    st = ctx.step_block(par, 1e-2, 0.025, 1, 3)
    got = download_state(ctx, n)
    assert st["substeps"] == 3 and st["evaluations"] == 3 * n
    for k in BLOCK_FIELDS:
        assert np.array_equal(want[k], got[k]), k


def test_block_steps_fp64_bit_exact_with_oracle(ctx):
    s = ics.plummer(4096, seed=13)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, "fp64")
    upload_state(ctx, s)
    st = ctx.step_block(par, 2e-2, 0.025, 6, 2)
    got = download_state(ctx, n)
    ref = {k: s[k].copy() for k in (*BLOCK_FIELDS, "mass")}
    events, walked = O.block_kdk(ref, dt=2e-2, eta=0.025, levels=6, eps=0.01, theta=0.5, leaf=8, nsteps=2, workers=1)
    assert (st["substeps"], st["evaluations"]) == (events, walked)
    for k in BLOCK_FIELDS:
        assert np.array_equal(got[k], ref[k]), k


def test_block_steps_conserve_energy_at_fewer_evaluations(ctx):
    """Plummer sphere, mixed walk: block steps with 6 levels conserve energy about as well as
    global steps at the finest step, while walking far fewer stars."""
    s = ics.plummer(16384, seed=0)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, "mixed")
    T = 1.6e-2
    upload_state(ctx, s)
    e0 = ctx.diagnostics(par)["total"]
    st = ctx.step_block(par, T, 0.025, 6, 10)
    e_block = ctx.diagnostics(par)["total"]
    upload_state(ctx, s)
    ctx.call("gbh_state_step", par, T / 32, 320)
    e_fine = ctx.diagnostics(par)["total"]
    d_block, d_fine = abs((e_block - e0) / e0), abs((e_fine - e0) / e0)
    assert st["evaluations"] < 0.5 * 320 * n
    assert d_block <= max(5 * d_fine, 2e-5)


def test_block_steps_reject_holes(ctx):
    """Holes take the split step (tests/test_gpu_split.py); block steps do not cover them."""
    s = ics.test_disk(500)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.06, 8, False, False, "mixed")
    ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
             P(s["mass"]), P(s["kind"]), P(s["alive"]))
    with pytest.raises(abi.GbhError) as ei:
        ctx.step_block(par, 1e-2, 0.025, 6, 1)
    assert ei.value.code == abi.ERR_UNSUPPORTED


def test_bad_arguments_are_errors(ctx):
    s = random_state(10, 1)
    with pytest.raises(abi.GbhError) as ei:
        gpu_acc(ctx, s, 1.5, 8, 0.01, "mixed")
    assert ei.value.code == abi.ERR_ARG
    with pytest.raises(abi.GbhError):
        gpu_acc(ctx, s, 0.5, 8, -1.0, "mixed")
    # the context stays usable
    a = gpu_acc(ctx, s, 0.5, 8, 0.01, "fp64")
    assert np.isfinite(a).all()


def test_empty_state(ctx):
    s = dict(px=np.zeros(0), py=np.zeros(0), pz=np.zeros(0), mass=np.zeros(0))
    assert gpu_acc(ctx, s, 0.5, 8, 0.01, "mixed").shape == (0, 3)
    s = dict(px=np.zeros(5), py=np.zeros(5), pz=np.zeros(5), mass=np.ones(5), kind=np.full(5, 1, np.uint8))
    assert np.all(gpu_acc(ctx, s, 0.5, 8, 0.01, "mixed") == 0)  # holes only: no stars, all zero


def test_mixed_walk_group_32_accuracy_and_determinism(ctx):
    """32-star groups: one star per lane. Same accuracy class as 64-star groups against the FP64
    direct sum, deterministic, and never less accurate per star than the group-64 bound allows."""
    s = ics.plummer(20000, seed=21)
    n = len(s["px"])
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], eps=0.01, targets=np.arange(0, n, 7))
    out = {}
    for g in (64, 32):
        a = [np.zeros(n) for _ in range(3)]
        par = abi.make_params(0.5, 0.01, 8, False, False, "mixed", group_size=g)
        for _ in range(2):
            b = [np.zeros(n) for _ in range(3)]
            ctx.call("gbh_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), None, None,
                     P(b[0]), P(b[1]), P(b[2]))
            if a[0].any():
                assert all(np.array_equal(x, y) for x, y in zip(a, b)), g
            a = b
        got = np.stack(a, 1)[::7]
        e = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
        out[g] = np.sqrt(np.mean(e ** 2))
    assert out[32] < 2e-3 and out[64] < 2e-3, out
    with pytest.raises(abi.GbhError) as ei:
        ctx.call("gbh_accelerations", abi.make_params(0.5, 0.01, 8, group_size=48), n, P(s["px"]), P(s["py"]),
                 P(s["pz"]), P(s["mass"]), None, None, P(np.zeros(n)), P(np.zeros(n)), P(np.zeros(n)))
    assert ei.value.code == abi.ERR_ARG


def test_autotune_single_system(ctx):
    s = ics.plummer(30000, seed=22)
    n = len(s["px"])
    ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
             P(s["mass"]), None, None)
    base = abi.make_params(0.5, 0.01, 8, False, False, "mixed")
    best, table = ctx.autotune(base, rms_bound=2e-3, sample=1024, reps=2, strict=True)
    assert len(table) == 3 * 4 * 4  # groups 64 and 32, each at list depths 24 and 56
    assert {(e["theta"], e["leaf_size"], e["group_size"], e["list_depth"]) for e in table} == {
        (t, l, g, d) for t in (0.4, 0.5, 0.7) for l in (4, 8, 16, 32) for g in (64, 32) for d in (24, 56)}
    for e in table:  # the error estimate does not depend on the timing
        assert 0 < e["rms_err"] < 2e-2 and e["ms"] > 0 and e["build_ms"] > 0 and e["walk_ms"] > 0
    chosen = [e for e in table if (e["theta"], e["leaf_size"], e["group_size"], e["list_depth"]) ==
              (best.theta, best.leaf_size, best.group_size, best.list_depth)][0]
    assert chosen["meets"] and chosen["ms"] == min(e["ms"] for e in table if e["meets"])
    # an unreachable bound: the most accurate candidate and GBH_ERR_LIMIT
    best2, table2 = ctx.autotune(base, thetas=[0.7], leaves=[16], groups=[64], rms_bound=1e-9, sample=64, reps=1)
    assert len(table2) == 2 and not any(e["meets"] for e in table2) and best2.theta == 0.7
    with pytest.raises(abi.GbhError) as ei:
        ctx.autotune(base, thetas=[0.7], leaves=[16], groups=[64], rms_bound=1e-9, sample=64, reps=1, strict=True)
    assert ei.value.code == abi.ERR_LIMIT
    # the state still steps with the chosen parameters
    ctx.call("gbh_state_step", best, 1e-3, 2)


def test_autotune_needs_a_state():
    c = abi.Context(0)
    try:
        with pytest.raises(abi.GbhError) as ei:
            c.autotune(abi.make_params(0.5, 0.01, 8))
        assert ei.value.code == abi.ERR_STATE
    finally:
        c.close()


def test_blocking_sync_frees_the_waiting_thread():
    """GBH_CFG_BLOCKING_SYNC: a thread waiting in a call sleeps instead of spinning (the process
    uses far less CPU time than the call's wall time) and the results are unchanged."""
    import time
    s = ics.plummer(1 << 19, seed=31)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, "mixed")
    out = {}
    for flags in (0, abi.CFG_BLOCKING_SYNC):
        c = abi.Context(0, flags)
        try:
            c.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                   P(s["mass"]), None, None)
            c.call("gbh_state_step", par, 1e-3, 2)  # warm-up: allocation and graph capture
            w0, c0 = time.perf_counter(), time.process_time()
            c.call("gbh_state_step", par, 1e-3, 40)
            wall, cpu = time.perf_counter() - w0, time.process_time() - c0
            st = {k: np.zeros(n) for k in ("px", "vx", "ax")}
            c.call("gbh_state_download", P(st["px"]), None, None, P(st["vx"]), None, None, P(st["ax"]), None, None)
            out[flags] = (wall, cpu, st)
        finally:
            c.close()
    wall, cpu, st = out[abi.CFG_BLOCKING_SYNC]
    assert cpu < 0.5 * wall, (cpu, wall)
    for k in st:
        assert np.array_equal(st[k], out[0][2][k]), k


def test_diagnostics_switch_to_the_tree_above_30000_bodies(ctx):
    """diag.go:16-40: exact up to exactEnergyLimit = 30,000 bodies, the tree potential above."""
    for n, quality in ((30000, 2), (30001, 1)):
        s = ics.plummer(n, seed=41)
        s["kind"][::97] = O.DARK_MATTER
        ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                 P(s["mass"]), P(s["kind"]), P(s["alive"]))
        par = abi.make_params(0.5, 0.01, 8, False, True, "fp64")
        d = ctx.diagnostics(par)
        assert d["quality"] == quality
        exact = O.potential_exact(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.01, dm_off=True)
        if quality == 2:
            assert d["potential"] == exact
        else:
            t = O.Tree(s["px"], s["py"], s["pz"], s["mass"], s["kind"], s["alive"], theta=0.5, leaf=8, dm_off=True)
            assert abs(d["potential"] - t.potential(0.01)) <= 1e-12 * abs(exact)
            assert abs(d["potential"] - exact) <= 1e-4 * abs(exact)


def test_no_device_allocation_after_warm_up():
    """The context owns grow-only device buffers: once every entry point has run on a state,
    repeating the calls on the same sizes allocates nothing (the device's free memory stays)."""
    torch = pytest.importorskip("torch")
    s = ics.test_disk(3000)
    n = len(s["px"])
    F = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")
    tg = np.arange(0, n, 5, dtype=np.int64)
    out = [np.zeros(len(tg)) for _ in range(3)]
    c = abi.Context(0)
    try:
        def every_call():
            par = abi.make_params(0.5, 0.06, 8, False, False, "mixed")
            a = [np.zeros(n) for _ in range(3)]
            c.call("gbh_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s["kind"]),
                   P(s["alive"]), P(a[0]), P(a[1]), P(a[2]))
            c.call("gbh_direct_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s["kind"]),
                   P(tg), len(tg), P(out[0]), P(out[1]), P(out[2]))
            st = {k: s[k].copy() for k in F}
            c.call("gbh_step_kdk", par, 4e-3, 2, 0, n, *[P(st[k]) for k in F], P(s["mass"]), P(s["kind"]),
                   P(s["alive"]))
            c.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                   P(s["mass"]), P(s["kind"]), P(s["alive"]))
            c.call("gbh_state_step", par, 4e-3, 2)
            c.diagnostics(par, c=0.0)
            c.call("gbh_state_accelerations", par)
            c.autotune(par, thetas=[0.5], leaves=[8, 16], groups=[64], sample=256, reps=1)
            x0 = np.stack([s["px"], s["py"], s["pz"]], 1)
            v0 = np.stack([s["vx"], s["vy"], s["vz"]], 1)
            xT, _ = c.fwd_save(x0, v0, s["mass"], 1e-3, 0.06, 4, 2)
            c.bwd(xT, None)
        every_call()
        every_call()
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        for _ in range(3):
            every_call()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(0)[0] == free0
    finally:
        c.close()


def test_snapshot_save_load_continues_bit_identically(tmp_path):
    """save_test.go:17-52 through the library: a run saved to a .gravitas snapshot and loaded
    continues exactly as the run that was not interrupted (holes included: split steps)."""
    from gravitas_gb300.sim import Params, Simulation, Solver, State
    s = ics.test_disk(3000)
    solver = Solver(theta=0.5, leaf_size=8)
    a = Simulation(State.from_dict(s), solver, Params(dt=4e-3, softening=0.06))
    b = Simulation(State.from_dict(s), solver, Params(dt=4e-3, softening=0.06))
    a.step(6)
    b.step(3)
    path = os.path.join(str(tmp_path), "run.gravitas")
    b.save(path)
    c = Simulation.load(path, solver)
    assert c.steps == 3 and c.acc_valid
    c.step(3)
    for f in ("pos_x", "pos_y", "pos_z", "vel_x", "vel_y", "vel_z", "acc_x", "acc_y", "acc_z"):
        assert np.array_equal(getattr(a.state, f), getattr(c.state, f)), f


def test_evolve_driver_continues_a_snapshot(tmp_path):
    """The headless driver: evolve a scene to t, continue the written snapshot to 2t; the result
    equals one run to 2t (steps are deterministic and the snapshot keeps the forces)."""
    from gravitas_gb300 import evolve, snapshot
    d = str(tmp_path)
    a, b, c = (os.path.join(d, f) for f in ("a.gravitas", "b.gravitas", "c.gravitas"))
    common = ["--scene", "plummer", "--n", "4096", "--dt", "1e-3", "--chunk", "7"]
    assert evolve.main(common + ["-t", "0.02", "-o", a]) == 0
    assert evolve.main(["--in", a, "-t", "0.04", "-o", b, "--chunk", "7"]) == 0
    assert evolve.main(common + ["-t", "0.04", "-o", c]) == 0
    sb, _, mb = snapshot.load_state(b)
    sc, _, mc = snapshot.load_state(c)
    assert mb["Steps"] == mc["Steps"] == 40
    for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az"):
        assert np.array_equal(sb[k], sc[k]), k


def test_resident_calls_need_a_state():
    """Calls on the resident state fail with GBH_ERR_STATE before an upload, and after a call that
    reused the state buffers for host arrays (gbh_accelerations)."""
    c = abi.Context(0)
    try:
        par = abi.make_params(0.5, 0.01, 8)
        for call in (lambda: c.diagnostics(par), lambda: c.call("gbh_state_step", par, 1e-3, 1),
                     lambda: c.call("gbh_state_accelerations", par)):
            with pytest.raises(abi.GbhError) as ei:
                call()
            assert ei.value.code == abi.ERR_STATE
        s = ics.plummer(1000, seed=3)
        n = len(s["px"])
        c.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
               P(s["mass"]), None, None)
        c.diagnostics(par)
        a = [np.zeros(n) for _ in range(3)]
        c.call("gbh_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), None, None,
               P(a[0]), P(a[1]), P(a[2]))
        with pytest.raises(abi.GbhError) as ei:
            c.diagnostics(par)
        assert ei.value.code == abi.ERR_STATE
    finally:
        c.close()


def test_results_do_not_depend_on_a_contexts_history():
    """Buffers only grow, so a context that held a larger state keeps larger buffers; the walk's
    launch shape (split parts, group order) is a function of the inputs alone, so block steps and
    forces of the same state are bit-identical in a fresh context and in one that held 200,000
    bodies before."""
    small = ics.galaxy(60000, seed=6)
    big = ics.galaxy(200000, seed=7)
    par = abi.make_params(0.5, 0.02, 16, False, False, "mixed")
    out = []
    for history in (None, big):
        c = abi.Context(0)
        try:
            if history is not None:
                upload_state(c, history)
                c.step_block(par, 1.6e-2, 0.025, 6, 1)
            upload_state(c, small)
            c.step_block(par, 1.6e-2, 0.025, 6, 2)
            st = download_state(c, len(small["px"]))
            c.call("gbh_state_accelerations", par)
            st["forces"] = download_state(c, len(small["px"]))["ax"]
            out.append(st)
        finally:
            c.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
