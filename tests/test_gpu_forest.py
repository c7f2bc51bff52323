"""GPU tests of the batched forest: many independent systems in one state, one build and one
walk launch. Each system's tree and forces must be exactly those of the system alone."""
import numpy as np
import pytest

from gravitas_gb300 import abi, ics
from oracle import oracle as O

pytestmark = pytest.mark.gpu
P = abi.ptr
F9 = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")


@pytest.fixture(scope="module")
def ctx():
    c = abi.Context(0)
    yield c
    c.close()


def small_forest():
    """Mixed systems, with the edge cases: an empty system, a one-star system, a system of
    coincident stars, one with dead bodies and dark matter."""
    parts = [ics.plummer(3000, seed=1), ics.plummer(1, seed=2), ics.galaxy(5000, seed=3),
             {k: v[:0] for k, v in ics.plummer(5, seed=4).items()}, ics.plummer(777, seed=5, a=0.1)]
    coinc = ics.plummer(40, seed=6)
    for k in ("px", "py", "pz"):
        coinc[k][:] = 1.5
    parts.append(coinc)
    dead = ics.plummer(2000, seed=7)
    dead["alive"][::7] = 0
    dead["kind"][::5] = O.DARK_MATTER
    parts.append(dead)
    offsets = np.cumsum([0] + [len(p["px"]) for p in parts]).astype(np.int64)
    state = {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}
    for p, (lo, hi) in zip(parts, zip(offsets[:-1], offsets[1:])):  # offset each system in space
        state["px"][lo:hi] += 100.0 * len(p["px"]) % 37
    return state, offsets


def upload_forest(ctx, s, off):
    ctx.forest_upload(off, s["px"], s["py"], s["pz"], s["vx"], s["vy"], s["vz"], s["mass"], s["kind"], s["alive"])


def download(ctx, n):
    st = {k: np.zeros(n) for k in F9}
    ctx.call("gbh_state_download", *[P(st[k]) for k in F9])
    return st


@pytest.mark.parametrize("theta,leaf", [(0.5, 8), (0.9, 24)])
def test_forest_trees_and_fp64_forces_equal_each_system_alone(ctx, theta, leaf):
    s, off = small_forest()
    nsys, n = len(off) - 1, int(off[-1])
    upload_forest(ctx, s, off)
    par = abi.make_params(theta, 0.01, leaf, False, True, "fp64")
    ctx.call("gbh_state_accelerations", par)
    got = download(ctx, n)
    tree = ctx.tree_export()
    stars, nodes = ctx.forest_layout(nsys)
    for q in range(nsys):
        lo, hi = off[q], off[q + 1]
        sub = {k: s[k][lo:hi] for k in s}
        t = O.Tree(sub["px"], sub["py"], sub["pz"], sub["mass"], sub["kind"], sub["alive"], theta=theta, leaf=leaf,
                   dm_off=True, workers=1)
        e = t.export()
        a, b = stars[q]
        assert b - a == t.nstars, q
        assert np.array_equal(tree["keys"][a:b], e["keys"]), q
        assert np.array_equal(tree["order"][a:b] - lo, e["order"]), q
        c, d = nodes[q]
        assert d - c == t.nnodes, q
        mine = tree["nodes"][c:d].copy()
        for f in ("first", "next"):
            m = mine[f] >= 0
            mine[f][m] -= c
        for f in ("lo", "hi"):
            mine[f] -= a
        for f in abi.NODE_DTYPE.names:
            assert np.array_equal(mine[f], e["nodes"][f]), (q, f)
        want = t.accelerations(0.01)
        alive = sub["alive"] == 1
        for k, j in zip(("ax", "ay", "az"), range(3)):
            assert np.array_equal(got[k][lo:hi][alive], want[:, j][alive]), (q, k)


@pytest.mark.parametrize("walk,group", [("mixed", 64), ("mixed", 32), ("plain", 0), ("fp64", 0)])
def test_forest_steps_equal_each_system_stepped_alone(walk, group):
    """Bit-identical: the same per-system trees, the same 64- (32-) star groups, the same kernels
    (a forest never splits a group's walk over several warps; the small systems alone would, so
    this comparison runs with GBH_CFG_NO_SPLIT)."""
    ctx = abi.Context(0, abi.CFG_NO_SPLIT)
    s, off = ics.forest(nsys=6, seed=3, nmin=500, nmax=4000)
    nsys, n = len(off) - 1, int(off[-1])
    par = abi.make_params(0.5, 0.02, 8, False, False, walk, group_size=group)
    upload_forest(ctx, s, off)
    ctx.call("gbh_state_step", par, 1e-3, 3)
    forest = download(ctx, n)
    for q in range(nsys):
        lo, hi = off[q], off[q + 1]
        sub = {k: np.ascontiguousarray(s[k][lo:hi]) for k in s}
        ctx.call("gbh_state_upload", hi - lo, *[P(sub[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None,
                 None, P(sub["mass"]), P(sub["kind"]), P(sub["alive"]))
        ctx.call("gbh_state_step", par, 1e-3, 3)
        alone = download(ctx, hi - lo)
        for k in F9:
            assert np.array_equal(forest[k][lo:hi], alone[k]), (q, k)
    ctx.close()


def test_forest_mixed_accuracy_per_system(ctx):
    s, off = ics.forest(nsys=8, seed=4, nmin=1000, nmax=6000)
    n = int(off[-1])
    upload_forest(ctx, s, off)
    ctx.call("gbh_state_accelerations", abi.make_params(0.5, 0.01, 8, False, False, "mixed"))
    got = download(ctx, n)
    a = np.stack([got["ax"], got["ay"], got["az"]], 1)
    for q in range(len(off) - 1):
        lo, hi = off[q], off[q + 1]
        want = O.direct(s["px"][lo:hi], s["py"][lo:hi], s["pz"][lo:hi], s["mass"][lo:hi], s["kind"][lo:hi], eps=0.01)
        e = np.linalg.norm(a[lo:hi] - want, axis=1) / np.linalg.norm(want, axis=1)
        assert np.sqrt(np.mean(e ** 2)) < 2e-3, q


def test_forest_upload_validates_offsets(ctx):
    s, off = ics.forest(nsys=3, seed=5, nmin=100, nmax=200)
    bad = off.copy()
    bad[1], bad[2] = bad[2], bad[1]
    with pytest.raises(abi.GbhError) as ei:
        upload_forest(ctx, s, bad)
    assert ei.value.code == abi.ERR_ARG
    upload_forest(ctx, s, off)
    with pytest.raises(abi.GbhError) as ei:
        ctx.step_block(abi.make_params(0.5, 0.01, 8), 1e-3, 0.025, 3, 1)
    assert ei.value.code == abi.ERR_UNSUPPORTED


def test_autotune_on_a_forest_meets_the_bound(ctx):
    s, off = ics.forest(nsys=5, seed=8, nmin=800, nmax=5000)
    n = int(off[-1])
    upload_forest(ctx, s, off)
    base = abi.make_params(0.5, 0.01, 8, False, False, "mixed")
    best, table = ctx.autotune(base, thetas=[0.4, 0.7], leaves=[8, 16], groups=[64, 32], rms_bound=2e-3,
                               sample=512, reps=2, strict=True)
    assert len(table) == 16  # groups 64 and 32 (the list walk), each at two list depths
    meets = [e for e in table if e["meets"]]
    assert meets and min(e["ms"] for e in meets) == min(
        e["ms"] for e in meets if (e["theta"], e["leaf_size"], e["group_size"], e["list_depth"]) ==
        (best.theta, best.leaf_size, best.group_size, best.list_depth))
    # the chosen parameters step the forest, and its forces meet the bound per system
    ctx.call("gbh_state_step", best, 1e-3, 1)
    ctx.call("gbh_state_accelerations", best)
    got = download(ctx, n)
    a = np.stack([got["ax"], got["ay"], got["az"]], 1)
    for q in range(len(off) - 1):
        lo, hi = int(off[q]), int(off[q + 1])
        t = np.arange(0, hi - lo, max(1, (hi - lo) // 200))
        want = O.direct(got["px"][lo:hi], got["py"][lo:hi], got["pz"][lo:hi], s["mass"][lo:hi], s["kind"][lo:hi],
                        eps=0.01, targets=t)
        e = np.linalg.norm(a[lo:hi][t] - want, axis=1) / np.linalg.norm(want, axis=1)
        assert np.sqrt(np.mean(e ** 2)) < 4e-3, q


def test_longest_first_order_changes_no_bit(ctx):
    """The mixed walk launches its groups in the order the previous walk's group costs give
    (longest first) unless GBH_CFG_NO_LPT; every group sums only its own interactions, so the
    order changes no result, for a forest and for a single system."""
    s, off = ics.forest(nsys=6, seed=5, nmin=500, nmax=8000)
    n = int(off[-1])
    par = abi.make_params(0.5, 0.02, 16, False, False, "mixed")
    other = abi.Context(0, abi.CFG_NO_LPT)
    try:
        got = []
        for c in (ctx, other):
            upload_forest(c, s, off)
            c.call("gbh_state_step", par, 1e-3, 4)
            got.append(download(c, n))
        for k in F9:
            assert np.array_equal(got[0][k], got[1][k]), k
        m = ics.merger(60000, seed=2)
        got = []
        for c in (ctx, other):
            c.call("gbh_state_upload", 60000, *[P(m[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None,
                   None, P(m["mass"]), None, None)
            c.call("gbh_state_step", par, 1e-3, 4)
            got.append(download(c, 60000))
        for k in F9:
            assert np.array_equal(got[0][k], got[1][k]), k
    finally:
        other.close()
