"""CPU tests pinning the oracle to the reference's own tests.

The reference (Go) cannot run here and stores no golden vectors for this path; its tests are a
known-answer test and relations. Each test below restates one of them against the C++ oracle
(internal/sim/bh/bh_test.go, gpu_test.go, internal/sim/direct/direct_test.go), then checks the
committed fixtures of tests/golden/ (made by tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

from gravitas_gb300 import ics
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel_errors(got, want):
    """Median and max of |got - want| / |want| per body (bh_test.go:76-86)."""
    e = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    e = np.sort(e)
    return e[len(e) // 2], e[-1]


def tree_of(s, **kw):
    return O.Tree(s["px"], s["py"], s["pz"], s["mass"], s.get("kind"), s.get("alive"), **kw)


def test_morton_key_interleaves_bits():  # bh_test.go:16-31
    def naive(x, y, z):
        k = 0
        for b in range(21):
            k |= ((x >> b) & 1) << (3 * b + 2) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b)
        return k

    rng = np.random.default_rng(12)
    for x, y, z in rng.integers(0, 1 << 21, size=(1000, 3)):
        assert O.morton_key(int(x), int(y), int(z)) == naive(int(x), int(y), int(z))


def test_radix_sort():  # bh_test.go:33-52
    rng = np.random.default_rng(34)
    keys = rng.integers(0, 1 << 63, size=5000, dtype=np.uint64)
    k, i = O.radix_sort(keys, np.arange(5000, dtype=np.int32))
    assert np.all(k[1:] >= k[:-1])
    assert np.array_equal(keys[i], k)


def test_parallel_radix_sort_is_stable_and_correct():  # bh_test.go:353-367
    rng = np.random.default_rng(89)
    keys = rng.integers(0, 1 << 20, size=200_000, dtype=np.uint64) << np.uint64(40)
    idx = np.arange(len(keys), dtype=np.int32)
    k1, i1 = O.radix_sort(keys, idx, workers=1)
    k7, i7 = O.radix_sort(keys, idx, workers=7)
    assert np.array_equal(k1, k7) and np.array_equal(i1, i7)
    # stable: equal keys keep index order
    same = k1[1:] == k1[:-1]
    assert np.all(i1[1:][same] > i1[:-1][same])
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(i1, order)


def test_solver_leaves_holes_to_the_integrator():  # bh_test.go:137-147 (known answer)
    g = np.load(os.path.join(GOLDEN, "kat.npz"))
    t = O.Tree(g["px"], g["py"], g["pz"], g["mass"], g["kind"], g["alive"])
    assert np.array_equal(t.accelerations(0.0), g["acc"])
    assert np.array_equal(g["acc"], [[2, 0, 0], [-1, 0, 0], [0, 0, 0]])


def test_coincident_stars_do_not_recurse_forever():  # bh_test.go:149-163
    n = 101
    px, py, pz = np.full(n, 1.0), np.full(n, 2.0), np.full(n, 3.0)
    px[-1] = py[-1] = pz[-1] = 0.0
    t = O.Tree(px, py, pz, np.ones(n))
    a = t.accelerations(0.01)
    assert not np.isnan(a).any()
    nodes = t.export()["nodes"]
    leaves = nodes[nodes["first"] < 0]
    assert (leaves["hi"] - leaves["lo"]).max() == 100  # oversize leaf at the depth cap


def test_tiny_theta_matches_direct():  # bh_test.go:88-97
    s = ics.test_disk(3000)
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.06)
    got = tree_of(s, theta=1e-9).accelerations(0.06)
    stars = s["kind"] != O.BLACK_HOLE
    _, mx = rel_errors(got[stars], want[stars])
    assert mx < 1e-10
    assert np.all(got[~stars] == 0) and np.all(want[~stars] == 0)


def test_default_theta_accuracy():  # bh_test.go:124-135 (star-star part; holes are summed outside)
    s = ics.test_disk(5000)
    stars = s["kind"] == O.STAR
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.06)[stars]
    got = tree_of(s).accelerations(0.06)[stars]
    med, mx = rel_errors(got, want)
    assert med < 4e-3 and mx < 6e-2


@pytest.mark.parametrize("n", [4000, 40_000, 60_000])
def test_parallel_build_is_bit_identical(n):  # bh_test.go:192-199, 369-394
    s = ics.test_disk(n)
    t1, t8 = tree_of(s, workers=1), tree_of(s, workers=8)
    assert t1.nnodes == t8.nnodes
    assert np.array_equal(t1.accelerations(0.06, workers=1), t8.accelerations(0.06, workers=8))
    u1, u8 = t1.potential(0.06, c=10), t8.potential(0.06, c=10)
    assert abs((u1 - u8) / u1) <= 1e-12


def test_potential_energy_matches_exact():  # bh_test.go:280-293
    s = ics.test_disk(3000)
    want = O.potential_exact(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=0.06, c=10)
    got = tree_of(s, theta=1e-9).potential(0.06, c=10)
    assert abs((got - want) / want) < 1e-10
    got = tree_of(s, theta=0.9).potential(0.06, c=10)
    assert abs((got - want) / want) < 1e-3


def test_quadrupole_improves_far_field():  # bh_test.go:309-330
    s = ics.far_cluster()
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], eps=1e-3)[0]
    err = {}
    for mono in (True, False):
        got = tree_of(s, theta=0.95).accelerations(1e-3, monopole_only=mono)[0]
        err[mono] = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err[False] < err[True] / 5


def test_quadrupole_force_is_gradient_of_potential():  # bh_test.go:332-351
    s = ics.far_cluster()
    t = tree_of(s, theta=0.95)
    eps2, h = 1e-6, 1e-6
    x, y, z = 0.0, 0.5, 0.2
    a = t.walk_point(x, y, z, eps2)
    g = [(t.walk_potential_point(x + h * (d == 0), y + h * (d == 1), z + h * (d == 2), eps2) -
          t.walk_potential_point(x - h * (d == 0), y - h * (d == 1), z - h * (d == 2), eps2)) / (2 * h)
         for d in range(3)]
    assert np.all(np.abs(a - np.array(g)) <= 1e-6 * abs(a[0]))


def test_fp32_walk_matches_fp64_walk():  # gpu_test.go:8-21, on the CPU restatement of the Metal walk
    s = ics.test_disk(20000)
    t = tree_of(s)
    want = t.accelerations(0.06)
    e = t.export()
    got32 = t.walk_fp32(0.06).astype(np.float64)
    stars = s["kind"] == O.STAR
    got = np.zeros_like(want)
    got[e["order"]] = got32
    med, mx = rel_errors(got[stars], want[stars])
    assert med <= 1e-5 and mx <= 1e-3


def test_kepler_conservation():  # direct_test.go:37-63, KDK with the tree solver on two bodies
    e = 0.3
    st = dict(px=np.array([0.0, 1 - e]), py=np.zeros(2), pz=np.zeros(2), vx=np.zeros(2),
              vy=np.array([0.0, np.sqrt((1 + e) / (1 - e))]), vz=np.zeros(2), ax=np.zeros(2), ay=np.zeros(2),
              az=np.zeros(2), mass=np.array([1.0, 1e-12]))
    # a fixed central mass: a massive body at rest with negligible pull from the test body
    period = 2 * np.pi
    steps_per_orbit = 2000
    dt = period / steps_per_orbit

    def energy(s):
        dx, dy = s["px"][1] - s["px"][0], s["py"][1] - s["py"][0]
        v2 = (s["vx"][1] - s["vx"][0]) ** 2 + (s["vy"][1] - s["vy"][0]) ** 2
        return 0.5 * v2 - 1 / np.hypot(dx, dy)

    def ang(s):
        dx, dy = s["px"][1] - s["px"][0], s["py"][1] - s["py"][0]
        return dx * (s["vy"][1] - s["vy"][0]) - dy * (s["vx"][1] - s["vx"][0])

    e0, l0 = energy(st), ang(st)
    O.kdk(st, dt=dt, eps=0.0, theta=0.5, leaf=24, nsteps=steps_per_orbit * 20, workers=1)
    assert abs((energy(st) - e0) / e0) <= 1e-4
    assert abs(ang(st) - l0) <= 1e-10
    r = np.hypot(st["px"][1] - st["px"][0], st["py"][1] - st["py"][0])
    assert abs(r - 0.7) < 0.05


def test_momentum_conservation_direct():  # direct_test.go:65-75
    rng = np.random.default_rng(7)
    n = 1000
    p = rng.normal(size=(n, 3))
    m = rng.uniform(0.5, 1.5, n)
    a = O.direct(p[:, 0], p[:, 1], p[:, 2], m, eps=0.05)
    assert np.abs((m[:, None] * a).sum(axis=0)).max() <= 1e-12 * np.abs(m[:, None] * a).sum()


@pytest.mark.parametrize("name", ["plummer", "disk"])
def test_oracle_matches_golden(name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    t = O.Tree(g["px"], g["py"], g["pz"], g["mass"], g["kind"], g["alive"], theta=float(g["theta"]),
               leaf=int(g["leaf"]), workers=1)
    e = t.export()
    assert np.array_equal(e["keys"], g["keys"])
    assert np.array_equal(e["order"], g["order"])
    assert np.array_equal(e["nodes"], g["nodes"])
    assert np.array_equal(t.accelerations(float(g["eps"])), g["acc"])
    assert np.array_equal(np.array(t.counts(float(g["eps"]))), g["counts"])
    if "acc_fp32_sorted" in g:
        assert np.array_equal(t.walk_fp32(float(g["eps"])), g["acc_fp32_sorted"])


def test_oracle_kdk_matches_golden():
    g = np.load(os.path.join(GOLDEN, "kdk.npz"))
    st = {k: g[f"in_{k}"].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
    n = len(st["px"])
    st.update(ax=np.zeros(n), ay=np.zeros(n), az=np.zeros(n))
    O.kdk(st, dt=float(g["dt"]), eps=float(g["eps"]), theta=float(g["theta"]), leaf=int(g["leaf"]),
          nsteps=int(g["nsteps"]), workers=1)
    for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az"):
        assert np.array_equal(st[k], g[f"out_{k}"])


def test_node_table_invariants():
    """Structure of the reference's serial layout: children contiguous, skip pointers pre-order."""
    g = np.load(os.path.join(GOLDEN, "plummer.npz"))
    nodes = g["nodes"]
    n = len(g["keys"])
    assert nodes[0]["lo"] == 0 and nodes[0]["hi"] == n and nodes[0]["next"] == -1
    for i, nd in enumerate(nodes):
        if nd["first"] >= 0:
            c = nd["first"]
            lo = nd["lo"]
            while True:  # children tile the parent's range in order
                assert nodes[c]["lo"] == lo
                lo = nodes[c]["hi"]
                if nodes[c]["next"] != c + 1:
                    assert nodes[c]["next"] == nd["next"]
                    break
                c += 1
            assert lo == nd["hi"]
        else:
            assert nd["hi"] - nd["lo"] <= int(g["leaf"])


def test_block_steps_one_level_is_global_kdk():
    s = ics.plummer(1024, seed=5)
    g = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")}
    b = {k: s[k].copy() for k in g}
    O.kdk(g, dt=1e-2, eps=0.01, theta=0.5, leaf=8, nsteps=3, workers=1)
    events, walked = O.block_kdk(b, dt=1e-2, eta=0.025, levels=1, eps=0.01, theta=0.5, leaf=8, nsteps=3, workers=1)
    assert (events, walked) == (3, 3 * 1024)
    for k in g:
        assert np.array_equal(g[k], b[k]), k


def test_block_steps_rungs_follow_accelerations():
    """Denser regions take shorter steps: with 6 levels the walked stars per global step lie
    between one (all on rung 0) and 32 (all on the finest rung) per star."""
    s = ics.plummer(2048, seed=6)
    b = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")}
    events, walked = O.block_kdk(b, dt=2e-2, eta=0.025, levels=6, eps=0.01, theta=0.5, leaf=8, nsteps=2, workers=1)
    assert 2 < events <= 2 * 32
    assert 2 * 2048 < walked < 2 * 32 * 2048


# ---- adjoint of the KDK leapfrog with the direct-sum force (no reference counterpart; pinned by
# central finite differences in FP64, the pattern of pair_test.go:8 and bh_test.go:332-351) ----

def _adjoint_case(n=48, seed=3):
    s, targets = ics.adjoint_problem(n, seed=seed)
    return s, targets


def _loss_fd(s, targets, key, idx, h, dt, eps, nsteps):
    vals = []
    for sign in (1.0, -1.0):
        st = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
        st[key][idx] += sign * h
        O.kdk_direct(st, dt, eps, nsteps, workers=1)
        x = np.stack([st["px"], st["py"], st["pz"]], 1)
        vals.append(np.sum((x - targets) ** 2) / len(x))
    return (vals[0] - vals[1]) / (2 * h)


def test_adjoint_oracle_matches_central_differences():
    s, targets = _adjoint_case()
    dt, eps, nsteps = 1e-2, 0.05, 40
    st = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
    O.kdk_direct(st, dt, eps, nsteps, workers=1)
    x = np.stack([st["px"], st["py"], st["pz"]], 1)
    gx = 2 * (x - targets) / len(x)
    dx, dv, dm = O.adjoint_direct(s, dt, eps, nsteps, 7, gx, np.zeros_like(gx), workers=1)
    rng = np.random.default_rng(0)
    grads = {"px": dx[:, 0], "py": dx[:, 1], "vx": dv[:, 0], "vz": dv[:, 2], "mass": dm}
    for key, g in grads.items():
        for idx in rng.choice(len(g), 4, replace=False):
            fd = _loss_fd(s, targets, key, idx, 1e-4, dt, eps, nsteps)
            assert abs(g[idx] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(g).max()), (key, idx, g[idx], fd)


def test_adjoint_oracle_checkpoint_interval_does_not_change_bits():
    s, targets = _adjoint_case(n=40, seed=4)
    gx = np.random.default_rng(1).normal(size=(40, 3))
    gv = np.random.default_rng(2).normal(size=(40, 3))
    ref = O.adjoint_direct(s, 5e-3, 0.02, 23, 1, gx, gv, workers=1)
    for every in (4, 7, 23, 100):
        got = O.adjoint_direct(s, 5e-3, 0.02, 23, every, gx, gv, workers=1)
        for a, b in zip(ref, got):
            assert np.array_equal(a, b), every


# ---- hole-aware split step (split.go, c = 0) ----

def _three_body(r):
    z = np.zeros(3)
    return dict(px=np.array([0.0, r, 50.0]), py=z.copy(), pz=z.copy(), vx=z.copy(), vy=z.copy(), vz=z.copy(),
                ax=z.copy(), ay=z.copy(), az=z.copy(), mass=np.array([2.0, 1e-6, 1e-6]),
                kind=np.array([O.BLACK_HOLE, 0, 0], np.uint8), alive=np.ones(3, np.uint8))


def test_split_substeps_follow_closest_encounter():  # accrete_test.go:122-143
    far, far_near = O.split_kdk(_three_body(5.0), 0.004, 0.01, 0.5, 8, 1, workers=1)
    close, close_near = O.split_kdk(_three_body(0.05), 0.004, 0.01, 0.5, 8, 1, workers=1)
    assert far == 1 and not far_near.any()
    assert close == 16 and list(close_near) == [False, True, False]


def _energy(s, eps):
    ke = 0.5 * np.sum(s["mass"] * (s["vx"] ** 2 + s["vy"] ** 2 + s["vz"] ** 2))
    return ke + O.potential_exact(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=eps)


def test_split_energy_drift_comparable_to_direct():
    """bh_test.go:165-184 with c = 0: 500 steps of the disk with two holes; the Barnes-Hut drift
    stays within 2x the drift of the (tiny-theta, i.e. direct) run + 1e-4. With c = 0 the holes
    pass through each other instead of merging, and that passage sets the drift of both runs."""
    drift = []
    for theta, leaf in ((1e-9, 24), (0.0, 0)):
        s = ics.test_disk(2000)
        e0 = _energy(s, 0.06)
        O.split_kdk(s, 0.004, 0.06, theta, leaf, 500)
        drift.append(abs((_energy(s, 0.06) - e0) / e0))
    ref, got = drift
    assert ref < 2e-2 and got <= 2 * ref + 1e-4, drift


def test_split_conserves_momentum_with_exact_pairs():
    """Both partners of every pair are kicked at the same times with the same force
    (split.go:8-15): with tiny theta the total momentum is conserved to rounding."""
    s = ics.test_disk(1500)
    p0 = np.array([np.sum(s["mass"] * s[k]) for k in ("vx", "vy", "vz")])
    scale = np.sum(s["mass"] * np.sqrt(s["vx"] ** 2 + s["vy"] ** 2 + s["vz"] ** 2))
    O.split_kdk(s, 0.004, 0.06, 1e-9, 8, 40)
    p1 = np.array([np.sum(s["mass"] * s[k]) for k in ("vx", "vy", "vz")])
    assert np.abs(p1 - p0).max() < 1e-12 * scale


def test_split_without_holes_is_the_plain_step():
    s = ics.plummer(3000, seed=9)
    a = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")}
    b = {k: s[k].copy() for k in a}
    O.kdk(a, dt=1e-3, eps=0.01, theta=0.5, leaf=8, nsteps=4, workers=1)
    sub, near = O.split_kdk(b, 1e-3, 0.01, 0.5, 8, 4, workers=1)
    assert sub == 1 and not near.any()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


# ---- the pair model (pair.go), behind the split step for c > 0 ----

def test_pair_force_is_gradient_of_potential():  # pair_test.go:8-18
    m, eps2, h = 0.7, 0.01 * 0.01, 1e-7
    for rs in (0.0, 0.05):
        for r in (0.06, 0.074, 0.08, 0.15, 0.4, 2.0):  # below and above 1.5 rs
            du = (O.pair_potential(1, m, (r + h) ** 2, eps2, rs) - O.pair_potential(1, m, (r - h) ** 2, eps2, rs)) / (2 * h)
            f = O.pair_force(m, r * r, eps2, rs) * r
            assert abs(f - du) <= 1e-6 * abs(f), (rs, r, f, du)


def test_pair_potential_limits():  # pair_test.go:20-31
    assert O.pair_potential(2, 3, 4, 0, 0) == -3.0
    assert abs(O.pair_potential(1, 1, 1, 0, 0.1) - (-1 / 0.9)) <= 1e-15
    S, H, D = O.STAR, O.BLACK_HOLE, O.DARK_MATTER
    assert O.pair_rs(S, 1, S, 1, 10) == 0 and O.pair_rs(H, 1, H, 1, 10) == 0 and O.pair_rs(S, 1, H, 5, 10) == 0.1


def test_dark_matter_pairs_are_newtonian_except_with_holes():  # pair_test.go:32-39
    S, H, D = O.STAR, O.BLACK_HOLE, O.DARK_MATTER
    assert O.pair_rs(D, 1, S, 1, 10) == 0 and O.pair_rs(S, 1, D, 1, 10) == 0 and O.pair_rs(D, 1, D, 1, 10) == 0
    assert O.pair_rs(D, 1, H, 5, 10) == 0.1


def test_relativistic_drift_slows_fast_bodies():
    """sim.go:315-343: with c > 0 a body moves by dt u / gamma; a body at u = c sqrt(3) drifts half
    as far as with c = 0 (gamma = 2), and slow bodies agree with the Newtonian drift."""
    z = np.zeros(2)
    s = dict(px=np.array([0.0, 1e6]), py=z.copy(), pz=z.copy(), vx=np.array([10 * np.sqrt(3), 1e-3]), vy=z.copy(),
             vz=z.copy(), ax=z.copy(), ay=z.copy(), az=z.copy(), mass=np.array([1e-12, 1e-12]))
    O.kdk(s, dt=1e-2, eps=0.1, theta=0.5, leaf=8, nsteps=1, c=10.0, workers=1)
    assert abs(s["px"][0] - 1e-2 * 10 * np.sqrt(3) / 2) <= 1e-12
    assert abs(s["px"][1] - (1e6 + 1e-5)) <= 1e-9


def test_group_walk_counts():
    """The group-walk counts behind the executed-work figure: a group of one star is the
    per-star walk, and an aligned group of 64 is the union of two of 32 (of 32 single stars), so
    it opens every node they open: openings, leaf pairs and the FLOP count can only grow."""
    s = ics.galaxy(20000, seed=9)
    t = O.Tree(s["px"], s["py"], s["pz"], s["mass"], s["kind"], theta=0.5, leaf=16)
    per_star = t.counts(0.01)
    assert t.group_counts(1) == per_star
    assert t.group_counts(1, workers=1) == t.group_counts(1, workers=4)
    prev = per_star
    for g in (32, 64):
        got = t.group_counts(g)
        assert got[1] >= prev[1] and got[2] >= prev[2]  # more leaf pairs and openings
        flops = [50 * c[0] + 18 * c[1] + 8 * c[2] for c in (prev, got)]
        assert flops[1] >= flops[0]
        prev = got
    empty = O.Tree(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), theta=0.5, leaf=16)
    assert empty.group_counts(64) == (0, 0, 0)
