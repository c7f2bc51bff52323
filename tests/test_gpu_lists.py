"""GPU tests of the list walk (GBH_WALK_MIXED with 32-star groups, or 64-star groups of two stars a
lane, walk_lists.cu): a warp builds its group's interaction lists with node-parallel opening tests
and evaluates them from shared memory two entries at a time. The context is made with
GBH_CFG_NO_SPLIT, so that one warp walks each group (the split mode is tested at the end). Its opening
test takes the reference criterion (bh.go:116) over every star of the group, with a margin for
FP32 rounding, so every star sees each accepted node where the reference accepts it or deeper:
against the FP64 direct sum it is at least as accurate as the reference's per-star walk, and
against the reference walk it differs by part of the tree's own error. Results do not depend on
the launch order, the list depth beyond FP32 summation rounding, or a target list that holds
every star."""
import numpy as np
import pytest

from gravitas_gb300 import abi, ics
from oracle import oracle as O

pytestmark = pytest.mark.gpu
P = abi.ptr
F9 = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")


@pytest.fixture(scope="module")
def ctx():
    c = abi.Context(0, abi.CFG_NO_SPLIT)
    yield c
    c.close()


def forces(ctx, s, par):
    n = len(s["px"])
    a = [np.zeros(n) for _ in range(3)]
    ctx.call("gbh_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s.get("kind")),
             P(s.get("alive")), P(a[0]), P(a[1]), P(a[2]))
    return np.stack(a, 1)


def lists(theta, eps, leaf, depth=0, mono=False, dm_off=False, group=32):
    return abi.make_params(theta, eps, leaf, mono, dm_off, "mixed", group_size=group, list_depth=depth)


def rel(got, want):
    return np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)


def rms(e):
    return float(np.sqrt(np.mean(e ** 2)))


@pytest.mark.parametrize("group", [32, 64])
@pytest.mark.parametrize("scene,theta,leaf,eps", [("plummer", 0.5, 8, 0.01), ("plummer", 0.7, 32, 0.01),
                                                  ("galaxy", 0.5, 16, 0.02), ("disk", 0.9, 24, 0.06)])
def test_list_walk_is_at_least_as_accurate_as_the_reference_walk(ctx, scene, theta, leaf, eps, group):
    """Against the FP64 direct sum: RMS and p99 error at most the reference per-star walk's
    (x1.001); against the reference walk: median below the reference's own median error and every
    star within 5x the reference's worst error."""
    s = {"plummer": lambda: ics.plummer(16384, seed=0), "galaxy": lambda: ics.galaxy(20000, seed=2),
         "disk": lambda: ics.test_disk(6000, seed=1)}[scene]()
    kind = s.get("kind")
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], kind, eps=eps)
    ref = O.Tree(s["px"], s["py"], s["pz"], s["mass"], kind, s.get("alive"), theta=theta, leaf=leaf).accelerations(eps)
    got = forces(ctx, s, lists(theta, eps, leaf, group=group))
    live = np.linalg.norm(want, axis=1) > 0  # holes get 0 from both
    e, e_ref = rel(got[live], want[live]), rel(ref[live], want[live])
    assert rms(e) <= 1.001 * rms(e_ref) + 1e-7 and np.percentile(e, 99) <= 1.001 * np.percentile(e_ref, 99) + 1e-7
    d = rel(got[live], ref[live])
    assert np.median(d) <= np.median(e_ref) and d.max() <= 5 * e_ref.max()
    assert np.array_equal(got[~live], ref[~live])


@pytest.mark.parametrize("group", [32, 64])
def test_list_walk_monopole_and_no_softening(ctx, group):
    rng = np.random.default_rng(21)
    p = rng.normal(size=(3000, 3))
    s = dict(px=p[:, 0].copy(), py=p[:, 1].copy(), pz=p[:, 2].copy(), mass=rng.uniform(0.5, 1.5, 3000))
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], eps=0.0)
    for mono in (False, True):
        ref = O.Tree(s["px"], s["py"], s["pz"], s["mass"], theta=0.5, leaf=8).accelerations(0.0, monopole_only=mono)
        got = forces(ctx, s, lists(0.5, 0.0, 8, mono=mono, group=group))
        assert np.isfinite(got).all()
        assert rms(rel(got, want)) <= 1.01 * rms(rel(ref, want)) + 1e-6


@pytest.mark.parametrize("group", [32, 64])
def test_list_walk_far_apart_clumps_use_exact_separations(ctx, group):
    """Two tight clumps 1e6 apart: groups that straddle the jump between them form separations
    from hi and lo parts apart; the forces stay at FP32 accuracy against the FP64 walk."""
    rng = np.random.default_rng(9)
    p = np.concatenate([rng.normal(size=(3000, 3)) * 1e-3, rng.normal(size=(3000, 3)) * 1e-3 + 1e6])
    s = dict(px=p[:, 0].copy(), py=p[:, 1].copy(), pz=p[:, 2].copy(), mass=np.ones(6000))
    a = forces(ctx, s, abi.make_params(0.5, 1e-4, 8, False, False, "fp64"))
    for eps in (1e-4, 0.0):
        am = forces(ctx, s, lists(0.5, eps, 8, group=group))
        b = a if eps else forces(ctx, s, abi.make_params(0.5, 0.0, 8, False, False, "fp64"))
        e = np.linalg.norm(am - b, axis=1) / np.linalg.norm(b, axis=1).mean()
        assert np.median(e) < 1e-5 and e.max() < 1e-3, (eps, np.median(e), e.max())


@pytest.mark.parametrize("group", [32, 64])
def test_list_walk_coincident_stars_and_tiny_systems(ctx, group):
    n = 101
    s = dict(px=np.full(n, 1.0), py=np.full(n, 2.0), pz=np.full(n, 3.0), mass=np.ones(n))
    s["px"][-1] = s["py"][-1] = s["pz"][-1] = 0.0
    a = forces(ctx, s, lists(0.0, 0.01, 0, group=group))
    want = forces(ctx, s, abi.make_params(0.0, 0.01, 0, False, False, "fp64"))
    assert np.isfinite(a).all() and np.allclose(a, want, rtol=1e-5, atol=1e-6)
    # One or two stars: nothing to approximate, so the FP64 walk's forces to FP32 rounding. More
    # stars: one or two groups cover the whole system (partly filled groups included), so the list
    # walk opens nodes that the per-star walk accepts for some stars; against the FP64 direct sum
    # it is at least as accurate.
    for m in (1, 2, 31, 33, 63, 64, 65, 97):
        t = ics.plummer(max(m, 2), seed=m)
        t = {k: v[:m] for k, v in t.items()}
        got = forces(ctx, t, lists(0.5, 0.01, 4, group=group))
        ref = forces(ctx, t, abi.make_params(0.5, 0.01, 4, False, False, "fp64"))
        assert np.isfinite(got).all(), m
        if m <= 2:
            assert np.allclose(got, ref, rtol=1e-5, atol=1e-7), m
        else:
            want = O.direct(t["px"], t["py"], t["pz"], t["mass"], eps=0.01)
            assert rms(rel(got, want)) <= 1.001 * rms(rel(ref, want)) + 1e-6, m


@pytest.mark.parametrize("group", [32, 64])
def test_list_walk_kinds_dead_holes_and_dark_matter_off(ctx, group):
    s = ics.test_disk(20000, seed=3)
    s["kind"][5::50] = abi.DARK_MATTER
    s["alive"][7::97] = 0
    rngacc = [np.full(len(s["px"]), 7.0) for _ in range(3)]
    n = len(s["px"])
    for dm_off in (False, True):
        a = [x.copy() for x in rngacc]
        ctx.call("gbh_accelerations", lists(0.5, 0.02, 16, dm_off=dm_off, group=group), n, P(s["px"]), P(s["py"]),
                 P(s["pz"]), P(s["mass"]), P(s["kind"]), P(s["alive"]), P(a[0]), P(a[1]), P(a[2]))
        got = np.stack(a, 1)
        dead = s["alive"] == 0
        holes = (s["kind"] == abi.BLACK_HOLE) & ~dead
        assert np.all(got[dead] == 7.0) and np.all(got[holes] == 0.0)
        live = ~dead & ~holes
        want = O.direct(s["px"], s["py"], s["pz"], s["mass"] * s["alive"], s["kind"], eps=0.02, dm_off=dm_off,
                        targets=np.flatnonzero(live)[::5])  # dead bodies pull nothing
        ref = O.Tree(s["px"], s["py"], s["pz"], s["mass"], s["kind"], s["alive"], theta=0.5, leaf=16,
                     dm_off=dm_off).accelerations(0.02)
        t = np.flatnonzero(live)[::5]
        assert rms(rel(got[t], want)) <= 1.001 * rms(rel(ref[t], want)) + 1e-7


@pytest.mark.parametrize("group", [32, 64])
def test_list_walk_is_deterministic_and_order_free(ctx, group):
    """The same bits run after run, with or without the longest-first group order."""
    s = ics.merger(200_000, seed=4)
    par = lists(0.5, 0.02, 32, group=group)
    a = forces(ctx, s, par)
    b = forces(ctx, s, par)  # the second walk takes the order the first one's costs give
    assert np.array_equal(a, b)
    other = abi.Context(0, abi.CFG_NO_LPT | abi.CFG_NO_SPLIT)
    try:
        assert np.array_equal(forces(other, s, par), a)
    finally:
        other.close()


@pytest.mark.parametrize("group", [32, 64])
def test_list_depth_changes_only_the_summation(ctx, group):
    """The list depth sets how many entries a list holds before it is evaluated: the same
    interactions, summed in other blocks (global relative norm <= 1e-6)."""
    s = ics.galaxy(60000, seed=5)
    base = forces(ctx, s, lists(0.5, 0.02, 16, depth=48, group=group))
    for depth in (2, 3, 24, 56):
        got = forces(ctx, s, lists(0.5, 0.02, 16, depth=depth, group=group))
        assert np.linalg.norm(got - base) <= 1e-6 * np.linalg.norm(base), depth
    with pytest.raises(abi.GbhError) as ei:
        forces(ctx, s, lists(0.5, 0.02, 16, depth=57, group=group))
    assert ei.value.code == abi.ERR_ARG


@pytest.mark.parametrize("group", [32, 64])
def test_block_steps_one_level_is_the_global_step_with_the_list_walk(ctx, group):
    """A target list that holds every star walks exactly as no list."""
    s = ics.merger(100_000, seed=6)
    n = len(s["px"])
    par = lists(0.5, 0.02, 16, group=group)
    up = lambda: ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None,
                          None, None, P(s["mass"]), P(s["kind"]), P(s["alive"]))

    def down():
        st = {k: np.zeros(n) for k in F9}
        ctx.call("gbh_state_download", *[P(st[k]) for k in F9])
        return st

    up()
    ctx.call("gbh_state_step", par, 4e-3, 2)
    want = down()
    up()
    st = ctx.step_block(par, 4e-3, 0.025, 1, 2)
    got = down()
    assert st["substeps"] == 2 and st["evaluations"] == 2 * n
    for k in F9:
        assert np.array_equal(want[k], got[k]), k
    # several levels: fewer walked stars at the energy drift of global steps
    up()
    e0 = ctx.diagnostics(par)["total"]
    st = ctx.step_block(par, 8e-3, 0.025, 4, 2)
    e1 = ctx.diagnostics(par)["total"]
    assert st["evaluations"] < 2 * 8 * n and abs((e1 - e0) / e0) < 1e-4


@pytest.mark.parametrize("group", [32, 64])
@pytest.mark.parametrize("scene,theta,leaf,eps", [("plummer", 0.5, 8, 0.01), ("galaxy", 0.6, 24, 0.02)])
def test_split_list_walk_sums_the_same_interactions(scene, theta, leaf, eps, group):
    """Few groups for the GPU: each group's walk is shared among several warps, each
    owning a range of source stars (a node counts where its first star is, a leaf's stars where
    they are). The parts add up to the same interactions as one warp's walk: the forces differ
    only by the order of the FP32 sums (global relative norm <= 1e-6), and the split walk meets
    the same accuracy bound against the FP64 direct sum."""
    s = {"plummer": lambda: ics.plummer(16384, seed=11), "galaxy": lambda: ics.galaxy(20000, seed=12)}[scene]()
    par = lists(theta, eps, leaf, group=group)
    split, whole = abi.Context(0), abi.Context(0, abi.CFG_NO_SPLIT)
    try:
        a = forces(split, s, par)
        b = forces(whole, s, par)
        assert np.array_equal(a, forces(split, s, par))  # deterministic
    finally:
        split.close()
        whole.close()
    assert not np.array_equal(a, b)  # the parts' sums are grouped differently: the split walk ran
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
    kind = s.get("kind")
    want = O.direct(s["px"], s["py"], s["pz"], s["mass"], kind, eps=eps)
    ref = O.Tree(s["px"], s["py"], s["pz"], s["mass"], kind, s.get("alive"), theta=theta, leaf=leaf).accelerations(eps)
    live = np.linalg.norm(want, axis=1) > 0
    e, e_ref = rel(a[live], want[live]), rel(ref[live], want[live])
    assert rms(e) <= 1.001 * rms(e_ref) + 1e-7
