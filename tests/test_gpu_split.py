"""GPU tests of the hole-aware split step (split.go, c = 0): the reference's substep
known-answer test, FP64-walk trajectories bit for bit against the oracle's restatement, and the
energy behaviour of the FP32 walks."""
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


def step_host(ctx, s, par, dt, nsteps, acc_valid=0):
    n = len(s["px"])
    st = {k: s[k].copy() for k in F9}
    ctx.call("gbh_step_kdk", par, dt, nsteps, acc_valid, n, *[P(st[k]) for k in F9], P(s["mass"]), P(s["kind"]),
             P(s["alive"]))
    return st, ctx.timings()["substeps"]


def three_body(r):
    z = np.zeros(3)
    return dict(px=np.array([0.0, r, 50.0]), py=z.copy(), pz=z.copy(), vx=z.copy(), vy=z.copy(), vz=z.copy(),
                ax=z.copy(), ay=z.copy(), az=z.copy(), mass=np.array([2.0, 1e-6, 1e-6]),
                kind=np.array([O.BLACK_HOLE, 0, 0], np.uint8), alive=np.ones(3, np.uint8))


@pytest.mark.parametrize("r,want", [(5.0, 1), (0.05, 16)])
def test_substeps_follow_closest_encounter(ctx, r, want):  # accrete_test.go:122-143
    s = three_body(r)
    par = abi.make_params(0.5, 0.01, 8, False, False, "fp64")
    got, sub = step_host(ctx, s, par, 0.004, 1)
    assert sub == want
    ref = {k: s[k].copy() for k in (*F9, "mass", "kind", "alive")}
    rsub, _ = O.split_kdk(ref, 0.004, 0.01, 0.5, 8, 1)
    assert rsub == want
    for k in F9:
        assert np.array_equal(got[k], ref[k]), k


def disk_with_extras(n, seed=1):
    """The reference test galaxy (two holes) plus dark matter and dead bodies."""
    s = ics.test_disk(n, seed=seed)
    s["kind"][5:40:3] = O.DARK_MATTER
    s["alive"][7:60:11] = 0
    return s


@pytest.mark.parametrize("dm_off", [False, True])
def test_fp64_split_steps_bit_exact_with_oracle(ctx, dm_off):
    s = disk_with_extras(4000)
    par = abi.make_params(0.5, 0.06, 8, False, dm_off, "fp64")
    got, sub = step_host(ctx, s, par, 0.004, 12)
    ref = {k: s[k].copy() for k in (*F9, "mass", "kind", "alive")}
    rsub, _ = O.split_kdk(ref, 0.004, 0.06, 0.5, 8, 12, dm_off=dm_off)
    assert sub == rsub and sub > 1
    for k in F9:
        assert np.array_equal(got[k], ref[k]), k


def test_resident_split_steps_equal_host_steps(ctx):
    s = disk_with_extras(3000, seed=2)
    n = len(s["px"])
    par = abi.make_params(0.5, 0.06, 8, False, False, "mixed")
    want, _ = step_host(ctx, s, par, 0.004, 6)
    ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
             P(s["mass"]), P(s["kind"]), P(s["alive"]))
    for _ in range(3):
        ctx.call("gbh_state_step", par, 0.004, 2)
    got = {k: np.zeros(n) for k in F9}
    ctx.call("gbh_state_download", *[P(got[k]) for k in F9])
    for k in F9:
        assert np.array_equal(got[k], want[k]), k


def _energy(s, eps):
    ke = 0.5 * np.sum(s["mass"] * (s["vx"] ** 2 + s["vy"] ** 2 + s["vz"] ** 2))
    return ke + O.potential_exact(s["px"], s["py"], s["pz"], s["mass"], s["kind"], eps=eps)


def test_mixed_walk_split_energy_tracks_fp64(ctx):
    """250 steps of the two-hole disk (before the holes' close passage): the mixed walk's energy
    error stays within 2x the FP64 walk's + 1e-5."""
    s = ics.test_disk(2000)
    e0 = _energy(s, 0.06)
    drift = {}
    for walk in ("fp64", "mixed"):
        st, _ = step_host(ctx, s, abi.make_params(0.5, 0.06, 8, False, False, walk), 0.004, 250)
        st["mass"], st["kind"] = s["mass"], s["kind"]
        drift[walk] = abs((_energy(st, 0.06) - e0) / e0)
    assert drift["mixed"] <= 2 * drift["fp64"] + 1e-5, drift


def test_forest_with_holes_is_rejected(ctx):
    a, b = ics.test_disk(300), ics.plummer(200, seed=3)
    s = {k: np.concatenate([a[k], b[k]]) for k in a}
    off = np.array([0, len(a["px"]), len(s["px"])], np.int64)
    ctx.forest_upload(off, s["px"], s["py"], s["pz"], s["vx"], s["vy"], s["vz"], s["mass"], s["kind"], s["alive"])
    with pytest.raises(abi.GbhError) as ei:
        ctx.call("gbh_state_step", abi.make_params(0.5, 0.06, 8), 0.004, 1)
    assert ei.value.code == abi.ERR_UNSUPPORTED


@pytest.mark.parametrize("c", [10.0, 3.0])
def test_fp64_split_steps_with_speed_of_light_bit_exact(ctx, c):
    """c > 0: Paczynski-Wiita star-hole pairs (pair.go:26-35) in the direct hole sums and the
    timescales, and every drift by u / gamma (split.go:226-250)."""
    s = disk_with_extras(3000, seed=3)
    par = abi.make_params(0.5, 0.06, 8, False, False, "fp64", c=c)
    got, sub = step_host(ctx, s, par, 0.004, 10)
    ref = {k: s[k].copy() for k in (*F9, "mass", "kind", "alive")}
    rsub, _ = O.split_kdk(ref, 0.004, 0.06, 0.5, 8, 10, c=c)
    assert sub == rsub
    for k in F9:
        assert np.array_equal(got[k], ref[k]), k
    newton, _ = step_host(ctx, s, abi.make_params(0.5, 0.06, 8, False, False, "fp64"), 0.004, 10)
    assert not np.array_equal(newton["px"], got["px"])  # the speed of light changed the run


def test_fp64_kdk_and_block_steps_with_speed_of_light_bit_exact(ctx):
    """Without holes: the global KDK's drift u / sqrt(1 + u^2 / c^2) (sim.go:335-343) and the block
    steps' driftOne (sim.go:345-350), against the oracle."""
    s = ics.plummer(5000, seed=8)
    for k in ("vx", "vy", "vz"):
        s[k] = s[k] * 4.0  # fast enough that gamma matters at c = 3
    n = len(s["px"])
    par = abi.make_params(0.5, 0.01, 8, False, False, "fp64", c=3.0)
    got, _ = step_host(ctx, s, par, 1e-3, 5)
    ref = {k: s[k].copy() for k in (*F9, "mass")}
    O.kdk(ref, dt=1e-3, eps=0.01, theta=0.5, leaf=8, nsteps=5, c=3.0)
    for k in F9:
        assert np.array_equal(got[k], ref[k]), k
    ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
             P(s["mass"]), None, None)
    st = ctx.step_block(par, 1e-2, 0.025, 6, 2)
    blk = {k: np.zeros(n) for k in F9}
    ctx.call("gbh_state_download", *[P(blk[k]) for k in F9])
    ref = {k: s[k].copy() for k in (*F9, "mass")}
    events, walked = O.block_kdk(ref, dt=1e-2, eta=0.025, levels=6, eps=0.01, theta=0.5, leaf=8, nsteps=2, c=3.0)
    assert (st["substeps"], st["evaluations"]) == (events, walked)
    for k in F9:
        assert np.array_equal(blk[k], ref[k]), k
