"""GPU tests of the adjoint pair gbh_fwd_save / gbh_bwd: the FP64 path bit for bit against the
oracle's FP64 direct-sum adjoint, the FP32 path against the oracle and against central finite
differences (h = 1e-4, FP64 state) of the library's own forward on 256 random coordinates."""
import numpy as np
import pytest

from gravitas_gb300 import abi, ics, sim
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = abi.Context(0)
    yield c
    c.close()


def xv(s):
    return np.stack([s["px"], s["py"], s["pz"]], 1), np.stack([s["vx"], s["vy"], s["vz"]], 1)


def test_fp64_forward_and_gradient_bit_identical_to_oracle(ctx):
    s, targets = ics.adjoint_problem(1000, seed=11)  # 1000: not a multiple of the 128-body tile
    dt, eps, nsteps, every = 1e-3, 0.01, 30, 7
    x0, v0 = xv(s)
    xT, vT = ctx.fwd_save(x0, v0, s["mass"], dt, eps, nsteps, every, abi.ADJ_FP64)
    ref = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
    O.kdk_direct(ref, dt, eps, nsteps)
    rx, rv = xv(ref)
    assert np.array_equal(xT, rx) and np.array_equal(vT, rv)
    gx = 2 * (xT - targets) / len(xT)
    gv = np.random.default_rng(3).normal(size=gx.shape) * 1e-3
    got = ctx.bwd(gx, gv)
    want = O.adjoint_direct(s, dt, eps, nsteps, every, gx, gv)
    for g, w, name in zip(got, want, ("dx", "dv", "dm")):
        assert np.array_equal(g, w), name


def test_checkpoint_interval_and_repeat_do_not_change_bits(ctx):
    s, targets = ics.adjoint_problem(3000, seed=12)
    x0, v0 = xv(s)
    gx = np.random.default_rng(4).normal(size=(3000, 3))
    for prec in (abi.ADJ_FP32, abi.ADJ_FP64):
        ref = None
        for every in (1, 6, 25, 1000):
            ctx.fwd_save(x0, v0, s["mass"], 2e-3, 0.01, 25, every, prec)
            got = ctx.bwd(gx, None)
            again = ctx.bwd(gx, None)  # the tape survives a backward
            for a, b in zip(got, again):
                assert np.array_equal(a, b)
            if ref is None:
                ref = got
            for a, b in zip(ref, got):
                assert np.array_equal(a, b), (prec, every)


def test_fp32_gradient_close_to_fp64_oracle(ctx):
    s, targets = ics.adjoint_problem(2048, seed=13)
    dt, eps, nsteps, every = 1e-3, 0.01, 50, 10
    loss, dx, dv, dm = sim.trajectory_loss_gradient(s, targets, dt, eps, nsteps, every, abi.ADJ_FP32, ctx)
    ref = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
    O.kdk_direct(ref, dt, eps, nsteps)
    rx, _ = xv(ref)
    gx = 2 * (rx - targets) / len(rx)
    wx, wv, wm = O.adjoint_direct(s, dt, eps, nsteps, every, gx, np.zeros_like(gx))
    for g, w in ((dx, wx), (dv, wv), (dm, wm)):
        assert np.linalg.norm(g - w) <= 1e-5 * np.linalg.norm(w)
    assert abs(loss - np.sum((rx - targets) ** 2) / len(rx)) <= 1e-9 * loss


def test_fp32_gradient_matches_central_differences_on_256_coordinates(ctx):
    """Central differences h = 1e-4 of the library's own FP32-force forward (FP64 state and
    loss) on 128 velocity and 128 mass coordinates. Tolerance: 1e-3 relative per coordinate,
    the error of the difference quotient itself bounding the denominator from below."""
    n, dt, eps, nsteps, every = 2048, 1e-3, 0.01, 200, 50
    s, targets = ics.adjoint_problem(n, seed=14)
    loss, dx, dv, dm = sim.trajectory_loss_gradient(s, targets, dt, eps, nsteps, every, abi.ADJ_FP32, ctx)
    rng = np.random.default_rng(5)
    coords = [("v", int(i), int(c)) for i, c in zip(rng.choice(n, 128, replace=False), rng.integers(0, 3, 128))]
    coords += [("m", int(i), 0) for i in rng.choice(n, 128, replace=False)]
    x0, v0 = xv(s)
    h = 1e-4

    def loss_of(x, v, m):
        xT, _ = ctx.fwd_save(x, v, m, dt, eps, nsteps, nsteps, abi.ADJ_FP32)
        return np.sum((xT - targets) ** 2) / n

    errs, scale = [], np.abs(np.concatenate([dv.ravel(), dm])).max()
    for kind, i, c in coords:
        vals = []
        for sign in (1.0, -1.0):
            v, m = v0.copy(), s["mass"].copy()
            if kind == "v":
                v[i, c] += sign * h
            else:
                m[i] += sign * h
            vals.append(loss_of(x0, v, m))
        fd = (vals[0] - vals[1]) / (2 * h)
        g = dv[i, c] if kind == "v" else dm[i]
        errs.append(abs(g - fd) / max(abs(fd), 1e-3 * scale))
    errs = np.array(errs)
    assert errs.max() <= 1e-3, (np.median(errs), errs.max())


def test_errors(ctx):
    c = abi.Context(0)
    try:
        with pytest.raises(abi.GbhError) as e:
            c.bwd(np.zeros((4, 3)), None)
        assert e.value.code == abi.ERR_STATE
    finally:
        c.close()
    s, _ = ics.adjoint_problem(16, seed=1)
    x0, v0 = xv(s)
    for args in ((1e-3, 0.0, 10, 5), (1e-3, 0.01, 0, 5), (1e-3, 0.01, 10, 0)):
        with pytest.raises(abi.GbhError) as e:
            ctx.fwd_save(x0, v0, s["mass"], *args)
        assert e.value.code == abi.ERR_ARG
    with pytest.raises(abi.GbhError):
        ctx.fwd_save(x0, v0, s["mass"], 1e-3, 0.01, 10, 5, precision=7)
    with pytest.raises(abi.GbhError) as e:  # a failed forward leaves no tape
        ctx.bwd(np.zeros((16, 3)), None)
    assert e.value.code == abi.ERR_STATE


def test_gradient_matches_central_differences_of_the_tree_dynamics(ctx):
    """The tree force at theta 0.5 changes discontinuously where a group's opening test flips; with
    h = 1e-4 those jumps are mostly far below the difference quotient: central differences of the
    library's own tree forward (mixed walk, theta 0.5, 200 KDK steps through gbh_step_kdk) agree
    with the direct-sum adjoint gradient at the median to 1e-4 relative and on nine in ten of 32
    velocity coordinates to 1e-3; a quotient that straddles a jump stays within 5e-3 (the full
    32,768-body, 1,000-step run's worst coordinate was 2.4e-3)."""
    n, dt, eps, nsteps = 2048, 1e-3, 0.01, 200
    s, targets = ics.adjoint_problem(n, seed=15)
    _, _, dv, _ = sim.trajectory_loss_gradient(s, targets, dt, eps, nsteps, 50, abi.ADJ_FP32, ctx)
    par = abi.make_params(0.5, eps, 8, False, False, "mixed")
    F = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")

    def tree_loss(v):
        st = {k: (s[k].copy() if k in s else np.zeros(n)) for k in F}
        st["vx"], st["vy"], st["vz"] = v[:, 0].copy(), v[:, 1].copy(), v[:, 2].copy()
        ctx.call("gbh_step_kdk", par, dt, nsteps, 0, n, *[abi.ptr(st[k]) for k in F], abi.ptr(s["mass"]), None, None)
        x = np.stack([st["px"], st["py"], st["pz"]], 1)
        return np.sum((x - targets) ** 2) / n

    _, v0 = xv(s)
    rng = np.random.default_rng(6)
    h, errs, scale = 1e-4, [], np.abs(dv).max()
    for i, c in zip(rng.choice(n, 32, replace=False), rng.integers(0, 3, 32)):
        vp, vm = v0.copy(), v0.copy()
        vp[i, c] += h
        vm[i, c] -= h
        fd = (tree_loss(vp) - tree_loss(vm)) / (2 * h)
        errs.append(abs(dv[i, c] - fd) / max(abs(fd), 1e-3 * scale))
    errs = np.array(errs)
    assert np.median(errs) <= 1e-4 and np.mean(errs <= 1e-3) >= 0.9 and errs.max() <= 5e-3, np.sort(errs)
