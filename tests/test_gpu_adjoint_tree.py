"""GPU tests of the tree adjoint (gbh_adjoint_params.force = GBH_ADJ_TREE): the gradient of a
final-state loss through KDK steps of the Barnes-Hut force (the mixed list walk, quadrupoles,
32-star groups, split among warps at these sizes), with each step's interaction lists and tree
topology frozen.

* With a tiny opening angle every node is opened and the tree force is the softened direct sum:
  the tree adjoint then equals the direct-sum adjoint (checked against the oracle and against
  finite differences in test_gpu_adjoint.py) to FP32 rounding.
* At theta 0.5-0.7 its gradient agrees with central differences of the library's own tree
  forward; a difference quotient whose perturbation flips an opening test measures a jump instead
  of a derivative, so the bound holds for nine in ten coordinates, and the median is far below it.
  The direct-sum gradient, the other dynamics, is farther from those quotients by more than ten
  times on the coordinates whose gradient the forces carry.
"""
import numpy as np
import pytest

from gravitas_gb300 import abi, ics

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = abi.Context(0)
    yield c
    c.close()


def xv(s):
    return np.stack([s["px"], s["py"], s["pz"]], 1), np.stack([s["vx"], s["vy"], s["vz"]], 1)


def gradient(ctx, s, targets, dt, eps, nsteps, every, force, theta=0.0, leaf=0):
    x0, v0 = xv(s)
    xT, _ = ctx.fwd_save(x0, v0, s["mass"], dt, eps, nsteps, every, abi.ADJ_FP32, force, theta, leaf)
    r = xT - targets
    n = len(r)
    return float(np.sum(r * r) / n), ctx.bwd(2.0 * r / n, None)


def loss_at(ctx, s, targets, x0, v0, m, dt, eps, nsteps, theta, leaf):
    xT, _ = ctx.fwd_save(x0, v0, m, dt, eps, nsteps, nsteps, abi.ADJ_FP32, abi.ADJ_TREE, theta, leaf)
    return float(np.sum((xT - targets) ** 2) / len(xT))


def rel_norm(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_tiny_theta_tree_adjoint_is_the_direct_sum_adjoint(ctx):
    s, targets = ics.adjoint_problem(3000, seed=31)
    dt, eps, nsteps, every = 1e-3, 0.01, 20, 6
    lt, gt = gradient(ctx, s, targets, dt, eps, nsteps, every, abi.ADJ_TREE, theta=1e-4, leaf=8)
    ld, gd = gradient(ctx, s, targets, dt, eps, nsteps, every, abi.ADJ_DIRECT)
    assert abs(lt - ld) <= 1e-9 * abs(ld)
    for a, b, name in zip(gt, gd, ("dx", "dv", "dm")):
        assert rel_norm(a, b) <= 2e-5, (name, rel_norm(a, b))


@pytest.mark.parametrize("theta,leaf", [(0.5, 8), (0.7, 16)])
def test_tree_adjoint_agrees_with_differences_of_the_tree_dynamics(ctx, theta, leaf):
    s, targets = ics.adjoint_problem(2048, seed=32)
    dt, eps, nsteps, every = 1e-3, 0.01, 10, 4
    x0, v0 = xv(s)
    m = s["mass"]
    _, (gx, gv, gm) = gradient(ctx, s, targets, dt, eps, nsteps, every, abi.ADJ_TREE, theta, leaf)
    _, (dx, dv, dm) = gradient(ctx, s, targets, dt, eps, nsteps, every, abi.ADJ_DIRECT)
    rng = np.random.default_rng(7)
    err_tree, err_direct = [], []
    scale_x, scale_v, scale_m = np.abs(gx).max(), np.abs(gv).max(), np.abs(gm).max()
    for q in range(36):
        kind = q % 3
        i, c = int(rng.integers(len(m))), int(rng.integers(3))
        if kind == 0:
            h, g, gdir, scale = 1e-5, gx[i, c], dx[i, c], scale_x
        elif kind == 1:
            h, g, gdir, scale = 1e-4, gv[i, c], dv[i, c], scale_v
        else:
            h, g, gdir, scale = 1e-2 * m[i], gm[i], dm[i], scale_m
        vals = []
        for sign in (1.0, -1.0):
            x, v, mm = x0.copy(), v0.copy(), m.copy()
            if kind == 0:
                x[i, c] += sign * h
            elif kind == 1:
                v[i, c] += sign * h
            else:
                mm[i] += sign * h
            vals.append(loss_at(ctx, s, targets, x, v, mm, dt, eps, nsteps, theta, leaf))
        fd = (vals[0] - vals[1]) / (2 * h)
        floor = max(abs(fd), 1e-3 * scale)
        err_tree.append(abs(g - fd) / floor)
        err_direct.append(abs(gdir - fd) / floor)
    err_tree, err_direct = np.array(err_tree), np.array(err_direct)
    assert np.median(err_tree) <= 1e-4, np.median(err_tree)
    assert np.mean(err_tree <= 1e-3) >= 0.9, np.sort(err_tree)
    # the tree adjoint differentiates the dynamics the quotients measure; the direct sum does not,
    # which shows on the coordinates whose gradient the forces carry (the upper decile)
    p_tree, p_direct = np.percentile(err_tree, 90), np.percentile(err_direct, 90)
    assert p_direct >= 10 * p_tree, (p_direct, p_tree)


def test_tree_adjoint_tape_survives_and_validates(ctx):
    s, targets = ics.adjoint_problem(1000, seed=33)
    x0, v0 = xv(s)
    ctx.fwd_save(x0, v0, s["mass"], 1e-3, 0.01, 8, 3, abi.ADJ_FP32, abi.ADJ_TREE, 0.5, 8)
    gxT = np.random.default_rng(5).normal(size=(1000, 3))
    a = ctx.bwd(gxT, None)
    # another force call on the context in between rebuilds its tree; the backward rebuilds its own
    acc = [np.zeros(1000) for _ in range(3)]
    ctx.call("gbh_accelerations", abi.make_params(0.5, 0.01, 32), 1000, abi.ptr(s["px"]), abi.ptr(s["py"]),
             abi.ptr(s["pz"]), abi.ptr(s["mass"]), None, None, abi.ptr(acc[0]), abi.ptr(acc[1]), abi.ptr(acc[2]))
    b = ctx.bwd(gxT, None)
    for p, q in zip(a, b):
        assert rel_norm(p, q) <= 1e-12
    with pytest.raises(abi.GbhError) as ei:
        ctx.fwd_save(x0, v0, s["mass"], 1e-3, 0.01, 8, 3, abi.ADJ_FP64, abi.ADJ_TREE, 0.5, 8)
    assert ei.value.code == abi.ERR_ARG
    with pytest.raises(abi.GbhError) as ei:
        ctx.fwd_save(x0, v0, s["mass"], 1e-3, 0.01, 8, 3, abi.ADJ_FP32, 2, 0.5, 8)
    assert ei.value.code == abi.ERR_ARG
