"""GPU tests of the failure paths driven from the host (no GPU fault is provoked): with the
allocation test hook armed (GBH_FAULT_ALLOC=k when a context is created, the allocation after k
successful ones fails once, without calling cudaMalloc), every call either succeeds or returns
GBH_ERR_NOMEM with a message, and the next call on the same context gives exactly the results
of a context that never failed; the hook is disarmed by a context created without it."""
import os

import numpy as np
import pytest

from gravitas_gb300 import abi, ics

pytestmark = pytest.mark.gpu
P = abi.ptr
F9 = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")


def arm(k):
    if k is None:
        os.environ.pop("GBH_FAULT_ALLOC", None)
    else:
        os.environ["GBH_FAULT_ALLOC"] = str(k)


def forces(ctx, s, par):
    n = len(s["px"])
    a = [np.zeros(n) for _ in range(3)]
    ctx.call("gbh_accelerations", par, n, P(s["px"]), P(s["py"]), P(s["pz"]), P(s["mass"]), P(s.get("kind")),
             P(s.get("alive")), P(a[0]), P(a[1]), P(a[2]))
    return np.stack(a, 1)


def steps(ctx, s, par, k=3):
    n = len(s["px"])
    st = {f: (s[f].copy() if f in s else np.zeros(n)) for f in F9}
    ctx.call("gbh_step_kdk", par, 1e-3, k, 0, n, *[P(st[f]) for f in F9], P(s["mass"]), P(s.get("kind")),
             P(s.get("alive")))
    return st


def run_with_faults(call, ks, want, same):
    fired = 0
    try:
        for k in ks:
            arm(k)
            try:
                c = abi.Context(0)
            except abi.GbhError as e:  # the context's own allocations may take the fault
                assert e.code == abi.ERR_NOMEM
                fired += 1
                continue
            arm(None)
            try:
                try:
                    call(c)
                except abi.GbhError as e:
                    msg = str(e).lower()
                    assert e.code == abi.ERR_NOMEM and ("alloc" in msg or "memory" in msg), e
                    fired += 1
                same(call(c), want)  # the context recovers: results of a context that never failed
            finally:
                c.close()
    finally:
        arm(None)
        abi.Context(0).close()  # disarmed for everyone after this test
    return fired


def test_allocation_failures_in_force_and_step_calls():
    s = ics.galaxy(30000, seed=4)
    par = abi.make_params(0.5, 0.02, 16, False, False, "mixed")
    with abi.Context(0) as c0:
        want_f = forces(c0, s, par)
        want_s = steps(c0, s, par)

    def same_f(got, want):
        assert np.array_equal(got, want)

    def same_s(got, want):
        for f in F9:
            assert np.array_equal(got[f], want[f]), f

    fired = run_with_faults(lambda c: forces(c, s, par), range(0, 60, 1), want_f, same_f)
    assert fired >= 40  # most allocation points of a force call were hit
    fired = run_with_faults(lambda c: steps(c, s, par), range(0, 60, 3), want_s, same_s)
    assert fired >= 10


def test_allocation_failures_in_hole_steps_and_the_adjoint():
    s = ics.test_disk(3000, seed=2)  # a disk with black holes: the split step
    par = abi.make_params(0.5, 0.06, 8, False, False, "mixed")
    with abi.Context(0) as c0:
        want = steps(c0, s, par)

    def same(got, w):
        for f in F9:
            assert np.array_equal(got[f], w[f]), f

    assert run_with_faults(lambda c: steps(c, s, par), range(0, 80, 4), want, same) >= 10
    a, _ = ics.adjoint_problem(512, seed=3)
    x0 = np.stack([a["px"], a["py"], a["pz"]], 1)
    v0 = np.stack([a["vx"], a["vy"], a["vz"]], 1)
    with abi.Context(0) as c0:
        want_a = c0.fwd_save(x0, v0, a["mass"], 1e-3, 0.01, 20, 5, abi.ADJ_FP32)

    def same_a(got, w):
        assert np.array_equal(got[0], w[0]) and np.array_equal(got[1], w[1])

    run_with_faults(lambda c: c.fwd_save(x0, v0, a["mass"], 1e-3, 0.01, 20, 5, abi.ADJ_FP32), range(0, 12),
                    want_a, same_a)
