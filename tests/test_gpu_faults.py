"""GPU tests of the failure paths driven from the host (no GPU fault is provoked). With the
allocation test hook armed (GBH_FAULT_ALLOC=k when a context is created, the allocation after k
successful ones fails once, without calling cudaMalloc), every call either succeeds or returns
GBH_ERR_NOMEM with a message, and the next call on the same context gives exactly the results
of a context that never failed; the hook is disarmed by a context created without it. Non-finite
positions and masses are rejected with GBH_ERR_ARG, and a corrupt tree (the GBH_FAULT_LINK hook)
stops each walk at its device-side step bound with GBH_ERR_LIMIT."""
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


def test_non_finite_positions_and_masses_are_rejected():
    """An alive star with a NaN or infinite coordinate or mass is rejected with GBH_ERR_ARG by the
    build's bounding-box reduction (collect, build.go:62-113, would otherwise carry a NaN into the
    root cube and every key); the context stays usable and dead bodies and black holes are not
    checked (they are not in the tree)."""
    s = ics.plummer(5000, seed=3)
    n = len(s["px"])
    s["kind"] = np.zeros(n, np.uint8)
    s["alive"] = np.ones(n, np.uint8)
    s["alive"][77] = 0
    s["kind"][91] = abi.BLACK_HOLE
    par = abi.make_params(0.5, 0.01, 16, False, False, "mixed")
    with abi.Context(0) as c0:
        want = forces(c0, s, par)
    with abi.Context(0) as c:
        for field in ("px", "py", "pz", "mass"):
            for bad in (np.nan, np.inf, -np.inf):
                t = dict(s)
                t[field] = s[field].copy()
                t[field][1234] = bad
                with pytest.raises(abi.GbhError) as ei:
                    forces(c, t, par)
                assert ei.value.code == abi.ERR_ARG and "non-finite" in str(ei.value), (field, bad)
                assert np.array_equal(forces(c, s, par), want)
        for i in (77, 91):  # the dead body and the black hole
            t = dict(s)
            t["px"] = s["px"].copy()
            t["px"][i] = np.nan
            assert np.array_equal(forces(c, t, par), want)
        # the step path and the other walks take the same check
        t = dict(s)
        t["pz"] = s["pz"].copy()
        t["pz"][4000] = np.inf
        with pytest.raises(abi.GbhError) as ei:
            steps(c, t, par, k=2)
        assert ei.value.code == abi.ERR_ARG
        for walk in ("plain", "fp64"):
            with pytest.raises(abi.GbhError) as ei:
                forces(c, t, abi.make_params(0.5, 0.01, 16, False, False, walk))
            assert ei.value.code == abi.ERR_ARG


def test_non_finite_inputs_of_a_forest_system_are_rejected():
    """Each system of a forest has its own bounding box; a non-finite star in one of them is
    rejected, and empty systems are not mistaken for non-finite ones."""
    parts = [ics.plummer(m, seed=10 + k) for k, m in enumerate((3000, 1700, 2500))]
    empty = {f: np.zeros(0) for f in parts[0]}
    parts.insert(1, empty)
    off = np.cumsum([0] + [len(p["px"]) for p in parts])
    cat = {f: np.concatenate([p[f] for p in parts]) for f in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
    par = abi.make_params(0.5, 0.01, 16, False, False, "mixed")
    with abi.Context(0) as c:
        c.forest_upload(off, *[cat[f] for f in ("px", "py", "pz", "vx", "vy", "vz", "mass")])
        c.call("gbh_state_accelerations", par)  # the empty system is fine
        bad = dict(cat)
        bad["mass"] = cat["mass"].copy()
        bad["mass"][off[2] + 5] = np.nan
        c.forest_upload(off, *[bad[f] for f in ("px", "py", "pz", "vx", "vy", "vz", "mass")])
        with pytest.raises(abi.GbhError) as ei:
            c.call("gbh_state_accelerations", par)
        assert ei.value.code == abi.ERR_ARG


@pytest.mark.parametrize("walk,group,kernel,flags", [("mixed", 64, 8, 0), ("mixed", 64, 4, abi.CFG_PAIRED),
                                                     ("mixed", 64, 4, abi.CFG_NO_SPLIT | abi.CFG_PAIRED),
                                                     ("mixed", 64, 8, abi.CFG_NO_SPLIT), ("mixed", 32, 8, 0),
                                                     ("plain", 0, 3, 0), ("fp64", 0, 1, 0)])
def test_walk_step_bound_stops_a_walk_on_a_corrupt_tree(walk, group, kernel, flags):
    """With the corrupt-link hook armed (GBH_FAULT_LINK when the context is created), the next
    tree's last leaf links back to node 0: every walk then cycles until its device-side step bound
    stops it, sets the error flag and the call returns GBH_ERR_LIMIT naming the walk kernel. The
    hook fires once, and the next call on the same context gives exactly the results of a fresh
    context. Indices stay in range, so the cycle is bounded work, not a fault."""
    s = ics.plummer(4096, seed=5)
    par = abi.make_params(0.5, 0.01, 8, False, False, walk, group_size=group)
    with abi.Context(0, flags) as c0:
        want = forces(c0, s, par)
    os.environ["GBH_FAULT_LINK"] = "1"
    try:
        c = abi.Context(0, flags)
    finally:
        os.environ.pop("GBH_FAULT_LINK", None)
    try:
        with pytest.raises(abi.GbhError) as ei:
            forces(c, s, par)
        assert ei.value.code == abi.ERR_LIMIT and f"kernel {kernel}" in str(ei.value), str(ei.value)
        assert np.array_equal(forces(c, s, par), want)
    finally:
        c.close()


def test_evolve_driver_stops_at_the_first_bad_body(tmp_path, capsys):
    """The headless driver checks the state after every step (firstBad, tools/evolve/main.go:63-74)
    and exits with status 1 naming the body, without writing the output file."""
    from gravitas_gb300 import evolve, snapshot

    s = ics.plummer(2000, seed=8)
    s["px"][17] = 2e6  # beyond the watchdog's bound once the first step has run
    src = os.path.join(tmp_path, "in.gravitas")
    out = os.path.join(tmp_path, "out.gravitas")
    snapshot.save(src, s, {"Dt": 1e-3, "Softening": 0.01})
    assert evolve.main(["--in", src, "-t", "0.005", "-o", out, "--leaf", "16"]) == 1
    assert "body 17" in capsys.readouterr().out and not os.path.exists(out)
    s["px"][17] = 0.5
    snapshot.save(src, s, {"Dt": 1e-3, "Softening": 0.01})
    assert evolve.main(["--in", src, "-t", "0.005", "-o", out, "--leaf", "16"]) == 0 and os.path.exists(out)
