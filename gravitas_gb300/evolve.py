"""Headless evolution to a save file, the gravity-only counterpart of tools/evolve (main.go:22-100):
build a scene (or continue from a .gravitas snapshot), step it with the GPU solver until the
simulated time reaches -t, report progress, stop with exit status 1 at the first body whose state
is NaN or beyond 1e6 in magnitude (the watchdog firstBad, main.go:63-74 and 185-194), and write
the state as a snapshot.

    python -m gravitas_gb300.evolve --scene merger --n 1048576 -t 0.05 -o evolved.gravitas
    python -m gravitas_gb300.evolve --in evolved.gravitas -t 0.1 -o later.gravitas

The scenes are this package's generators (ics.py); the reference's presets and its SPH gas are
not part of this library.
"""
from __future__ import annotations

import argparse
import sys
import time

import numpy as np

from . import abi, ics
from .sim import Params, Simulation, Solver, State

SCENES = {
    "plummer": lambda n, seed: ics.plummer(n, seed=seed),
    "galaxy": lambda n, seed: ics.galaxy(n, seed=seed),
    "merger": lambda n, seed: ics.merger(n, seed=seed),
    "disk": lambda n, seed: ics.test_disk(n, seed=seed),
}


def first_bad(s: State) -> int:
    """firstBad (tools/evolve/main.go:185-194): the first body whose x position, x velocity or x
    acceleration is NaN or larger than 1e6 in magnitude (infinities included), or -1. The
    reference also tests the gas fields U and H, which this library does not hold."""
    bad = np.zeros(len(s), bool)
    for a in (s.pos_x, s.vel_x, s.acc_x):
        bad |= np.isnan(a) | (np.abs(a) > 1e6)
    idx = np.flatnonzero(bad)
    return int(idx[0]) if len(idx) else -1


def report_bad(m: Simulation, i: int, out=None) -> None:
    """The watchdog's report (main.go:64-72): the bad body, then every black hole's mass, distance
    and speed (to standard output, as the reference prints it)."""
    out = out or sys.stdout
    s = m.state
    print(f"step {m.steps} t={m.time:.5f}: body {i} kind {s.kind[i]} pos ({s.pos_x[i]:g} {s.pos_y[i]:g} "
          f"{s.pos_z[i]:g}) vel ({s.vel_x[i]:g} {s.vel_y[i]:g} {s.vel_z[i]:g}) acc ({s.acc_x[i]:g} {s.acc_y[i]:g} "
          f"{s.acc_z[i]:g}) m {s.mass[i]:g}", file=out)
    for h in np.flatnonzero(s.kind == abi.BLACK_HOLE):
        d = np.sqrt((s.pos_x[h] - s.pos_x[i]) ** 2 + (s.pos_y[h] - s.pos_y[i]) ** 2 + (s.pos_z[h] - s.pos_z[i]) ** 2)
        v = np.sqrt(s.vel_x[h] ** 2 + s.vel_y[h] ** 2 + s.vel_z[h] ** 2)
        print(f"  hole {h} m {s.mass[h]:g} at distance {d:g}, speed {v:g}", file=out)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--scene", choices=sorted(SCENES), default="plummer")
    ap.add_argument("--n", type=int, default=60000, help="number of bodies")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("-t", type=float, default=0.5, help="simulation time to reach")
    ap.add_argument("--dt", type=float, default=1e-3)
    ap.add_argument("--softening", type=float, default=0.01)
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--leaf", type=int, default=24)
    ap.add_argument("--every", type=float, default=0.0, help="also report progress every this much simulation time")
    ap.add_argument("--in", dest="inp", default="", help="continue from this save file instead of building the scene")
    ap.add_argument("-o", default="evolved.gravitas", help="save file to write")
    ap.add_argument("--chunk", type=int, default=1,
                    help="steps per library call; the watchdog looks at the state after every call (1: after "
                         "every step, as the reference does)")
    a = ap.parse_args(argv)

    solver = Solver(theta=a.theta, leaf_size=a.leaf)
    if a.inp:
        m = Simulation.load(a.inp, solver)
    else:
        m = Simulation(State.from_dict(SCENES[a.scene](a.n, a.seed)), solver, Params(dt=a.dt, softening=a.softening))
    if not m.params.dt > 0:
        print("evolve: the time step must be positive", file=sys.stderr)
        return 2
    start, nxt, steps = time.perf_counter(), m.time + a.every, 0
    while m.time < a.t:
        k = max(1, min(a.chunk, int(np.ceil((a.t - m.time) / m.params.dt - 1e-9))))
        m.step(k)
        steps += k
        i = first_bad(m.state)
        if i >= 0:
            report_bad(m, i)
            return 1
        if a.every > 0 and m.time >= nxt:
            nxt += a.every
            el = time.perf_counter() - start
            print(f"t={m.time:.4f} steps={m.steps} {len(m.state) * steps / el:.3g} particle-steps/s", flush=True)
    m.save(a.o)
    el = time.perf_counter() - start
    print(f"wrote {a.o}: {len(m.state)} bodies, t={m.time:.5f}, {m.steps} steps "
          f"({steps} this run, {el:.1f} s)", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
