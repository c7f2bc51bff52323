"""Generates the golden fixtures in tests/golden/ from the CPU oracle.

The reference stores no golden vectors for its Barnes-Hut path (its tests build fixtures in
code, internal/sim/bh/bh_test.go:54-63); these fixtures freeze the oracle's outputs for seeded
inputs, so the CUDA path and future oracle changes are checked against fixed numbers:

  kat.npz         bh_test.go:137-147 known answer (two stars and a hole, eps = 0)
  plummer.npz     Plummer N=2048, theta 0.5, leaf 8, eps 0.01: keys, order, node table,
                  FP64 accelerations, float32 Metal-walk accelerations, potential
  disk.npz        test disk N=1500 + 2 holes, theta 0.9, leaf 24, eps 0.06: accelerations,
                  node table, potential with c = 10
  kdk.npz         Plummer N=512, theta 0.5, leaf 8, eps 0.01, dt 1e-3: 5 KDK steps

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from gravitas_gb300 import ics  # noqa: E402
from oracle import oracle as O  # noqa: E402


def state_arrays(s):
    return {k: s[k] for k in ("px", "py", "pz", "vx", "vy", "vz", "mass", "kind", "alive")}


def tree_fixture(s, theta, leaf, eps, c=0.0):
    t = O.Tree(s["px"], s["py"], s["pz"], s["mass"], s["kind"], s["alive"], theta=theta, leaf=leaf, workers=1)
    e = t.export()
    acc = t.accelerations(eps)
    out = dict(state_arrays(s), theta=theta, leaf=leaf, eps=eps, keys=e["keys"], order=e["order"],
               nodes=e["nodes"], acc=acc, counts=np.array(t.counts(eps)))
    if not np.any(s["kind"] == O.BLACK_HOLE):
        out["acc_fp32_sorted"] = t.walk_fp32(eps)
    tp = O.Tree(s["px"], s["py"], s["pz"], s["mass"], s["kind"], s["alive"], theta=min(theta, 0.9), leaf=leaf,
                workers=1)
    out["potential"] = np.array(tp.potential(eps, c=c))
    out["c"] = c
    return out


def main():
    z = np.zeros(3)
    np.savez_compressed(os.path.join(HERE, "kat.npz"), px=np.array([1.0, 2.0, 0.0]), py=z, pz=z,
                        mass=np.array([1.0, 2.0, 4.0]), kind=np.array([0, 0, 1], np.uint8),
                        alive=np.ones(3, np.uint8),
                        acc=np.array([[2.0, 0, 0], [-1.0, 0, 0], [0, 0, 0]]))
    np.savez_compressed(os.path.join(HERE, "plummer.npz"), **tree_fixture(ics.plummer(2048, seed=3), 0.5, 8, 0.01))
    np.savez_compressed(os.path.join(HERE, "disk.npz"), **tree_fixture(ics.test_disk(1500, seed=1), 0.9, 24, 0.06,
                                                                       c=10.0))
    s = ics.plummer(512, seed=4)
    init = state_arrays(s)
    st = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")}
    O.kdk(st, dt=1e-3, eps=0.01, theta=0.5, leaf=8, nsteps=5, workers=1)
    np.savez_compressed(os.path.join(HERE, "kdk.npz"), **{f"in_{k}": v for k, v in init.items()},
                        **{f"out_{k}": st[k] for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")},
                        dt=1e-3, eps=0.01, theta=0.5, leaf=8, nsteps=5)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
