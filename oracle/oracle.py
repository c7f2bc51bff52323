"""ctypes binding of the CPU oracle (oracle/bh_oracle.cpp).

TEST INFRASTRUCTURE ONLY: a C++ restatement of gravitas' CPU Barnes-Hut path
(internal/sim/bh/*.go, internal/sim/direct/direct.go, internal/sim/sim.go) used
as the parity oracle in tests/ and as the timed CPU baseline in bench.py. The
product path (gravitas_gb300) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

STAR, BLACK_HOLE, DARK_MATTER, GAS = 0, 1, 2, 3

NODE_DTYPE = np.dtype(
    [("x", "f8"), ("y", "f8"), ("z", "f8"), ("m", "f8"),
     ("qxx", "f8"), ("qyy", "f8"), ("qzz", "f8"), ("qxy", "f8"), ("qxz", "f8"), ("qyz", "f8"),
     ("crit2", "f8"), ("first", "i4"), ("next", "i4"), ("lo", "i4"), ("hi", "i4")])
assert NODE_DTYPE.itemsize == 104

_lib = None

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_INT = ctypes.c_int


def build() -> str:
    """Compile the oracle with its Makefile (a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "orc_morton_key": (ctypes.c_uint64, [ctypes.c_uint64] * 3),
            "orc_radix_sort": (None, [_P, _P, _I64]),
            "orc_radix_sort_parallel": (None, [_P, _P, _I64, _INT]),
            "orc_tree_new": (_P, []),
            "orc_tree_free": (None, [_P]),
            "orc_tree_build": (_I64, [_P, _I64, _P, _P, _P, _P, _P, _P, _D, _INT, _INT, _INT]),
            "orc_tree_nstars": (_I64, [_P]),
            "orc_tree_nnodes": (_I64, [_P]),
            "orc_tree_nholes": (_I64, [_P]),
            "orc_tree_box": (None, [_P, _P, _P]),
            "orc_tree_export": (None, [_P] * 9),
            "orc_tree_accelerations": (None, [_P, _I64, _D, _INT, _INT, _P, _P, _P]),
            "orc_tree_walk_point": (None, [_P, _D, _D, _D, ctypes.c_int32, _D, _INT, _P]),
            "orc_tree_walk_potential_point": (_D, [_P, _D, _D, _D, ctypes.c_int32, _D, _INT]),
            "orc_tree_counts": (None, [_P, _D, _INT, _INT, _P, _I64, _P, _P, _P]),
            "orc_tree_group_counts": (None, [_P, _INT, _INT, _P, _P, _P]),
            "orc_tree_walk_fp32": (None, [_P, _D, _INT, _P]),
            "orc_tree_potential": (_D, [_P, _I64, _P, _P, _P, _P, _P, _P, _D, _D, _INT, _INT, _INT]),
            "orc_direct": (None, [_I64, _P, _P, _P, _P, _P, _D, _INT, _INT, _P, _P, _P]),
            "orc_direct_targets": (None, [_I64, _P, _P, _P, _P, _P, _D, _INT, _P, _I64, _INT, _P, _P, _P]),
            "orc_kdk": (None, [_I64] + [_P] * 12 + [_D, _D, _D, _INT, _INT, _INT, _INT, _I64, _INT, _D]),
            "orc_potential_exact": (_D, [_I64, _P, _P, _P, _P, _P, _D, _D, _INT, _INT]),
            "orc_split_kdk": (None, [_I64] + [_P] * 12 + [_D, _D, _D, _INT, _INT, _INT, _INT, _I64, _INT, _P, _P, _D]),
            "orc_pair_force": (_D, [_D, _D, _D, _D]),
            "orc_pair_potential": (_D, [_D, _D, _D, _D, _D]),
            "orc_pair_rs": (_D, [ctypes.c_uint8, _D, ctypes.c_uint8, _D, _D]),
            "orc_adjoint_direct": (None, [_I64] + [_P] * 7 + [_D, _D, _I64, _I64] + [_P] * 13 + [_INT]),
            "orc_kdk_direct": (None, [_I64] + [_P] * 7 + [_D, _D, _I64, _INT]),
            "orc_block_kdk": (None, [_I64] + [_P] * 12 + [_D, _D, _INT, _D, _D, _INT, _INT, _INT, _INT, _I64, _INT,
                                                         _P, _P, _D]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


def morton_key(x: int, y: int, z: int) -> int:
    return int(lib().orc_morton_key(x, y, z))


def radix_sort(keys, idx, workers: int = 1):
    """Stable LSD sort of keys, applying the permutation to idx (in place copies returned)."""
    k = np.array(keys, dtype=np.uint64, copy=True)
    i = np.array(idx, dtype=np.int32, copy=True)
    if workers == 1:
        lib().orc_radix_sort(_ptr(k), _ptr(i), len(k))
    else:
        lib().orc_radix_sort_parallel(_ptr(k), _ptr(i), len(k), workers)
    return k, i


class Tree:
    """A Barnes-Hut tree built by the oracle for one state snapshot."""

    def __init__(self, px, py, pz, mass, kind=None, alive=None, theta=0.9, leaf=24,
                 dm_off=False, workers=0):
        n = len(px)
        self.n = n
        self.px, self.py, self.pz, self.mass = _f64(px), _f64(py), _f64(pz), _f64(mass)
        self.kind = _u8(kind if kind is not None else np.zeros(n, np.uint8))
        self.alive = _u8(alive if alive is not None else np.ones(n, np.uint8))
        self.dm_off = int(bool(dm_off))
        self.workers = workers
        self._t = lib().orc_tree_new()
        self.nnodes = lib().orc_tree_build(self._t, n, _ptr(self.px), _ptr(self.py), _ptr(self.pz),
                                           _ptr(self.mass), _ptr(self.kind), _ptr(self.alive),
                                           theta, leaf, self.dm_off, workers)
        self.nstars = lib().orc_tree_nstars(self._t)

    def __del__(self):
        if getattr(self, "_t", None):
            lib().orc_tree_free(self._t)
            self._t = None

    def box(self):
        mn = np.zeros(3)
        side = np.zeros(1)
        lib().orc_tree_box(self._t, _ptr(mn), _ptr(side))
        return mn, float(side[0])

    def export(self):
        ns, nn = self.nstars, self.nnodes
        keys = np.zeros(ns, np.uint64)
        order = np.zeros(ns, np.int32)
        nodes = np.zeros(nn, NODE_DTYPE)
        sx, sy, sz, sm = (np.zeros(ns) for _ in range(4))
        holes = np.zeros(lib().orc_tree_nholes(self._t), np.int32)
        lib().orc_tree_export(self._t, _ptr(keys), _ptr(order), _ptr(nodes), _ptr(sx), _ptr(sy),
                              _ptr(sz), _ptr(sm), _ptr(holes))
        return dict(keys=keys, order=order, nodes=nodes, sx=sx, sy=sy, sz=sz, sm=sm, holes=holes)

    def accelerations(self, eps, monopole_only=False, workers=None, acc=None):
        """Accelerations in state order; entries of dead bodies keep acc's values."""
        n = self.n
        ax, ay, az = (np.zeros(n) for _ in range(3)) if acc is None else acc
        lib().orc_tree_accelerations(self._t, n, eps, int(monopole_only),
                                     self.workers if workers is None else workers,
                                     _ptr(ax), _ptr(ay), _ptr(az))
        return np.stack([ax, ay, az], axis=1)

    def walk_point(self, x, y, z, eps2, self_idx=-1, monopole_only=False):
        a = np.zeros(3)
        lib().orc_tree_walk_point(self._t, x, y, z, self_idx, eps2, int(monopole_only), _ptr(a))
        return a

    def walk_potential_point(self, x, y, z, eps2, self_idx=-1, monopole_only=False):
        return lib().orc_tree_walk_potential_point(self._t, x, y, z, self_idx, eps2, int(monopole_only))

    def counts(self, eps, monopole_only=False, targets=None, workers=None):
        """(accepted nodes, leaf pairs, opened nodes) of the per-target reference walk."""
        a, b, c = (np.zeros(1, np.int64) for _ in range(3))
        t = None if targets is None else np.ascontiguousarray(targets, np.int32)
        lib().orc_tree_counts(self._t, eps, int(monopole_only),
                              self.workers if workers is None else workers,
                              _ptr(t), 0 if t is None else len(t), _ptr(a), _ptr(b), _ptr(c))
        return int(a[0]), int(b[0]), int(c[0])

    def group_counts(self, group=64, workers=None):
        """(accepted nodes, leaf pairs, opened nodes) summed over the stars of the group walk the
        GPU's mixed walk executes (groups of `group` consecutive sorted stars, any-open)."""
        a, b, c = (np.zeros(1, np.int64) for _ in range(3))
        lib().orc_tree_group_counts(self._t, int(group), self.workers if workers is None else workers,
                                    _ptr(a), _ptr(b), _ptr(c))
        return int(a[0]), int(b[0]), int(c[0])

    def walk_fp32(self, eps, workers=None):
        out = np.zeros((self.nstars, 3), np.float32)
        lib().orc_tree_walk_fp32(self._t, eps, self.workers if workers is None else workers, _ptr(out))
        return out

    def potential(self, eps, c=0.0, monopole_only=False, workers=None):
        return lib().orc_tree_potential(self._t, self.n, _ptr(self.px), _ptr(self.py), _ptr(self.pz),
                                        _ptr(self.mass), _ptr(self.kind), _ptr(self.alive), eps, c,
                                        self.dm_off, int(monopole_only),
                                        self.workers if workers is None else workers)


def direct(px, py, pz, mass, kind=None, eps=0.0, dm_off=False, workers=0, targets=None):
    """FP64 direct-sum accelerations (direct.go:18-48); rows follow targets when given."""
    n = len(px)
    px, py, pz, mass = _f64(px), _f64(py), _f64(pz), _f64(mass)
    kind = _u8(kind if kind is not None else np.zeros(n, np.uint8))
    if targets is None:
        ax, ay, az = (np.zeros(n) for _ in range(3))
        lib().orc_direct(n, _ptr(px), _ptr(py), _ptr(pz), _ptr(mass), _ptr(kind), eps, int(dm_off),
                         workers, _ptr(ax), _ptr(ay), _ptr(az))
    else:
        t = np.ascontiguousarray(targets, np.int64)
        ax, ay, az = (np.zeros(len(t)) for _ in range(3))
        lib().orc_direct_targets(n, _ptr(px), _ptr(py), _ptr(pz), _ptr(mass), _ptr(kind), eps,
                                 int(dm_off), _ptr(t), len(t), workers, _ptr(ax), _ptr(ay), _ptr(az))
    return np.stack([ax, ay, az], axis=1)


def potential_exact(px, py, pz, mass, kind=None, eps=0.0, c=0.0, dm_off=False, workers=0):
    n = len(px)
    kind = _u8(kind if kind is not None else np.zeros(n, np.uint8))
    return lib().orc_potential_exact(n, _ptr(_f64(px)), _ptr(_f64(py)), _ptr(_f64(pz)),
                                     _ptr(_f64(mass)), _ptr(kind), eps, c, int(dm_off), workers)


def kdk(state: dict, dt, eps, theta, leaf, nsteps, monopole_only=False, dm_off=False,
        acc_valid=False, workers=0, c=0.0):
    """nsteps KDK steps (sim.go:252-288, no holes, no gas; drift of u / gamma when c > 0) on a
    dict of SoA arrays, in place."""
    s = state
    n = len(s["px"])
    for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass"):
        assert s[k].dtype == np.float64 and s[k].flags.c_contiguous
    kind = _u8(s.get("kind", np.zeros(n, np.uint8)))
    alive = _u8(s.get("alive", np.ones(n, np.uint8)))
    lib().orc_kdk(n, *[_ptr(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")],
                  _ptr(kind), _ptr(alive), dt, eps, theta, leaf, int(monopole_only), int(dm_off),
                  int(acc_valid), nsteps, workers, float(c))
    return s


def block_kdk(state: dict, dt, eta, levels, eps, theta, leaf, nsteps, monopole_only=False, dm_off=False,
              acc_valid=False, workers=0, c=0.0):
    """Block-step KDK (the scheme of gbh_state_step_block) on a dict of SoA arrays, in place;
    returns (events, walked stars)."""
    s = state
    n = len(s["px"])
    kind = _u8(s.get("kind", np.zeros(n, np.uint8)))
    alive = _u8(s.get("alive", np.ones(n, np.uint8)))
    a, b = np.zeros(1, np.int64), np.zeros(1, np.int64)
    lib().orc_block_kdk(n, *[_ptr(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")],
                        _ptr(kind), _ptr(alive), dt, eta, levels, eps, theta, leaf, int(monopole_only), int(dm_off),
                        int(acc_valid), nsteps, workers, _ptr(a), _ptr(b), float(c))
    return int(a[0]), int(b[0])


def kdk_direct(state: dict, dt, eps, nsteps, workers=0):
    """nsteps KDK steps with the FP64 direct-sum force, in place on px..vz (mass read)."""
    s = state
    n = len(s["px"])
    lib().orc_kdk_direct(n, *[_ptr(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")], eps, dt, nsteps,
                         workers)
    return s


def adjoint_direct(state: dict, dt, eps, nsteps, every, gx, gv, workers=0):
    """Gradient w.r.t. initial (x, v, m) of a loss whose gradient w.r.t. the final positions and
    velocities is (gx, gv) (each n x 3), for the KDK trajectory with the direct-sum force."""
    s = state
    n = len(s["px"])
    gx = np.ascontiguousarray(np.asarray(gx, np.float64).T)
    gv = np.ascontiguousarray(np.asarray(gv, np.float64).T)
    out = np.zeros((7, n))
    lib().orc_adjoint_direct(n, *[_ptr(_f64(s[k])) for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")], eps, dt,
                             nsteps, every, _ptr(gx[0]), _ptr(gx[1]), _ptr(gx[2]), _ptr(gv[0]), _ptr(gv[1]),
                             _ptr(gv[2]), *[_ptr(out[k]) for k in range(7)], workers)
    return out[0:3].T.copy(), out[3:6].T.copy(), out[6].copy()


def split_kdk(state: dict, dt, eps, theta, leaf, nsteps, monopole_only=False, dm_off=False, acc_valid=False,
              workers=0, c=0.0):
    """The hole-aware step (split.go, no gas, instant gravity, no spins) on a dict of SoA arrays,
    in place; returns (substeps of the last step, near flags of the last step)."""
    s = state
    n = len(s["px"])
    for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass"):
        assert s[k].dtype == np.float64 and s[k].flags.c_contiguous
    kind = _u8(s.get("kind", np.zeros(n, np.uint8)))
    alive = _u8(s.get("alive", np.ones(n, np.uint8)))
    sub = np.zeros(1, np.int64)
    near = np.zeros(n, np.uint8)
    lib().orc_split_kdk(n, *[_ptr(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az", "mass")],
                        _ptr(kind), _ptr(alive), dt, eps, theta, leaf, int(monopole_only), int(dm_off),
                        int(acc_valid), nsteps, workers, _ptr(sub), _ptr(near), float(c))
    return int(sub[0]), near.astype(bool)


def pair_force(m, r2, eps2, rs):
    return lib().orc_pair_force(m, r2, eps2, rs)


def pair_potential(mi, mj, r2, eps2, rs):
    return lib().orc_pair_potential(mi, mj, r2, eps2, rs)


def pair_rs(ki, mi, kj, mj, c):
    return lib().orc_pair_rs(ki, mi, kj, mj, c)
