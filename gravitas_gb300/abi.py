"""ctypes binding of libgbh.so (include/gbh.h).

The library is the only compute path: there is no CPU fallback. Loading fails with a
RuntimeError when libgbh.so has not been built (gravitas_gb300.build.build()), and every
call that fails raises GbhError with the library's message.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "gbh.h")

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_LIMIT, ERR_STATE, ERR_UNSUPPORTED = range(7)
STAR, BLACK_HOLE, DARK_MATTER, GAS = 0, 1, 2, 3
WALK_MIXED, WALK_PLAIN, WALK_FP64 = 0, 1, 2
WALKS = {"mixed": WALK_MIXED, "plain": WALK_PLAIN, "fp64": WALK_FP64}


class GbhError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gbh error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [("theta", ctypes.c_double), ("softening", ctypes.c_double), ("leaf_size", ctypes.c_int32),
                ("monopole_only", ctypes.c_int32), ("dark_matter_off", ctypes.c_int32), ("walk", ctypes.c_int32),
                ("group_size", ctypes.c_int32), ("list_depth", ctypes.c_int32), ("c", ctypes.c_double)]


CFG_NO_GRAPHS = 1
CFG_BLOCKING_SYNC = 2
CFG_NO_LPT = 4
CFG_NO_SPLIT = 8
CFG_PAIRED = 16


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("flags", ctypes.c_int32), ("reserved", ctypes.c_int32 * 6)]


class Timings(ctypes.Structure):
    _fields_ = [("build_ms", ctypes.c_double), ("walk_ms", ctypes.c_double), ("step_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("nstars", ctypes.c_int64), ("nnodes", ctypes.c_int64),
                ("launches", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64),
                ("substeps", ctypes.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BlockStats(ctypes.Structure):
    _fields_ = [("substeps", ctypes.c_int64), ("evaluations", ctypes.c_int64), ("min_substep_ticks", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class Diagnostics(ctypes.Structure):
    _fields_ = [("kinetic", ctypes.c_double), ("potential", ctypes.c_double), ("total", ctypes.c_double),
                ("momentum", ctypes.c_double * 3), ("angular_momentum", ctypes.c_double * 3),
                ("center_of_mass", ctypes.c_double * 3), ("mass", ctypes.c_double), ("quality", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {k: (list(getattr(self, k)) if k in ("momentum", "angular_momentum", "center_of_mass")
                    else getattr(self, k)) for k, _ in self._fields_}


class AdjointParams(ctypes.Structure):
    _fields_ = [("dt", ctypes.c_double), ("softening", ctypes.c_double), ("nsteps", ctypes.c_int64),
                ("every", ctypes.c_int64), ("precision", ctypes.c_int32), ("force", ctypes.c_int32),
                ("leaf_size", ctypes.c_int32), ("reserved", ctypes.c_int32), ("theta", ctypes.c_double)]


ADJ_FP32 = 0
ADJ_FP64 = 1
ADJ_DIRECT = 0
ADJ_TREE = 1


class TuneEntry(ctypes.Structure):
    _fields_ = [("theta", ctypes.c_double), ("leaf_size", ctypes.c_int32), ("group_size", ctypes.c_int32),
                ("ms", ctypes.c_double), ("build_ms", ctypes.c_double), ("walk_ms", ctypes.c_double),
                ("rms_err", ctypes.c_double), ("p99_err", ctypes.c_double), ("meets", ctypes.c_int32),
                ("list_depth", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

NODE_DTYPE = np.dtype(
    [("x", "f8"), ("y", "f8"), ("z", "f8"), ("m", "f8"),
     ("qxx", "f8"), ("qyy", "f8"), ("qzz", "f8"), ("qxy", "f8"), ("qxz", "f8"), ("qyz", "f8"),
     ("crit2", "f8"), ("first", "i4"), ("next", "i4"), ("lo", "i4"), ("hi", "i4")])
assert NODE_DTYPE.itemsize == 104

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_D = ctypes.c_double
_I32 = ctypes.c_int32
_PP = ctypes.POINTER(Params)

SIGNATURES = {
    "gbh_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_P), ctypes.c_char_p, ctypes.c_int]),
    "gbh_destroy": (None, [_P]),
    "gbh_last_error": (ctypes.c_char_p, [_P]),
    "gbh_device_name": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int]),
    "gbh_accelerations": (ctypes.c_int, [_P, _PP, _I64] + [_P] * 9),
    "gbh_potential_energy": (ctypes.c_int, [_P, _PP, _I64] + [_P] * 6 + [_D, _P]),
    "gbh_direct_accelerations": (ctypes.c_int, [_P, _PP, _I64] + [_P] * 6 + [_I64, _P, _P, _P]),
    "gbh_step_kdk": (ctypes.c_int, [_P, _PP, _D, _I64, _I32, _I64] + [_P] * 12),
    "gbh_state_upload": (ctypes.c_int, [_P, _I64] + [_P] * 12),
    "gbh_state_download": (ctypes.c_int, [_P] + [_P] * 9),
    "gbh_state_step": (ctypes.c_int, [_P, _PP, _D, _I64]),
    "gbh_state_accelerations": (ctypes.c_int, [_P, _PP]),
    "gbh_tree_size": (ctypes.c_int, [_P, _P, _P]),
    "gbh_tree_export": (ctypes.c_int, [_P, _P, _P, _P, _I64]),
    "gbh_last_timings": (ctypes.c_int, [_P, ctypes.POINTER(Timings)]),
    "gbh_probe_fp32_peak": (ctypes.c_int, [_P, _D, _P]),
    "gbh_state_diagnostics": (ctypes.c_int, [_P, _PP, _D, _P]),
    "gbh_state_step_block": (ctypes.c_int, [_P, _PP, _D, _D, _I32, _I64, _P]),
    "gbh_forest_upload": (ctypes.c_int, [_P, _I32, _P] + [_P] * 12),
    "gbh_forest_layout": (ctypes.c_int, [_P, _I32, _P, _P]),
    "gbh_morton_order_noalloc": (ctypes.c_int, [_I32, _P, _I64] + [_P] * 8 + [ctypes.c_char_p, ctypes.c_int]),
    "gbh_fwd_save": (ctypes.c_int, [_P, ctypes.POINTER(AdjointParams), _I64] + [_P] * 13),
    "gbh_bwd": (ctypes.c_int, [_P] + [_P] * 13),
    "gbh_autotune": (ctypes.c_int, [_P, _PP, _P, _I32, _P, _I32, _P, _I32, _D, _I32, _I32, _PP, _P, _I32, _P]),
}

_lib = None


def header_symbols() -> list[str]:
    """Function names declared in include/gbh.h."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbh_[a-z0-9_]+)\s*\(", text)))


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Loads libgbh.so. Raises RuntimeError when it is missing (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with gravitas_gb300.build.build() "
                               "(the CUDA library is the only compute path)")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    if isinstance(a, int):  # raw address (e.g. pinned host memory)
        return ctypes.c_void_p(a)
    return a


def make_params(theta=0.0, softening=0.0, leaf_size=0, monopole_only=False, dark_matter_off=False,
                walk="mixed", group_size=0, c=0.0, list_depth=0) -> Params:
    w = WALKS[walk] if isinstance(walk, str) else int(walk)
    return Params(float(theta), float(softening), int(leaf_size), int(bool(monopole_only)),
                  int(bool(dark_matter_off)), w, int(group_size), int(list_depth), float(c))


class Context:
    """One gbh_ctx (one device, one stream)."""

    def __init__(self, device: int = 0, flags: int = 0):
        L = load()
        cfg = Config(device, flags, (ctypes.c_int32 * 6)())
        h = _P()
        err = ctypes.create_string_buffer(512)
        rc = L.gbh_create(ctypes.byref(cfg), ctypes.byref(h), err, 512)
        if rc != OK:
            raise GbhError(rc, err.value.decode())
        self._h = h
        self._L = L

    def close(self):
        if getattr(self, "_h", None):
            self._L.gbh_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def check(self, rc: int):
        if rc != OK:
            raise GbhError(rc, self._L.gbh_last_error(self._h).decode())

    def call(self, name: str, *args):
        self.check(getattr(self._L, name)(self._h, *args))

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        self.call("gbh_device_name", buf, 256)
        return buf.value.decode()

    def timings(self) -> dict:
        t = Timings()
        self.check(self._L.gbh_last_timings(self._h, ctypes.byref(t)))
        return t.as_dict()

    def tree_size(self):
        a, b = np.zeros(1, np.int64), np.zeros(1, np.int64)
        self.call("gbh_tree_size", ptr(a), ptr(b))
        return int(a[0]), int(b[0])

    def tree_export(self):
        ns, nn = self.tree_size()
        keys = np.zeros(ns, np.uint64)
        order = np.zeros(ns, np.int32)
        nodes = np.zeros(nn, NODE_DTYPE)
        self.call("gbh_tree_export", ptr(keys), ptr(order), ptr(nodes), nn)
        return dict(keys=keys, order=order, nodes=nodes)

    def forest_upload(self, offsets, px, py, pz, vx, vy, vz, mass, kind=None, alive=None, acc=None):
        off = np.ascontiguousarray(offsets, np.int64)
        ax, ay, az = (None, None, None) if acc is None else acc
        self.call("gbh_forest_upload", len(off) - 1, ptr(off), ptr(px), ptr(py), ptr(pz), ptr(vx), ptr(vy), ptr(vz),
                  ptr(ax), ptr(ay), ptr(az), ptr(mass), ptr(kind), ptr(alive))

    def forest_layout(self, nsys: int):
        stars = np.zeros(2 * nsys, np.int64)
        nodes = np.zeros(2 * nsys, np.int64)
        self.call("gbh_forest_layout", nsys, ptr(stars), ptr(nodes))
        return stars.reshape(nsys, 2), nodes.reshape(nsys, 2)

    def step_block(self, params: Params, dt: float, eta: float, levels: int, nsteps: int) -> dict:
        st = BlockStats()
        self.call("gbh_state_step_block", params, float(dt), float(eta), int(levels), int(nsteps), ctypes.byref(st))
        return st.as_dict()

    def diagnostics(self, params: Params, c: float = 0.0) -> dict:
        d = Diagnostics()
        self.call("gbh_state_diagnostics", params, float(c), ctypes.byref(d))
        return d.as_dict()

    def fwd_save(self, x0: np.ndarray, v0: np.ndarray, mass: np.ndarray, dt: float, softening: float,
                 nsteps: int, every: int, precision: int = ADJ_FP32, force: int = ADJ_DIRECT, theta: float = 0.0,
                 leaf: int = 0):
        """Forward half of the adjoint pair: (x_T, v_T), each n x 3, with the tape kept on the device.
        force=ADJ_TREE steps with the Barnes-Hut force at theta and leaf size leaf."""
        x0 = np.ascontiguousarray(np.asarray(x0, np.float64).T)
        v0 = np.ascontiguousarray(np.asarray(v0, np.float64).T)
        m = np.ascontiguousarray(mass, np.float64)
        n = m.shape[0]
        out = np.empty((6, n))
        ap = AdjointParams(float(dt), float(softening), int(nsteps), int(every), int(precision), int(force),
                           int(leaf), 0, float(theta))
        self.call("gbh_fwd_save", ctypes.byref(ap), n, *[ptr(x0[k]) for k in range(3)],
                  *[ptr(v0[k]) for k in range(3)], ptr(m), *[ptr(out[k]) for k in range(6)])
        return out[0:3].T.copy(), out[3:6].T.copy()

    def bwd(self, gx: np.ndarray | None, gv: np.ndarray | None):
        """Backward half: (dL/dx_0, dL/dv_0) as n x 3 and dL/dm, from dL/dx_T and dL/dv_T."""
        g = [None] * 6
        keep = []
        for k, a in ((0, gx), (3, gv)):
            if a is not None:
                a = np.ascontiguousarray(np.asarray(a, np.float64).T)
                keep.append(a)
                for c in range(3):
                    g[k + c] = ptr(a[c])
        n = keep[0].shape[1] if keep else None
        if n is None:
            raise ValueError("bwd needs gx or gv")
        out = np.empty((7, n))
        self.call("gbh_bwd", *g, *[ptr(out[k]) for k in range(7)])
        return out[0:3].T.copy(), out[3:6].T.copy(), out[6].copy()

    def autotune(self, params: Params, thetas=None, leaves=None, groups=None, rms_bound: float = 2e-3,
                 sample: int = 1024, reps: int = 3, strict: bool = False):
        """gbh_autotune on the resident state: (best Params, candidates as dicts). With strict,
        a sweep in which no candidate meets rms_bound raises; otherwise the most accurate wins."""
        th = None if thetas is None else np.ascontiguousarray(thetas, np.float64)
        lv = None if leaves is None else np.ascontiguousarray(leaves, np.int32)
        gr = None if groups is None else np.ascontiguousarray(groups, np.int32)
        cap = 4096
        table = (TuneEntry * cap)()
        best = Params()
        cnt = np.zeros(1, np.int32)
        rc = self._L.gbh_autotune(self._h, ctypes.byref(params), ptr(th), 0 if th is None else len(th), ptr(lv),
                                   0 if lv is None else len(lv), ptr(gr), 0 if gr is None else len(gr),
                                   float(rms_bound), int(sample), int(reps), ctypes.byref(best),
                                   ctypes.cast(table, ctypes.c_void_p), cap, ptr(cnt))
        if rc != OK and (strict or rc != ERR_LIMIT):
            raise GbhError(rc, self._L.gbh_last_error(self._h).decode())
        return best, [table[k].as_dict() for k in range(min(int(cnt[0]), cap))]

    def probe_fp32_peak(self, ms: float = 50.0) -> float:
        out = np.zeros(1)
        self.call("gbh_probe_fp32_peak", ms, ptr(out))
        return float(out[0])
