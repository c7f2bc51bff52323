"""CPU tests of the C-ABI library: it builds, loads, exports every declared symbol, and fails
cleanly (an error code, no abort) where no GPU is present."""
import ctypes
import subprocess

import pytest

from gravitas_gb300 import abi, build


def test_library_builds_and_loads():
    path = build.build()
    L = abi.load()
    assert L is not None and path.endswith("libgbh.so")


def test_exports_every_declared_symbol():
    declared = abi.header_symbols()
    assert len(declared) >= 16
    L = abi.load()
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(abi.SIGNATURES), "binding and header disagree"
    out = subprocess.run(["nm", "-D", "--defined-only", abi.lib_path()], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(declared) <= exported


def test_create_fails_cleanly_without_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = abi.load()
    h = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    rc = L.gbh_create(None, ctypes.byref(h), err, 256)
    assert rc in (abi.ERR_CUDA, abi.ERR_ARG)
    assert not h.value
    assert err.value  # a message, not a crash
    with pytest.raises(abi.GbhError):
        abi.Context(0)


def test_null_context_is_rejected():
    L = abi.load()
    assert L.gbh_last_error(None) == b"NULL context"
    assert L.gbh_accelerations(None, None, 0, *([None] * 9)) == abi.ERR_ARG
    L.gbh_destroy(None)  # no-op


def test_params_layout_matches_header():
    assert ctypes.sizeof(abi.Params) == 48
    assert ctypes.sizeof(abi.AdjointParams) == 56
    assert ctypes.sizeof(abi.TuneEntry) == 64
    assert ctypes.sizeof(abi.Diagnostics) == 112
    assert ctypes.sizeof(abi.Config) == 32
    assert ctypes.sizeof(abi.Timings) == 80
    assert abi.NODE_DTYPE.itemsize == 104
