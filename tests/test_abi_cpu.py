"""CPU: the C-ABI library loads and exports every symbol the header declares;
argument checks that fail before any CUDA call behave as documented."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lightprop2d_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from lightprop2d_gb300 import build
    build.build()
    from lightprop2d_gb300 import _lib
    return _lib.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lp_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "lp_propagate" in names and "lp_propagate_field" in names
    assert len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    from lightprop2d_gb300 import _lib
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} missing from the shared library"
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"


def test_meta_calls(lib):
    assert lib.lp_abi_version() == 1
    # powers of two 16..8192 (the pass kernels) and any other n in 2..4096
    # (Bluestein transforms)
    for n in (2, 3, 8, 100, 75, 4095, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192):
        assert lib.lp_is_supported_n(n) == 1
    for n in (0, 1, 4097, 6000, 16384, -4):
        assert lib.lp_is_supported_n(n) == 0
    assert lib.lp_status_string(0) == b"ok"


def test_validation_before_any_device_call(lib):
    from lightprop2d_gb300 import _lib as L
    vp = ctypes.c_void_p
    # unsupported size: rejected before touching CUDA
    st = lib.lp_fft2(vp(256), vp(256), 5000, 0, vp(0))
    assert st == L.LP_ERR_UNSUPPORTED_SIZE
    assert b"npoints=5000" in lib.lp_last_error()
    # NULL pointer
    st = lib.lp_fft2(vp(0), vp(256), 64, 0, vp(0))
    assert st == L.LP_ERR_INVALID_ARGUMENT
    # misaligned pointer
    st = lib.lp_fft2(vp(260), vp(256), 64, 0, vp(0))
    assert st == L.LP_ERR_MISALIGNED
    # bad geometry
    st = lib.lp_propagate(vp(256), vp(512), 64, -1.0, 1e-4, 1.0, vp(0), 0, 0, vp(0))
    assert st == L.LP_ERR_INVALID_ARGUMENT
    # bad mask type
    st = lib.lp_propagate(vp(256), vp(512), 64, 1.0, 1e-4, 1.0, vp(0), 99, 0, vp(0))
    assert st == L.LP_ERR_INVALID_ARGUMENT
    with pytest.raises(ValueError):
        L.check(L.LP_ERR_UNSUPPORTED_SIZE, "x")
    with pytest.raises(MemoryError):
        L.check(L.LP_ERR_OUT_OF_MEMORY, "x")
    with pytest.raises(L.BackendError):
        L.check(L.LP_ERR_CUDA, "x")


def test_batch_validation_before_any_device_call(lib):
    from lightprop2d_gb300 import _lib as L
    vp = ctypes.c_void_p
    out = vp()

    def create(descs, opts=None):
        arr = (L.BeamDesc * max(1, len(descs)))(*descs)
        return lib.lp_batch_create(arr, len(descs), opts, ctypes.byref(out))

    ok = dict(field=4096, iprofile=0, n=256, area_size=0.2, wl=632e-7, z=1.0, lens_f=0.0,
              flags=0)
    assert create([]) == L.LP_ERR_INVALID_ARGUMENT
    assert create([L.BeamDesc(**{**ok, "n": 100})]) == L.LP_ERR_UNSUPPORTED_SIZE
    assert create([L.BeamDesc(**{**ok, "n": 32})]) == L.LP_ERR_UNSUPPORTED_SIZE
    assert create([L.BeamDesc(**ok), L.BeamDesc(**{**ok, "n": 8192})]) == \
        L.LP_ERR_UNSUPPORTED_SIZE
    assert b"beam 1" in lib.lp_last_error()
    assert create([L.BeamDesc(**{**ok, "field": 0})]) == L.LP_ERR_INVALID_ARGUMENT
    assert create([L.BeamDesc(**{**ok, "field": 4100})]) == L.LP_ERR_MISALIGNED
    assert create([L.BeamDesc(**{**ok, "iprofile": 4098})]) == L.LP_ERR_MISALIGNED
    assert create([L.BeamDesc(**{**ok, "wl": 0.0})]) == L.LP_ERR_INVALID_ARGUMENT
    assert create([L.BeamDesc(**{**ok, "z": float("nan")})]) == L.LP_ERR_INVALID_ARGUMENT
    assert create([L.BeamDesc(**{**ok, "flags": L.LP_FLAG_ADJOINT})]) == \
        L.LP_ERR_INVALID_ARGUMENT
    assert out.value is None
    assert lib.lp_batch_run(vp(0), vp(0)) == L.LP_ERR_INVALID_ARGUMENT
    assert lib.lp_batch_status(vp(0), vp(0)) == L.LP_ERR_INVALID_ARGUMENT
