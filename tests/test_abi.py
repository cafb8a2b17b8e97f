"""CPU checks of the drop-in boundary: libtitgpu.so loads, exports every
entry point include/titgpu.h declares, and the host-only calls behave (no
kernel runs here)."""

from __future__ import annotations

import ctypes
import pathlib
import re

import pytest

from titsolver_gb300 import _abi

HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "titgpu.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    names = re.findall(r"^(?:int|void|const char\*)\s+(tg_\w+)\s*\(", text, flags=re.M)
    assert len(names) >= 20
    return names


def test_library_exports_every_declared_symbol(gpu_lib):
    names = declared_functions()
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing
    # The Python binding covers exactly the declared set.
    assert sorted(n for n, _, _ in _abi.SIGNATURES) == sorted(names)


def test_struct_layouts_match_header():
    # 14 int32 fields, then 8 doubles.
    assert ctypes.sizeof(_abi.TgParams) == 14 * 4 + 8 * 8
    assert _abi.TgParams.xi.offset == 56
    assert _abi.TgParams.resort.offset == 52
    assert ctypes.sizeof(_abi.TgTank) == 2 * 8 + 4 * 8
    assert ctypes.sizeof(_abi.TgProfile) == 5 * 8 + 3 * 8


def test_params_default_are_reference_values(gpu_lib):
    p = _abi.default_params()
    assert (p.dim, p.precision, p.kernel, p.integrator) == (2, _abi.TG_FP64,
                                                           _abi.TG_KERNEL_WENDLAND_C4,
                                                           _abi.TG_SSPRK3)
    assert (p.viscosity, p.diffusion) == (_abi.TG_VISC_MORRIS, _abi.TG_DIFF_FERRARI)
    assert (p.cfl, p.c_force, p.c_visc, p.xi, p.g, p.mu) == (0.4, 0.25, 0.125, 7.0, 9.81, 0.001)
    assert (p.eos, p.face_fp32) == (_abi.TG_EOS_TAIT, 0)


def test_status_strings(gpu_lib):
    for code in range(8):
        assert gpu_lib.tg_status_string(code)
    assert gpu_lib.tg_status_string(0) == b"ok"


def test_invalid_params_rejected_before_device(gpu_lib):
    p = _abi.default_params()
    p.dim = 4
    h = ctypes.c_void_p()
    assert gpu_lib.tg_context_create(ctypes.byref(p), ctypes.byref(h)) == _abi.TG_ERR_INVALID_ARGUMENT
    p = _abi.default_params()
    p.cells_per_radius = 9
    assert gpu_lib.tg_context_create(ctypes.byref(p), ctypes.byref(h)) == _abi.TG_ERR_INVALID_ARGUMENT
    # FP32 face integrals belong to the compensated form only.
    p = _abi.default_params()
    p.face_fp32 = 1
    assert gpu_lib.tg_context_create(ctypes.byref(p), ctypes.byref(h)) == _abi.TG_ERR_INVALID_ARGUMENT
    p.precision = _abi.TG_FP32C
    p.face_fp32 = 2
    assert gpu_lib.tg_context_create(ctypes.byref(p), ctypes.byref(h)) == _abi.TG_ERR_INVALID_ARGUMENT
    assert gpu_lib.tg_context_destroy(None) == _abi.TG_OK


def test_context_without_device_fails_cleanly(gpu_lib):
    p = _abi.default_params()
    h = ctypes.c_void_p()
    st = gpu_lib.tg_context_create(ctypes.byref(p), ctypes.byref(h))
    if st == _abi.TG_OK:  # a GPU is present: creation works, clean up
        assert gpu_lib.tg_context_destroy(h) == _abi.TG_OK
        pytest.skip("a CUDA device is visible")
    assert st == _abi.TG_ERR_NO_DEVICE


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _abi.load(tmp_path / "libtitgpu.so")


def test_null_context_rejected_by_every_entry(gpu_lib):
    # Every entry point that takes a context returns TG_ERR_INVALID_ARGUMENT
    # for a null one, before touching a device.
    null = None
    d = ctypes.POINTER(ctypes.c_double)()
    bad = _abi.TG_ERR_INVALID_ARGUMENT
    assert gpu_lib.tg_particles_download_state(null, d, d, d, d, d) == bad
    assert gpu_lib.tg_particles_download(null, 0, d) == bad
    assert gpu_lib.tg_particles_update(null, d, d, d, d) == bad
    assert gpu_lib.tg_step(null, 1, d) == bad
    assert gpu_lib.tg_prepare(null) == bad
    assert gpu_lib.tg_tank_faces(null, 0, 0, ctypes.POINTER(ctypes.c_int32)(), 0, d) == bad
    assert gpu_lib.tg_time(null, d) == bad
