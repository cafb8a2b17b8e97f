"""Python binding of the oracle: a CPU restatement of TitSolver's WCSPH path.

TEST INFRASTRUCTURE ONLY.  The tests, ``__graft_entry__.smoke()`` and the
benchmark's CPU-baseline leg load it as the checker or the timed CPU
baseline; the product package never imports it.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_F = ctypes.POINTER(ctypes.c_float)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U64 = ctypes.POINTER(ctypes.c_uint64)

_lib = None


class _Params(ctypes.Structure):
    # Same layout as tg_params of include/titgpu.h.
    _fields_ = [(n, ctypes.c_int32) for n in (
        "dim", "precision", "kernel", "integrator", "viscosity", "diffusion",
        "post_integrate", "cells_per_radius", "kahan", "device", "staging",
        "eos", "face_fp32")] + [
        (n, ctypes.c_double) for n in (
            "xi", "g", "mu", "alpha", "delta", "cfl", "c_force", "c_visc")]


class _Faces(ctypes.Structure):
    _fields_ = [("n_faces", ctypes.c_int32), ("face_verts", ctypes.POINTER(ctypes.c_int32)),
                ("n_poly", ctypes.c_int32), ("poly", ctypes.POINTER(ctypes.c_double))]


class _Tank(ctypes.Structure):
    _fields_ = [("n_fluid", ctypes.c_int64), ("n_wall", ctypes.c_int64),
                ("h", ctypes.c_double), ("m", ctypes.c_double),
                ("rho0", ctypes.c_double), ("cs0", ctypes.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(str(path))
        sig = {
            "or_kernel_info": (None, [ctypes.c_int32, ctypes.c_int32, _D, _D]),
            "or_kernel_value": (ctypes.c_double, [ctypes.c_int32, ctypes.c_int32, _D, ctypes.c_double]),
            "or_kernel_grad": (None, [ctypes.c_int32, ctypes.c_int32, _D, ctypes.c_double, _D]),
            "or_kernel_unit_value": (ctypes.c_double, [ctypes.c_int32, ctypes.c_double]),
            "or_kernel_unit_deriv": (ctypes.c_double, [ctypes.c_int32, ctypes.c_double]),
            "or_tait": (None, [ctypes.c_double] * 4 + [_D, _D, _D]),
            "or_eos": (None, [ctypes.c_int32] + [ctypes.c_double] * 4 + [_D, _D, _D, _D]),
            "or_tait_density_from_potential": (ctypes.c_double, [ctypes.c_double] * 4),
            "or_splitmix64": (ctypes.c_uint64, [ctypes.c_uint64]),
            "or_grid_search": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int64, _D, ctypes.c_double,
                                                ctypes.c_double, _I64, _I32, ctypes.c_int64,
                                                ctypes.c_int32]),
            "or_grid_search_f32": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int64, _F, ctypes.c_float,
                                                    ctypes.c_float, _I64, _I32, ctypes.c_int64,
                                                    ctypes.c_int32]),
            "or_naive_search": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int64, _D, ctypes.c_double,
                                                 ctypes.c_int32, _I64, _I32, ctypes.c_int64]),
            "or_mt19937_uniform_points": (None, [ctypes.c_uint32, ctypes.c_int64, _D]),
            "or_summation_density": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                                      ctypes.c_int64, _D, ctypes.c_double,
                                                      ctypes.c_double, _D, _I32, _U64,
                                                      ctypes.c_int32]),
            "or_wcsph_step": (ctypes.c_int32, [ctypes.POINTER(_Params), ctypes.c_int32,
                                               ctypes.POINTER(_Tank), _D, _D, _D, _D, _D,
                                               ctypes.c_int32, _D, _D, ctypes.c_int32]),
            "or_wcsph_step_faces": (ctypes.c_int32, [ctypes.POINTER(_Params), ctypes.c_int32,
                                                     ctypes.POINTER(_Tank), _D, _D, _D, _D, _D,
                                                     ctypes.c_int32, _D, _D, ctypes.c_int32,
                                                     ctypes.POINTER(_Faces)]),
            "or_kernel_flux2": (None, [ctypes.c_int32, _D, _D, _D, ctypes.c_double, _D]),
            "or_kernel_antigrad_flux2": (ctypes.c_double, [ctypes.c_int32, _D, _D, _D,
                                                           ctypes.c_double]),
            "or_winding_number2": (ctypes.c_double, [ctypes.c_int32, _D, _D]),
            "or_kernel_flux3": (None, [ctypes.c_int32, _D, _D, _D, _D, ctypes.c_double, _D]),
            "or_kernel_antigrad_flux3": (ctypes.c_double, [ctypes.c_int32, _D, _D, _D, _D,
                                                           ctypes.c_double]),
            "or_winding_number3": (ctypes.c_double, [ctypes.c_int32, _D, _D]),
            "or_triangle_in_sphere": (ctypes.c_int32, [_D, _D, _D, _D, ctypes.c_double]),
            "or_triangle_clamp": (None, [_D, _D, _D, _D, _D]),
            "or_triangle_project": (None, [_D, _D, _D, _D, _D]),
            "or_tank_neighbour_counts": (ctypes.c_int32, [ctypes.POINTER(_Params), ctypes.c_int32,
                                                          ctypes.POINTER(_Tank), _D, _I32, _U64,
                                                          ctypes.c_int32]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def default_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ct))


def _params(p) -> _Params:
    out = _Params()
    for name, _ in _Params._fields_:
        setattr(out, name, getattr(p, name))
    return out


def _tanks(tanks):
    arr = (_Tank * len(tanks))()
    for i, t in enumerate(tanks):
        arr[i] = _Tank(int(t["n_fluid"]), int(t["n_wall"]), float(t["h"]), float(t["m"]),
                       float(t["rho0"]), float(t["cs0"]))
    return arr


def kernel_info(kernel: int, dim: int):
    r = ctypes.c_double()
    w = ctypes.c_double()
    lib().or_kernel_info(kernel, dim, ctypes.byref(r), ctypes.byref(w))
    return r.value, w.value


def kernel_value(kernel: int, x, h: float) -> float:
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().or_kernel_value(kernel, x.shape[0], _p(x, ctypes.c_double), h)


def kernel_grad(kernel: int, x, h: float) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros_like(x)
    lib().or_kernel_grad(kernel, x.shape[0], _p(x, ctypes.c_double), h, _p(out, ctypes.c_double))
    return out


def unit_value(kernel: int, q: float) -> float:
    return lib().or_kernel_unit_value(kernel, q)


def unit_deriv(kernel: int, q: float) -> float:
    return lib().or_kernel_unit_deriv(kernel, q)


def tait(rho, rho0, cs0, xi=7.0):
    p, c, H = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    lib().or_tait(rho, rho0, cs0, xi, ctypes.byref(p), ctypes.byref(c), ctypes.byref(H))
    return p.value, c.value, H.value


def eos(kind: int, rho, rho0, cs0, xi=7.0):
    """(p, c, H(rho), rho(H(rho))) of TG_EOS_TAIT (0) or TG_EOS_LINEAR_TAIT (1)."""
    out = [ctypes.c_double() for _ in range(4)]
    lib().or_eos(kind, rho, rho0, cs0, xi, *(ctypes.byref(o) for o in out))
    return tuple(o.value for o in out)


def density_from_potential(H, rho0, cs0, xi=7.0):
    return lib().or_tait_density_from_potential(H, rho0, cs0, xi)


def splitmix64(x: int) -> int:
    return lib().or_splitmix64(x)


def _csr(call, n):
    off = np.zeros(n + 1, dtype=np.int64)
    total = call(off, None, 0)
    idx = np.zeros(max(total, 1), dtype=np.int32)
    call(off, idx, idx.shape[0])
    return off, idx[:total]


def grid_search(r: np.ndarray, radius: float, size_hint: float, nthreads: int = 0):
    r = np.ascontiguousarray(r, dtype=np.float64)
    n, d = r.shape
    nt = nthreads or default_threads()
    return _csr(lambda off, idx, cap: lib().or_grid_search(
        d, n, _p(r, ctypes.c_double), radius, size_hint, _p(off, ctypes.c_int64),
        _p(idx, ctypes.c_int32), cap, nt), n)


def grid_search_f32(r: np.ndarray, radius: float, size_hint: float, nthreads: int = 0):
    r = np.ascontiguousarray(r, dtype=np.float32)
    n, d = r.shape
    nt = nthreads or default_threads()
    return _csr(lambda off, idx, cap: lib().or_grid_search_f32(
        d, n, _p(r, ctypes.c_float), np.float32(radius), np.float32(size_hint),
        _p(off, ctypes.c_int64), _p(idx, ctypes.c_int32), cap, nt), n)


def naive_search(r: np.ndarray, radius: float, inclusive: bool = True):
    r = np.ascontiguousarray(r, dtype=np.float64)
    n, d = r.shape
    return _csr(lambda off, idx, cap: lib().or_naive_search(
        d, n, _p(r, ctypes.c_double), radius, int(inclusive), _p(off, ctypes.c_int64),
        _p(idx, ctypes.c_int32), cap), n)


def mt19937_uniform_points(seed: int, count: int, dim: int) -> np.ndarray:
    out = np.zeros(count * dim, dtype=np.float64)
    lib().or_mt19937_uniform_points(seed, count * dim, _p(out, ctypes.c_double))
    return out.reshape(count, dim)


def summation_density(r: np.ndarray, h: float, m: float, kernel: int,
                      pos_precision: int = 0, nthreads: int = 0):
    r = np.ascontiguousarray(r, dtype=np.float64)
    n, d = r.shape
    rho = np.zeros(n)
    cnt = np.zeros(n, dtype=np.int32)
    hs = np.zeros(n, dtype=np.uint64)
    st = lib().or_summation_density(d, kernel, pos_precision, n, _p(r, ctypes.c_double), h, m,
                                    _p(rho, ctypes.c_double), _p(cnt, ctypes.c_int32),
                                    _p(hs, ctypes.c_uint64), nthreads or default_threads())
    if st != 0:
        raise RuntimeError(f"or_summation_density: status {st}")
    return rho, cnt, hs


class State:
    """Host state of a scenario for the oracle's in-place stepping."""

    def __init__(self, scn: dict):
        self.dim = scn["dim"]
        self.tanks = [dict(t) for t in scn["tanks"]]
        self.r = np.array(scn["r"], dtype=np.float64, copy=True)
        self.v = np.array(scn["v"], dtype=np.float64, copy=True)
        self.rho = np.array(scn["rho"], dtype=np.float64, copy=True)
        n = self.rho.shape[0]
        self.drho_dt = np.zeros(n)
        self.dv_dt = np.zeros((n, self.dim))
        self.time = np.zeros(len(self.tanks))
        self.dt = np.zeros(len(self.tanks))
        # Per-tank boundary faces (face-boundary scenarios): face_verts
        # (n, 2) indices into the tank's fixed particles, poly (m, 2).
        self.faces = None
        if scn.get("faces") is not None:
            self.faces = [None if fc is None else
                          (np.ascontiguousarray(fc["face_verts"], dtype=np.int32),
                           np.ascontiguousarray(fc["poly"], dtype=np.float64))
                          for fc in scn["faces"]]


def step(params, state: State, n_steps: int = 1, nthreads: int = 0) -> np.ndarray:
    P = _params(params)
    T = _tanks(state.tanks)
    args = (ctypes.byref(P), len(state.tanks), T,
            _p(state.r, ctypes.c_double), _p(state.v, ctypes.c_double),
            _p(state.rho, ctypes.c_double), _p(state.drho_dt, ctypes.c_double),
            _p(state.dv_dt, ctypes.c_double), n_steps,
            _p(state.dt, ctypes.c_double), _p(state.time, ctypes.c_double),
            nthreads or default_threads())
    if state.faces is None:
        st = lib().or_wcsph_step(*args)
    else:
        F = (_Faces * len(state.tanks))()
        for t, fc in enumerate(state.faces):
            if fc is None:
                continue
            fv, poly = fc
            F[t].n_faces = fv.shape[0]
            F[t].face_verts = _p(fv, ctypes.c_int32)
            F[t].n_poly = poly.shape[0]
            F[t].poly = _p(poly, ctypes.c_double)
        st = lib().or_wcsph_step_faces(*args, F)
    if st != 0:
        raise RuntimeError(f"or_wcsph_step: status {st}")
    return state.dt.copy()


def kernel_flux2(kernel: int, a, b, x, h: float) -> np.ndarray:
    """Kernel flux of segment a-b at x (kernel.hpp:194-206)."""
    out = np.zeros(2)
    A, B, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, x))
    lib().or_kernel_flux2(kernel, _p(A, ctypes.c_double), _p(B, ctypes.c_double),
                          _p(X, ctypes.c_double), h, _p(out, ctypes.c_double))
    return out


def kernel_antigrad_flux2(kernel: int, a, b, x, h: float) -> float:
    """Antigradient flux of segment a-b at x (kernel.hpp:209-221)."""
    A, B, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, x))
    return lib().or_kernel_antigrad_flux2(kernel, _p(A, ctypes.c_double),
                                          _p(B, ctypes.c_double), _p(X, ctypes.c_double), h)


def winding_number2(poly, x) -> float:
    P, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (poly, x))
    return lib().or_winding_number2(P.shape[0], _p(P, ctypes.c_double), _p(X, ctypes.c_double))


def kernel_flux3(kernel: int, a, b, c, x, h: float) -> np.ndarray:
    """Kernel flux of triangle a-b-c at x (kernel.hpp:194-206)."""
    out = np.zeros(3)
    A, B, C, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, c, x))
    lib().or_kernel_flux3(kernel, _p(A, ctypes.c_double), _p(B, ctypes.c_double),
                          _p(C, ctypes.c_double), _p(X, ctypes.c_double), h,
                          _p(out, ctypes.c_double))
    return out


def kernel_antigrad_flux3(kernel: int, a, b, c, x, h: float) -> float:
    """Antigradient flux of triangle a-b-c at x (kernel.hpp:209-221)."""
    A, B, C, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, c, x))
    return lib().or_kernel_antigrad_flux3(kernel, _p(A, ctypes.c_double),
                                          _p(B, ctypes.c_double), _p(C, ctypes.c_double),
                                          _p(X, ctypes.c_double), h)


def winding_number3(tris, x) -> float:
    """Generalized winding number of a triangle mesh (n, 3, 3) at x."""
    T, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (tris, x))
    return lib().or_winding_number3(T.shape[0], _p(T, ctypes.c_double), _p(X, ctypes.c_double))


def triangle_in_sphere(a, b, c, x, radius: float) -> bool:
    A, B, C, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, c, x))
    return bool(lib().or_triangle_in_sphere(_p(A, ctypes.c_double), _p(B, ctypes.c_double),
                                            _p(C, ctypes.c_double), _p(X, ctypes.c_double),
                                            radius))


def triangle_clamp(a, b, c, x) -> np.ndarray:
    out = np.zeros(3)
    A, B, C, X = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, c, x))
    lib().or_triangle_clamp(_p(A, ctypes.c_double), _p(B, ctypes.c_double),
                            _p(C, ctypes.c_double), _p(X, ctypes.c_double),
                            _p(out, ctypes.c_double))
    return out


def triangle_project(a, b, c, origin) -> np.ndarray:
    out = np.zeros(6)
    A, B, C, O = (np.ascontiguousarray(u, dtype=np.float64) for u in (a, b, c, origin))
    lib().or_triangle_project(_p(A, ctypes.c_double), _p(B, ctypes.c_double),
                              _p(C, ctypes.c_double), _p(O, ctypes.c_double),
                              _p(out, ctypes.c_double))
    return out.reshape(3, 2)


def tank_neighbour_counts(params, tanks, r: np.ndarray, nthreads: int = 0):
    r = np.ascontiguousarray(r, dtype=np.float64)
    n = r.shape[0]
    cnt = np.zeros(n, dtype=np.int32)
    hs = np.zeros(n, dtype=np.uint64)
    P = _params(params)
    st = lib().or_tank_neighbour_counts(ctypes.byref(P), len(tanks), _tanks(tanks),
                                        _p(r, ctypes.c_double), _p(cnt, ctypes.c_int32),
                                        _p(hs, ctypes.c_uint64), nthreads or default_threads())
    if st != 0:
        raise RuntimeError(f"or_tank_neighbour_counts: status {st}")
    return cnt, hs
