"""ctypes binding of the C ABI in ``include/titgpu.h``.

This is the only way Python reaches the GPU path: every call goes through
``libtitgpu.so``.  If the library is missing, importing the GPU API raises;
there is no CPU fallback.
"""

from __future__ import annotations

import ctypes
import pathlib

import numpy as np

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libtitgpu.so"

# Status codes.
TG_OK = 0
TG_ERR_INVALID_ARGUMENT = 1
TG_ERR_CUDA = 2
TG_ERR_OUT_OF_MEMORY = 3
TG_ERR_NOT_READY = 4
TG_ERR_DEVICE_STATE = 5
TG_ERR_CAPACITY = 6
TG_ERR_NO_DEVICE = 7

TG_NOALLOC_MAX_POINTS = 65536

TG_DEV_NONFINITE_STATE = 1
TG_DEV_OUTSIDE_GRID = 2
TG_DEV_BAD_DT = 4

TG_FP64, TG_FP32C = 0, 1
TG_POS_FP64, TG_POS_FP32 = 0, 1
(TG_KERNEL_CUBIC_SPLINE, TG_KERNEL_QUARTIC_SPLINE, TG_KERNEL_QUINTIC_SPLINE,
 TG_KERNEL_WENDLAND_C2, TG_KERNEL_WENDLAND_C4, TG_KERNEL_WENDLAND_C6) = range(6)
TG_SSPRK3, TG_SSPRK2, TG_EULER, TG_VERLET = range(4)
TG_VISC_MORRIS, TG_VISC_MONAGHAN = 0, 1
TG_DIFF_FERRARI, TG_DIFF_MOLTENI, TG_DIFF_NONE = 0, 1, 2
TG_POST_PREPARE, TG_POST_SHIFTING = 0, 1
TG_EOS_TAIT, TG_EOS_LINEAR_TAIT = 0, 1
(TG_FIELD_R, TG_FIELD_V, TG_FIELD_RHO, TG_FIELD_DRHO_DT, TG_FIELD_DV_DT,
 TG_FIELD_P, TG_FIELD_CS) = range(7)

VECTOR_FIELDS = {TG_FIELD_R, TG_FIELD_V, TG_FIELD_DV_DT}


class TgParams(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("viscosity", ctypes.c_int32),
        ("diffusion", ctypes.c_int32),
        ("post_integrate", ctypes.c_int32),
        ("cells_per_radius", ctypes.c_int32),
        ("kahan", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("staging", ctypes.c_int32),
        ("eos", ctypes.c_int32),
        ("face_fp32", ctypes.c_int32),
        ("resort", ctypes.c_int32),
        ("xi", ctypes.c_double),
        ("g", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("delta", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("c_force", ctypes.c_double),
        ("c_visc", ctypes.c_double),
    ]


class TgTank(ctypes.Structure):
    _fields_ = [
        ("n_fluid", ctypes.c_int64),
        ("n_wall", ctypes.c_int64),
        ("h", ctypes.c_double),
        ("m", ctypes.c_double),
        ("rho0", ctypes.c_double),
        ("cs0", ctypes.c_double),
    ]


class TgProfile(ctypes.Structure):
    _fields_ = [
        ("sort_ms", ctypes.c_double),
        ("reorder_ms", ctypes.c_double),
        ("walls_ms", ctypes.c_double),
        ("forces_ms", ctypes.c_double),
        ("post_ms", ctypes.c_double),
        ("forces_launches", ctypes.c_int64),
        ("stages", ctypes.c_int64),
        ("steps", ctypes.c_int64),
    ]


class TgTuning(ctypes.Structure):
    _fields_ = [
        ("cells_per_radius", ctypes.c_int32),
        ("block_size", ctypes.c_int32),
        ("lanes_per_particle", ctypes.c_int32),
        ("candidates", ctypes.c_int32),
        ("ms_per_step", ctypes.c_double),
    ]


# (name, restype, argtypes) of every exported entry point.
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I32 = ctypes.POINTER(ctypes.c_int32)
_I64 = ctypes.POINTER(ctypes.c_int64)
_U32 = ctypes.POINTER(ctypes.c_uint32)
_U64 = ctypes.POINTER(ctypes.c_uint64)
SIGNATURES = [
    ("tg_params_default", None, [ctypes.POINTER(TgParams)]),
    ("tg_context_create", ctypes.c_int, [ctypes.POINTER(TgParams), ctypes.POINTER(_P)]),
    ("tg_context_destroy", ctypes.c_int, [_P]),
    ("tg_particles_upload", ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(TgTank), _D, _D, _D]),
    ("tg_particles_update", ctypes.c_int, [_P, _D, _D, _D, _D]),
    ("tg_prepare", ctypes.c_int, [_P]),
    ("tg_step", ctypes.c_int, [_P, ctypes.c_int32, _D]),
    ("tg_time", ctypes.c_int, [_P, _D]),
    ("tg_particles_download", ctypes.c_int, [_P, ctypes.c_int32, _D]),
    ("tg_particles_download_state", ctypes.c_int, [_P, _D, _D, _D, _D, _D]),
    ("tg_neighbour_counts", ctypes.c_int, [_P, _I32, _U64]),
    ("tg_neighbour_lists", ctypes.c_int, [_P, _I64, _I32, ctypes.c_int64]),
    ("tg_summation_density", ctypes.c_int, [_P, ctypes.c_int32, _D, _I32, _U64]),
    ("tg_summation_density_resident", ctypes.c_int, [_P, ctypes.c_int32]),
    ("tg_device_status", ctypes.c_int, [_P, _U32]),
    ("tg_profile_enable", ctypes.c_int, [_P, ctypes.c_int32]),
    ("tg_profile_read", ctypes.c_int, [_P, ctypes.POINTER(TgProfile)]),
    ("tg_set_graph", ctypes.c_int, [_P, ctypes.c_int32]),
    ("tg_launch_count", ctypes.c_int, [_P, _I64]),
    ("tg_synchronize", ctypes.c_int, [_P]),
    ("tg_timer_start", ctypes.c_int, [_P]),
    ("tg_timer_stop", ctypes.c_int, [_P, _D]),
    ("tg_host_alloc", ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(_P)]),
    ("tg_host_free", ctypes.c_int, [_P]),
    ("tg_summation_density_noalloc", ctypes.c_int,
     [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64, _P, ctypes.c_double, ctypes.c_double,
      _P, _P, _P, _P]),
    ("tg_tank_faces", ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, _I32,
                                     ctypes.c_int32, _D]),
    ("tg_get_tuning", ctypes.c_int, [_P, ctypes.POINTER(TgTuning)]),
    ("tg_set_tuning", ctypes.c_int, [_P, ctypes.POINTER(TgTuning)]),
    ("tg_autotune", ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(TgTuning)]),
    ("tg_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("tg_last_error", ctypes.c_char_p, [_P]),
]

_lib: ctypes.CDLL | None = None


def load(path: pathlib.Path | str | None = None) -> ctypes.CDLL:
    """Load libtitgpu.so (built by ``titsolver_gb300.build``); raise if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -m titsolver_gb300.build` "
            "(the GPU path has no CPU fallback)")
    lib = ctypes.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class TgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def default_params() -> TgParams:
    p = TgParams()
    load().tg_params_default(ctypes.byref(p))
    return p


class PinnedArray:
    """numpy view of page-locked host memory from tg_host_alloc."""

    def __init__(self, shape, dtype=np.float64):
        lib = load()
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        ptr = ctypes.c_void_p()
        st = lib.tg_host_alloc(max(self.nbytes, 16), ctypes.byref(ptr))
        if st != TG_OK:
            raise TgError(st, "tg_host_alloc failed")
        self._ptr = ptr
        buf = (ctypes.c_char * max(self.nbytes, 16)).from_address(ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        if getattr(self, "_ptr", None) is not None and _lib is not None:
            _lib.tg_host_free(self._ptr)
            self._ptr = None


class Context:
    """A tg_context: one device, one stream, one set of tanks."""

    def __init__(self, params: TgParams):
        self.lib = load()
        self.params = params
        h = ctypes.c_void_p()
        st = self.lib.tg_context_create(ctypes.byref(params), ctypes.byref(h))
        if st != TG_OK:
            raise TgError(st, f"tg_context_create: {self.lib.tg_status_string(st).decode()}")
        self.handle = h
        self.dim = params.dim
        self.n = 0
        self.n_tanks = 0

    def close(self):
        if getattr(self, "handle", None) is not None:
            self.lib.tg_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st: int, what: str):
        if st != TG_OK:
            err = self.lib.tg_last_error(self.handle)
            msg = err.decode() if err else ""
            raise TgError(st, f"{what}: {self.lib.tg_status_string(st).decode()}: {msg}")

    def upload(self, tanks, r: np.ndarray, v: np.ndarray, rho: np.ndarray):
        arr = (TgTank * len(tanks))()
        for i, t in enumerate(tanks):
            arr[i] = TgTank(int(t["n_fluid"]), int(t["n_wall"]), float(t["h"]),
                            float(t["m"]), float(t["rho0"]), float(t["cs0"]))
        r = np.ascontiguousarray(r, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        self._check(self.lib.tg_particles_upload(self.handle, len(tanks), arr,
                                                 _ptr(r, ctypes.c_double),
                                                 _ptr(v, ctypes.c_double),
                                                 _ptr(rho, ctypes.c_double)),
                    "tg_particles_upload")
        self.n = rho.shape[0]
        self.n_tanks = len(tanks)

    def update(self, r, v, rho, dv_dt=None):
        self._check(self.lib.tg_particles_update(self.handle, _ptr(r, ctypes.c_double),
                                                 _ptr(v, ctypes.c_double),
                                                 _ptr(rho, ctypes.c_double),
                                                 _ptr(dv_dt, ctypes.c_double)),
                    "tg_particles_update")

    def prepare(self):
        self._check(self.lib.tg_prepare(self.handle), "tg_prepare")

    def step(self, n_steps: int = 1) -> np.ndarray:
        dt = np.zeros(max(self.n_tanks, 1), dtype=np.float64)
        self._check(self.lib.tg_step(self.handle, int(n_steps), _ptr(dt, ctypes.c_double)),
                    "tg_step")
        return dt

    def time(self) -> np.ndarray:
        t = np.zeros(max(self.n_tanks, 1), dtype=np.float64)
        self._check(self.lib.tg_time(self.handle, _ptr(t, ctypes.c_double)), "tg_time")
        return t

    def download(self, field: int, out: np.ndarray | None = None) -> np.ndarray:
        comps = self.dim if field in VECTOR_FIELDS else 1
        shape = (self.n, comps) if comps > 1 else (self.n,)
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        self._check(self.lib.tg_particles_download(self.handle, field,
                                                   _ptr(out, ctypes.c_double)),
                    "tg_particles_download")
        return out

    def download_state(self, r=None, v=None, rho=None, drho_dt=None, dv_dt=None):
        """tg_particles_download_state into the given arrays (None: skipped)."""
        for a in (r, v, rho, drho_dt, dv_dt):
            assert a is None or (a.dtype == np.float64 and a.flags.c_contiguous)
        self._check(self.lib.tg_particles_download_state(
            self.handle, _ptr(r, ctypes.c_double), _ptr(v, ctypes.c_double),
            _ptr(rho, ctypes.c_double), _ptr(drho_dt, ctypes.c_double),
            _ptr(dv_dt, ctypes.c_double)), "tg_particles_download_state")

    def neighbour_counts(self):
        c = np.zeros(self.n, dtype=np.int32)
        h = np.zeros(self.n, dtype=np.uint64)
        self._check(self.lib.tg_neighbour_counts(self.handle, _ptr(c, ctypes.c_int32),
                                                 _ptr(h, ctypes.c_uint64)),
                    "tg_neighbour_counts")
        return c, h

    def neighbour_lists(self):
        off = np.zeros(self.n + 1, dtype=np.int64)
        st = self.lib.tg_neighbour_lists(self.handle, _ptr(off, ctypes.c_int64), None, 0)
        if st not in (TG_OK, TG_ERR_CAPACITY):
            self._check(st, "tg_neighbour_lists")
        idx = np.zeros(max(int(off[-1]), 1), dtype=np.int32)
        self._check(self.lib.tg_neighbour_lists(self.handle, _ptr(off, ctypes.c_int64),
                                                _ptr(idx, ctypes.c_int32), idx.shape[0]),
                    "tg_neighbour_lists")
        return off, idx[: off[-1]]

    def summation_density(self, pos_precision: int = TG_POS_FP64):
        rho = np.zeros(self.n, dtype=np.float64)
        c = np.zeros(self.n, dtype=np.int32)
        h = np.zeros(self.n, dtype=np.uint64)
        self._check(self.lib.tg_summation_density(self.handle, pos_precision,
                                                  _ptr(rho, ctypes.c_double),
                                                  _ptr(c, ctypes.c_int32),
                                                  _ptr(h, ctypes.c_uint64)),
                    "tg_summation_density")
        return rho, c, h

    def summation_density_resident(self, pos_precision: int = TG_POS_FP64):
        self._check(self.lib.tg_summation_density_resident(self.handle, pos_precision),
                    "tg_summation_density_resident")

    def device_status(self) -> int:
        f = ctypes.c_uint32()
        self._check(self.lib.tg_device_status(self.handle, ctypes.byref(f)), "tg_device_status")
        return f.value

    def profile_enable(self, on: bool = True):
        self._check(self.lib.tg_profile_enable(self.handle, int(on)), "tg_profile_enable")

    def profile_read(self) -> dict:
        p = TgProfile()
        self._check(self.lib.tg_profile_read(self.handle, ctypes.byref(p)), "tg_profile_read")
        return {k: getattr(p, k) for k, _ in TgProfile._fields_}

    def set_graph(self, on: bool):
        self._check(self.lib.tg_set_graph(self.handle, int(on)), "tg_set_graph")

    def launch_count(self) -> int:
        c = ctypes.c_int64()
        self._check(self.lib.tg_launch_count(self.handle, ctypes.byref(c)), "tg_launch_count")
        return c.value

    def synchronize(self):
        self._check(self.lib.tg_synchronize(self.handle), "tg_synchronize")

    def timer_start(self):
        self._check(self.lib.tg_timer_start(self.handle), "tg_timer_start")

    def timer_stop(self) -> float:
        ms = ctypes.c_double()
        self._check(self.lib.tg_timer_stop(self.handle, ctypes.byref(ms)), "tg_timer_stop")
        return ms.value

    def get_tuning(self) -> dict:
        t = TgTuning()
        self._check(self.lib.tg_get_tuning(self.handle, ctypes.byref(t)), "tg_get_tuning")
        return {k: getattr(t, k) for k, _ in TgTuning._fields_}

    def set_tuning(self, cells_per_radius: int, block_size: int = 128,
                   lanes_per_particle: int = 1):
        t = TgTuning(cells_per_radius, block_size, lanes_per_particle, 0, 0.0)
        self._check(self.lib.tg_set_tuning(self.handle, ctypes.byref(t)), "tg_set_tuning")

    def autotune(self, trial_steps: int = 3) -> dict:
        """Time candidate launch shapes and keep the fastest (state kept)."""
        t = TgTuning()
        self._check(self.lib.tg_autotune(self.handle, int(trial_steps), ctypes.byref(t)),
                    "tg_autotune")
        return {k: getattr(t, k) for k, _ in TgTuning._fields_}

    def set_faces(self, tank: int, face_verts, poly):
        """Boundary faces of a tank: dim vertex indices per face into the
        tank's fixed particles, and the containment surface (2D: a closed
        polygon, (n, 2); 3D: outward-oriented triangles, (n, 3, 3))."""
        d = self.params.dim
        fv = np.ascontiguousarray(face_verts, dtype=np.int32).reshape(-1, d)
        pl = np.ascontiguousarray(poly, dtype=np.float64).reshape(-1, 2 if d == 2 else 9)
        self._check(self.lib.tg_tank_faces(self.handle, int(tank), fv.shape[0],
                                           _ptr(fv, ctypes.c_int32), pl.shape[0],
                                           _ptr(pl, ctypes.c_double)), "tg_tank_faces")
