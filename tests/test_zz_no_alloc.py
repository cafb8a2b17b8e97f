"""The allocation-free summation density entry point.

tg_summation_density_noalloc serves callers that may not allocate device
memory (for example a host framework that owns all device memory and forbids
allocation inside its callbacks): its scratch is a fixed device array inside
the library.  This file is collected last so that a run stopping at the
first failure has already run every other test.  It checks, through the C
ABI, two calls in a row with different clouds (the scratch keeps the previous
call's contents) against the allocating entry point tg_summation_density, and
the size limit.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

import oracle
from helpers import gpu_context
from titsolver_gb300 import _abi, physics, scenarios

pytestmark = pytest.mark.gpu


def _cloud(n_total: int, seed: int) -> dict:
    scn = scenarios.cloud_3d(n_total=n_total, seed=seed)
    return scn


def _noalloc(lib, torch, r: np.ndarray, h: float, m: float, kernel: int, stream=None):
    n, dim = r.shape
    r_d = torch.from_numpy(np.ascontiguousarray(r)).cuda()
    rho_d = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    cnt_d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    hs_d = torch.zeros((n,), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
    st = lib.tg_summation_density_noalloc(dim, kernel, n, ctypes.c_void_p(r_d.data_ptr()),
                                          h, m, ctypes.c_void_p(rho_d.data_ptr()),
                                          ctypes.c_void_p(cnt_d.data_ptr()),
                                          ctypes.c_void_p(hs_d.data_ptr()), handle)
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    assert st == _abi.TG_OK, lib.tg_status_string(st)
    return rho_d.cpu().numpy(), cnt_d.cpu().numpy(), hs_d.cpu().numpy().view(np.uint64)


def test_noalloc_matches_allocating_entry_two_calls_in_a_row(gpu_lib):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    kernel = _abi.TG_KERNEL_WENDLAND_C2
    # Second cloud is smaller: the tail of the first call stays in the
    # scratch and must not leak into the second result.
    for n_total, seed in ((40_000, 31), (17_000, 32)):
        scn = _cloud(n_total, seed)
        t = scn["tanks"][0]
        with gpu_context(scn, physics.baseline_params(3, kernel=kernel)) as ctx:
            rho, cnt, hs = ctx.summation_density(_abi.TG_POS_FP64)
        nrho, ncnt, nhs = _noalloc(gpu_lib, torch, scn["r"], t["h"], t["m"], kernel)
        np.testing.assert_array_equal(ncnt, cnt)
        np.testing.assert_array_equal(nhs, hs)
        np.testing.assert_allclose(nrho, rho, rtol=1e-12)


def test_noalloc_2d_points(gpu_lib):
    torch = pytest.importorskip("torch")
    scn = scenarios.dam_break_2d(nx_per_H=20)
    t = scn["tanks"][0]
    pts = dict(scn, tanks=[dict(t, n_fluid=scn["r"].shape[0], n_wall=0)])
    with gpu_context(pts, physics.baseline_params(2)) as ctx:
        rho, cnt, hs = ctx.summation_density(_abi.TG_POS_FP64)
    nrho, ncnt, nhs = _noalloc(gpu_lib, torch, scn["r"], t["h"], t["m"],
                               _abi.TG_KERNEL_WENDLAND_C2)
    np.testing.assert_array_equal(ncnt, cnt)
    np.testing.assert_array_equal(nhs, hs)
    np.testing.assert_allclose(nrho, rho, rtol=1e-12)


def test_noalloc_rejects_sizes_above_the_limit(gpu_lib):
    n = _abi.TG_NOALLOC_MAX_POINTS + 1
    st = gpu_lib.tg_summation_density_noalloc(3, _abi.TG_KERNEL_WENDLAND_C2, n, None, 0.01,
                                              1.0, None, None, None, None)
    assert st == _abi.TG_ERR_CAPACITY


def _points(r: np.ndarray, h: float, m: float = 1.0) -> dict:
    r = np.ascontiguousarray(r, dtype=np.float64)
    return dict(dim=r.shape[1], tanks=[dict(n_fluid=r.shape[0], n_wall=0, h=h, m=m,
                                            rho0=1000.0, cs0=1.0)],
                r=r, v=np.zeros_like(r), rho=np.full(r.shape[0], 1000.0))


def test_noalloc_sparse_cloud_at_the_size_limit(gpu_lib):
    # 65,536 points over 100 support radii per axis: a grid of one cell per
    # radius would need ~10^6 cells, so the cells double until it fits.
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(77))
    h = 0.5
    r = rng.uniform(0.0, 100.0 * 2.0 * h, size=(_abi.TG_NOALLOC_MAX_POINTS, 3))
    kernel = _abi.TG_KERNEL_WENDLAND_C2
    with gpu_context(_points(r, h), physics.baseline_params(3, kernel=kernel)) as ctx:
        rho, cnt, hs = ctx.summation_density(_abi.TG_POS_FP64)
    nrho, ncnt, nhs = _noalloc(gpu_lib, torch, r, h, 1.0, kernel)
    orho, ocnt, ohs = oracle.summation_density(r, h, 1.0, kernel)
    assert ncnt.max() > 1
    np.testing.assert_array_equal(ncnt, cnt)
    np.testing.assert_array_equal(nhs, hs)
    np.testing.assert_array_equal(ncnt, ocnt)
    np.testing.assert_array_equal(nhs, ohs)
    np.testing.assert_allclose(nrho, rho, rtol=1e-12)
    np.testing.assert_allclose(nrho, orho, rtol=1e-12)


def test_noalloc_single_cell_fallback(gpu_lib):
    # Two points at -+8.9e307 beside a small cluster: the grid's extent plus
    # its margins overflows at every cell size, so one cell holds every
    # point and each pair is tested.  The far points are their own only
    # neighbours; the cluster's sums equal the oracle's on the cluster alone.
    torch = pytest.importorskip("torch")
    cl = scenarios.cloud_3d(n_total=2_000, seed=5)
    h = cl["tanks"][0]["h"]
    far = np.array([[-8.9e307, 0.0, 0.0], [8.9e307, 0.0, 0.0]])
    r = np.concatenate([cl["r"], far])
    kernel = _abi.TG_KERNEL_WENDLAND_C2
    nrho, ncnt, nhs = _noalloc(gpu_lib, torch, r, h, 1.0, kernel)
    orho, ocnt, ohs = oracle.summation_density(cl["r"], h, 1.0, kernel)
    nc = cl["r"].shape[0]
    np.testing.assert_array_equal(ncnt[:nc], ocnt)
    np.testing.assert_array_equal(nhs[:nc], ohs)
    np.testing.assert_allclose(nrho[:nc], orho, rtol=1e-12)
    lone, _, _ = oracle.summation_density(np.zeros((1, 3)), h, 1.0, kernel)
    np.testing.assert_array_equal(ncnt[nc:], [1, 1])
    np.testing.assert_array_equal(nhs[nc:], [oracle.splitmix64(nc + 1),
                                             oracle.splitmix64(nc + 2)])
    np.testing.assert_allclose(nrho[nc:], lone[0], rtol=1e-15)


def test_noalloc_cubic_spline_2d_on_a_side_stream(gpu_lib):
    torch = pytest.importorskip("torch")
    scn = scenarios.dam_break_2d(nx_per_H=40)
    t = scn["tanks"][0]
    kernel = _abi.TG_KERNEL_CUBIC_SPLINE
    pts = _points(scn["r"], t["h"], t["m"])
    with gpu_context(pts, physics.baseline_params(2, kernel=kernel)) as ctx:
        rho, cnt, hs = ctx.summation_density(_abi.TG_POS_FP64)
    side = torch.cuda.Stream()
    for _ in range(2):
        nrho, ncnt, nhs = _noalloc(gpu_lib, torch, scn["r"], t["h"], t["m"], kernel, side)
        np.testing.assert_array_equal(ncnt, cnt)
        np.testing.assert_array_equal(nhs, hs)
        np.testing.assert_allclose(nrho, rho, rtol=1e-12)
