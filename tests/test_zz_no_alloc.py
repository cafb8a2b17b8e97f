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

from helpers import gpu_context
from titsolver_gb300 import _abi, physics, scenarios

pytestmark = pytest.mark.gpu


def _cloud(n_total: int, seed: int) -> dict:
    scn = scenarios.cloud_3d(n_total=n_total, seed=seed)
    return scn


def _noalloc(lib, torch, r: np.ndarray, h: float, m: float, kernel: int):
    n, dim = r.shape
    r_d = torch.from_numpy(np.ascontiguousarray(r)).cuda()
    rho_d = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    cnt_d = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    hs_d = torch.zeros((n,), dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    st = lib.tg_summation_density_noalloc(dim, kernel, n, ctypes.c_void_p(r_d.data_ptr()),
                                          h, m, ctypes.c_void_p(rho_d.data_ptr()),
                                          ctypes.c_void_p(cnt_d.data_ptr()),
                                          ctypes.c_void_p(hs_d.data_ptr()), None)
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
