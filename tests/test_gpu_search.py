"""GPU neighbour search and summation density against the oracle, through
the C ABI.  Neighbour sets must match bit-exact (counts, order-independent
hashes, and full sorted lists on the small cases)."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from helpers import gpu_context
from titsolver_gb300 import _abi, physics, scenarios

pytestmark = pytest.mark.gpu


def _points_scenario(r: np.ndarray, h: float, m: float = 1.0) -> dict:
    r = np.ascontiguousarray(r, dtype=np.float64)
    return dict(dim=r.shape[1], tanks=[dict(n_fluid=r.shape[0], n_wall=0, h=h, m=m,
                                            rho0=1000.0, cs0=1.0)],
                r=r, v=np.zeros_like(r), rho=np.full(r.shape[0], 1000.0))


def _rows(off, idx):
    return [list(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


@pytest.mark.parametrize("nx", (10, 80))
def test_neighbour_sets_bitexact_dam_break_2d(gpu_lib, nx):
    # t = 0 lattice: exact-distance ties at 2h decided by the rounded predicate.
    scn = scenarios.dam_break_2d(nx_per_H=nx)
    P = physics.baseline_params(2)
    with gpu_context(scn, P) as ctx:
        cnt, hs = ctx.neighbour_counts()
        ocnt, ohs = oracle.tank_neighbour_counts(P, scn["tanks"], scn["r"])
        np.testing.assert_array_equal(cnt, ocnt)
        np.testing.assert_array_equal(hs, ohs)
        if nx == 10:
            off, idx = ctx.neighbour_lists()
            t = scn["tanks"][0]
            ooff, oidx = oracle.grid_search(scn["r"], 2 * t["h"], t["h"])
            assert _rows(off, idx) == _rows(ooff, oidx)


@pytest.mark.parametrize("dim", (2, 3))
def test_neighbour_sets_mt19937_match_naive(gpu_lib, dim):
    # The reference search test inputs: radii {0.01, 0.1, 0.5, 1.0} become
    # support radii 2h of the Wendland kernel.
    pts = oracle.mt19937_uniform_points(123, 200, dim)
    for radius in (0.01, 0.1, 0.5, 1.0):
        scn = _points_scenario(pts, radius / 2)
        with gpu_context(scn, physics.baseline_params(dim)) as ctx:
            off, idx = ctx.neighbour_lists()
        naive = _rows(*oracle.naive_search(pts, radius, inclusive=False))
        assert _rows(off, idx) == naive, radius


@pytest.mark.parametrize("cells_per_radius", (1, 2, 3))
def test_neighbour_sets_cloud_3d_fp64(gpu_lib, cells_per_radius):
    scn = scenarios.cloud_3d(n_total=30_000, seed=9)
    P = physics.baseline_params(3)
    P.cells_per_radius = cells_per_radius
    with gpu_context(scn, P) as ctx:
        cnt, hs = ctx.neighbour_counts()
    ocnt, ohs = oracle.tank_neighbour_counts(P, scn["tanks"], scn["r"])
    np.testing.assert_array_equal(cnt, ocnt)
    np.testing.assert_array_equal(hs, ohs)


def _fp32c_sets_match(scn, P32, steps=0):
    """Counts, hashes and (small cases) full lists of the compensated form's
    neighbour sets against the oracle's FP64 grid search, on the context's
    positions after `steps` steps."""
    with gpu_context(scn, P32) as ctx:
        if steps:
            ctx.step(steps)
        r = ctx.download(_abi.TG_FIELD_R)
        cnt, hs = ctx.neighbour_counts()
        lists = ctx.neighbour_lists() if r.shape[0] <= 20_000 else None
    ocnt, ohs = oracle.tank_neighbour_counts(P32, scn["tanks"], r)
    np.testing.assert_array_equal(cnt, ocnt)
    np.testing.assert_array_equal(hs, ohs)
    if lists is not None and len(scn["tanks"]) == 1:
        t = scn["tanks"][0]
        unit = 2.0  # support radius / h of the Wendland kernels used here
        ooff, oidx = oracle.grid_search(r, unit * t["h"], t["h"])
        assert _rows(*lists) == _rows(ooff, oidx)


@pytest.mark.parametrize("nx", (10, 80))
@pytest.mark.parametrize("steps", (0, 30))
def test_neighbour_sets_fp32c_dam_break_2d(gpu_lib, nx, steps):
    # At the lattice start, axis neighbours at exactly 2h fall in the band
    # around the support radius and are decided by the FP64 predicate.
    scn = scenarios.dam_break_2d(nx_per_H=nx)
    _fp32c_sets_match(scn, physics.baseline_params(2, precision=_abi.TG_FP32C), steps)


@pytest.mark.parametrize("steps", (0, 20))
def test_neighbour_sets_fp32c_dam_break_3d(gpu_lib, steps):
    scn = scenarios.dam_break_3d(nx_per_H=10)
    _fp32c_sets_match(scn, physics.baseline_params(3, precision=_abi.TG_FP32C), steps)


@pytest.mark.parametrize("cells_per_radius", (1, 2, 3))
def test_neighbour_sets_fp32c_cloud_3d(gpu_lib, cells_per_radius):
    scn = scenarios.cloud_3d(n_total=30_000, seed=9)
    P = physics.baseline_params(3, precision=_abi.TG_FP32C)
    P.cells_per_radius = cells_per_radius
    _fp32c_sets_match(scn, P)


@pytest.mark.parametrize("dim", (2, 3))
def test_neighbour_sets_fp32c_mt19937_match_naive(gpu_lib, dim):
    pts = oracle.mt19937_uniform_points(123, 200, dim)
    for radius in (0.01, 0.1, 0.5, 1.0):
        scn = _points_scenario(pts, radius / 2)
        with gpu_context(scn, physics.baseline_params(dim, precision=_abi.TG_FP32C)) as ctx:
            off, idx = ctx.neighbour_lists()
        naive = _rows(*oracle.naive_search(pts, radius, inclusive=False))
        assert _rows(off, idx) == naive, radius


def test_neighbour_sets_fp32c_batched_tanks(gpu_lib):
    scn = scenarios.batched_tanks(n_tanks=6, n_range=(8, 16), seed=4)
    _fp32c_sets_match(scn, physics.baseline_params(2, precision=_abi.TG_FP32C), 10)


def test_summation_density_golden_fp64_and_fp32(gpu_lib):
    import pathlib
    z = np.load(pathlib.Path(__file__).resolve().parent / "golden" / "cloud_small.npz")
    scn = _points_scenario(z["r"], float(z["h"]), float(z["m"]))
    with gpu_context(scn, physics.baseline_params(3)) as ctx:
        for prec in (0, 1):
            rho, cnt, hs = ctx.summation_density(prec)
            np.testing.assert_array_equal(cnt, z[f"count_{prec}"])
            np.testing.assert_array_equal(hs, z[f"hash_{prec}"])
            # FP64: summation order only; FP32: compensated FP32 vs plain FP32.
            np.testing.assert_allclose(rho, z[f"rho_{prec}"], rtol=1e-12 if prec == 0 else 2e-6)


def test_summation_density_cloud_vs_oracle(gpu_lib):
    scn = scenarios.cloud_3d(n_total=200_000, seed=21)
    t = scn["tanks"][0]
    with gpu_context(scn, physics.baseline_params(3)) as ctx:
        for prec in (0, 1):
            rho, cnt, hs = ctx.summation_density(prec)
            orho, ocnt, ohs = oracle.summation_density(scn["r"], t["h"], t["m"], 3, prec)
            np.testing.assert_array_equal(cnt, ocnt)
            np.testing.assert_array_equal(hs, ohs)
            # FP32: the oracle sums plainly in ascending order (error grows
            # with the ~900 terms of cluster cores), the GPU compensates.
            np.testing.assert_allclose(rho, orho, rtol=1e-12 if prec == 0 else 1e-5)


def test_batched_tank_neighbours_are_tank_local(gpu_lib):
    scn = scenarios.batched_tanks(n_tanks=6, n_range=(8, 16), seed=4)
    P = physics.baseline_params(2)
    with gpu_context(scn, P) as ctx:
        cnt, hs = ctx.neighbour_counts()
    ocnt, ohs = oracle.tank_neighbour_counts(P, scn["tanks"], scn["r"])
    np.testing.assert_array_equal(cnt, ocnt)
    np.testing.assert_array_equal(hs, ohs)


def test_neighbour_counts_empty_tank_list_rejected(gpu_lib):
    with _abi.Context(physics.baseline_params(2)) as ctx:
        with pytest.raises(_abi.TgError):
            ctx.upload([], np.zeros((0, 2)), np.zeros((0, 2)), np.zeros(0))
