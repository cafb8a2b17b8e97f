"""Launch shapes of the force pass and the autotuner, through the C ABI.

Every shape computes the same sums in a different order, so each one is held
to the oracle at the tolerances of the plain steps (FP64: 1e-12 relative L2
after one step) or of the compensated form (FP32C vs FP64 oracle: rho 1e-5,
r 1e-6 after 30 steps).  Changing the cell size or autotuning keeps the
particle state and clocks bit for bit (wall densities, which are derived
from the fluid, to rounding).
"""

from __future__ import annotations

import numpy as np
import pytest

from helpers import fluid_mask, gpu_context, gpu_state, oracle_run, rel_l2
from titsolver_gb300 import _abi, physics, scenarios

pytestmark = pytest.mark.gpu

SHAPES = [(k, block, lanes) for k in (1, 2, 3) for lanes in (1, 2, 4)
          for block in (64, 256)]


@pytest.mark.parametrize("term_set", ("baseline", "reference"))
def test_fp64_shapes_vs_oracle(gpu_lib, term_set):
    scn = scenarios.dam_break_2d(nx_per_H=20)
    P = getattr(physics, f"{term_set}_params")(2)
    o = oracle_run(scn, P, 2)
    f = fluid_mask(scn)
    for k, block, lanes in SHAPES:
        with gpu_context(scn, P) as ctx:
            ctx.set_tuning(k, block, lanes)
            ctx.step(2)
            g = gpu_state(ctx)
        assert rel_l2(g["r"][f], o.r[f]) <= 1e-12, (k, block, lanes)
        assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-12, (k, block, lanes)
        assert rel_l2(g["dv_dt"][f], o.dv_dt[f]) <= 1e-9, (k, block, lanes)


def test_fp64_shapes_3d(gpu_lib):
    scn = scenarios.dam_break_3d(nx_per_H=8)
    P = physics.baseline_params(3)
    o = oracle_run(scn, P, 1)
    f = fluid_mask(scn)
    for k, block, lanes in ((1, 128, 4), (2, 256, 2), (3, 64, 1)):
        with gpu_context(scn, P) as ctx:
            ctx.set_tuning(k, block, lanes)
            ctx.step(1)
            g = gpu_state(ctx)
        assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-12, (k, block, lanes)
        assert rel_l2(g["dv_dt"][f], o.dv_dt[f]) <= 1e-9, (k, block, lanes)


@pytest.mark.parametrize("dim", (2, 3))
def test_fp32c_shapes_vs_fp64_oracle(gpu_lib, dim):
    if dim == 2:
        scn = scenarios.dam_break_2d(nx_per_H=40)
    else:
        scn = scenarios.dam_break_3d(nx_per_H=10)
    P64 = physics.baseline_params(dim)
    o = oracle_run(scn, P64, 30)
    f = fluid_mask(scn)
    for k, block, lanes in ((1, 128, 1), (2, 128, 2), (2, 256, 4), (3, 64, 2)):
        P32 = physics.baseline_params(dim, precision=_abi.TG_FP32C)
        with gpu_context(scn, P32) as ctx:
            ctx.set_tuning(k, block, lanes)
            ctx.step(30)
            g = gpu_state(ctx)
        assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-5, (dim, k, block, lanes)
        assert rel_l2(g["r"][f], o.r[f]) <= 1e-6, (dim, k, block, lanes)


def test_team_variants_need_wendland(gpu_lib):
    scn = scenarios.dam_break_2d(nx_per_H=10)
    P = physics.reference_params(2, kernel=_abi.TG_KERNEL_CUBIC_SPLINE)
    with gpu_context(scn, P) as ctx:
        with pytest.raises(_abi.TgError) as ei:
            ctx.set_tuning(2, 128, 2)
        assert ei.value.status == _abi.TG_ERR_INVALID_ARGUMENT
        with pytest.raises(_abi.TgError):
            ctx.set_tuning(2, 96, 1)
        ctx.set_tuning(3, 256, 1)
        assert ctx.get_tuning()["cells_per_radius"] == 3


def _same_state(after, before, f, precision):
    # The state proper (positions, velocities, fluid densities, forces,
    # clocks) comes back bit for bit.  Wall densities are re-extrapolated
    # from the fluid on download and their sums follow the new grid's cell
    # order, so they agree to rounding only.
    for key in ("r", "v", "dv_dt", "time"):
        np.testing.assert_array_equal(after[key], before[key], err_msg=key)
    np.testing.assert_array_equal(after["rho"][f], before["rho"][f])
    rtol = 1e-13 if precision == _abi.TG_FP64 else 1e-8
    np.testing.assert_allclose(after["rho"][~f], before["rho"][~f], rtol=rtol)


@pytest.mark.parametrize("precision", (_abi.TG_FP64, _abi.TG_FP32C))
def test_regrid_keeps_state(gpu_lib, precision):
    scn = scenarios.dam_break_2d(nx_per_H=20)
    P = physics.baseline_params(2, precision=precision)
    f = fluid_mask(scn)
    with gpu_context(scn, P) as ctx:
        ctx.step(5)
        before = gpu_state(ctx)
        ctx.set_tuning(1, 128, 1)
        after = gpu_state(ctx)
        _same_state(after, before, f, precision)
        ctx.step(5)
        assert np.all(np.isfinite(ctx.download(_abi.TG_FIELD_RHO)))


@pytest.mark.parametrize("precision", (_abi.TG_FP64, _abi.TG_FP32C))
def test_autotune_keeps_state_and_picks_a_shape(gpu_lib, precision):
    scn = scenarios.dam_break_2d(nx_per_H=40)
    P = physics.baseline_params(2, precision=precision)
    f = fluid_mask(scn)
    with gpu_context(scn, P) as ctx, gpu_context(scn, P) as ref:
        ctx.step(3)
        ref.step(3)
        before = gpu_state(ctx)
        t = ctx.autotune(2)
        assert t["candidates"] >= 5
        assert t["ms_per_step"] > 0.0
        assert ctx.get_tuning()["cells_per_radius"] == t["cells_per_radius"]
        after = gpu_state(ctx)
        _same_state(after, before, f, precision)
        ctx.step(10)
        ref.step(10)
        a, b = gpu_state(ctx), gpu_state(ref)
    tol = 1e-11 if precision == _abi.TG_FP64 else 1e-5
    assert rel_l2(a["rho"][f], b["rho"][f]) <= tol
    assert rel_l2(a["r"][f], b["r"][f]) <= tol
    np.testing.assert_allclose(a["time"], b["time"], rtol=1e-9)
