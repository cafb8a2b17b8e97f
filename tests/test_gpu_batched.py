"""The 512-tank batched workload (512 independent 2D dam breaks of 0.4k-29k
fluid particles, one launch per stage for all tanks) against the oracle.

* plain FP64, 2 steps, every tank: per-tank dt within 1e-12, r, v, rho
  within the one-step tolerances (summation order only);
* FP32-compensated, 30 steps on the full batch, each of 32 tanks spread
  over the batch checked against the oracle run of that tank alone (the
  tanks are independent: each has its own grid, dt and time) at the
  compensated tolerances (rho 1e-5, r 1e-6 relative L2)."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import fluid_mask, gpu_context, gpu_state, oracle_run, rel_l2
from titsolver_gb300 import _abi, physics, scenarios

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    return scenarios.batched_tanks(512)


def _subset(scn: dict, tanks: list[int]) -> tuple[dict, np.ndarray]:
    """The scenario of the given tanks alone, and the rows of the full
    batch's arrays that hold them."""
    starts = np.cumsum([0] + [t["n_fluid"] + t["n_wall"] for t in scn["tanks"]])
    rows = np.concatenate([np.arange(starts[t], starts[t + 1]) for t in tanks])
    sub = dict(dim=scn["dim"], tanks=[scn["tanks"][t] for t in tanks],
               r=scn["r"][rows], v=scn["v"][rows], rho=scn["rho"][rows])
    return sub, rows


def test_batched_512_tanks_fp64_two_steps(gpu_lib, batch):
    P = physics.baseline_params(2)
    with gpu_context(batch, P) as ctx:
        dt = ctx.step(2)
        g = gpu_state(ctx)
    o = oracle_run(batch, P, 2)
    f = fluid_mask(batch)
    np.testing.assert_allclose(dt, o.dt, rtol=1e-12)
    np.testing.assert_allclose(g["time"], o.time, rtol=1e-12)
    assert rel_l2(g["r"][f], o.r[f]) <= 1e-12
    assert rel_l2(g["v"][f], o.v[f]) <= 1e-9
    assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-12
    assert rel_l2(g["rho"][~f], o.rho[~f]) <= 1e-12


def test_batched_512_tanks_fp32c_thirty_steps(gpu_lib, batch):
    P32 = physics.baseline_params(2, precision=_abi.TG_FP32C)
    with gpu_context(batch, P32) as ctx:
        ctx.step(30)
        g = gpu_state(ctx)
    assert np.all(np.isfinite(g["r"])) and np.all(np.isfinite(g["rho"]))
    tanks = list(range(0, 512, 16))
    sub, rows = _subset(batch, tanks)
    o = oracle_run(sub, physics.baseline_params(2), 30)
    f = fluid_mask(sub)
    np.testing.assert_allclose(g["time"][tanks], o.time, rtol=1e-5)
    assert rel_l2(g["rho"][rows][f], o.rho[f]) <= 1e-5
    assert rel_l2(g["r"][rows][f], o.r[f]) <= 1e-6
    # Per tank as well: no tank hides behind the others.
    start = 0
    for t in sub["tanks"]:
        sl = slice(start, start + t["n_fluid"])
        assert rel_l2(g["rho"][rows][sl], o.rho[sl]) <= 1e-5
        assert rel_l2(g["r"][rows][sl], o.r[sl]) <= 1e-6
        start += t["n_fluid"] + t["n_wall"]
