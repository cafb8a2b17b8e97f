"""Shared helpers of the GPU parity tests: run a scenario through the C ABI
and through the oracle, and compare fields."""

from __future__ import annotations

import numpy as np

import oracle
from titsolver_gb300 import _abi


def gpu_context(scn: dict, params) -> _abi.Context:
    ctx = _abi.Context(params)
    ctx.upload(scn["tanks"], scn["r"], scn["v"], scn["rho"])
    for t, fc in enumerate(scn.get("faces") or []):
        if fc is not None:
            ctx.set_faces(t, fc["face_verts"], fc["poly"])
    return ctx


def gpu_state(ctx: _abi.Context) -> dict:
    return dict(r=ctx.download(_abi.TG_FIELD_R), v=ctx.download(_abi.TG_FIELD_V),
                rho=ctx.download(_abi.TG_FIELD_RHO),
                dv_dt=ctx.download(_abi.TG_FIELD_DV_DT),
                drho_dt=ctx.download(_abi.TG_FIELD_DRHO_DT), time=ctx.time())


def oracle_run(scn: dict, params, steps: int) -> oracle.State:
    st = oracle.State(scn)
    if steps:
        oracle.step(params, st, steps)
    return st


def fluid_mask(scn: dict) -> np.ndarray:
    mask = []
    for t in scn["tanks"]:
        mask.append(np.ones(t["n_fluid"], dtype=bool))
        mask.append(np.zeros(t["n_wall"], dtype=bool))
    return np.concatenate(mask)


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    den = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (den if den > 0 else 1.0)
