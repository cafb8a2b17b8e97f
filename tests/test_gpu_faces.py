"""Semi-analytical face boundaries on the GPU (FP64 and the compensated
form) against the oracle: in 2D on the titwcsph scenario itself
(source/titwcsph/wcsph.cpp:37-142: tessellated pool faces with one fixed
particle per vertex, containment by the pool polygon), in 3D on the same
pool extruded, with triangulated sides and a box containment mesh.
Tolerances (relative L2 over the fluid): 1 step r, v, rho <= 1e-11 and
dv/dt, drho/dt <= 1e-9; 5 steps <= 1e-10."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import fluid_mask, gpu_context, gpu_state, oracle_run, rel_l2
from titsolver_gb300 import _abi, physics, scenarios

pytestmark = pytest.mark.gpu


def _compare(scn, P, steps, tol, tol_deriv=None):
    with gpu_context(scn, P) as ctx:
        dt = ctx.step(steps)
        g = gpu_state(ctx)
    o = oracle_run(scn, P, steps)
    f = fluid_mask(scn)
    np.testing.assert_allclose(dt, o.dt, rtol=1e-12)
    assert rel_l2(g["r"][f], o.r[f]) <= tol
    assert rel_l2(g["v"][f], o.v[f]) <= tol * 1e2
    assert rel_l2(g["rho"][f], o.rho[f]) <= tol
    assert rel_l2(g["rho"][~f], o.rho[~f]) <= tol
    if tol_deriv is not None:
        assert rel_l2(g["dv_dt"][f], o.dv_dt[f]) <= tol_deriv
        assert rel_l2(g["drho_dt"][f], o.drho_dt[f]) <= tol_deriv
    return g, o


@pytest.mark.parametrize("shifting", (False, True))
def test_titwcsph_faces_vs_oracle(gpu_lib, shifting):
    scn = scenarios.dam_break_2d_faces(nx_per_H=20)
    P = physics.reference_params(2)
    P.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    _compare(scn, P, 1, 1e-11, 1e-9)
    _compare(scn, P, 5, 1e-10)


@pytest.mark.parametrize("kernel", (_abi.TG_KERNEL_WENDLAND_C2, _abi.TG_KERNEL_CUBIC_SPLINE,
                                    _abi.TG_KERNEL_QUINTIC_SPLINE))
def test_faces_other_kernels_and_term_sets(gpu_lib, kernel):
    scn = scenarios.dam_break_2d_faces(nx_per_H=16)
    _compare(scn, physics.reference_params(2, kernel=kernel), 2, 1e-10)
    _compare(scn, physics.baseline_params(2, kernel=kernel), 2, 1e-10)


def test_faces_linear_tait(gpu_lib):
    scn = scenarios.dam_break_2d_faces(nx_per_H=16)
    P = physics.reference_params(2)
    P.eos = _abi.TG_EOS_LINEAR_TAIT
    P.post_integrate = _abi.TG_POST_SHIFTING
    _compare(scn, P, 1, 1e-11, 1e-9)
    _compare(scn, P, 3, 1e-10)


@pytest.mark.parametrize("integrator", (_abi.TG_EULER, _abi.TG_VERLET, _abi.TG_SSPRK2))
def test_faces_other_integrators(gpu_lib, integrator):
    scn = scenarios.dam_break_2d_faces(nx_per_H=16)
    P = physics.reference_params(2)
    P.integrator = integrator
    _compare(scn, P, 3, 1e-10)


def test_faces_batched_with_a_particle_wall_tank(gpu_lib):
    a = scenarios.dam_break_2d_faces(nx_per_H=12)
    b = scenarios.dam_break_2d(nx_per_H=10)
    c = scenarios.dam_break_2d_faces(nx_per_H=16)
    scn = dict(dim=2, tanks=a["tanks"] + b["tanks"] + c["tanks"],
               r=np.concatenate([a["r"], b["r"], c["r"]]),
               v=np.concatenate([a["v"], b["v"], c["v"]]),
               rho=np.concatenate([a["rho"], b["rho"], c["rho"]]),
               faces=[a["faces"][0], None, c["faces"][0]])
    _compare(scn, physics.reference_params(2), 3, 1e-10)


def test_faces_survive_autotune_and_reject_bad_vertices(gpu_lib):
    scn = scenarios.dam_break_2d_faces(nx_per_H=16)
    P = physics.reference_params(2)
    f = fluid_mask(scn)
    with gpu_context(scn, P) as ctx, gpu_context(scn, P) as ref:
        ctx.step(2)
        ref.step(2)
        ctx.autotune(2)
        ctx.step(3)
        ref.step(3)
        a, b = gpu_state(ctx), gpu_state(ref)
    assert rel_l2(a["rho"][f], b["rho"][f]) <= 1e-11
    assert rel_l2(a["r"][f], b["r"][f]) <= 1e-11
    with _abi.Context(P) as ctx:
        ctx.upload(scn["tanks"], scn["r"], scn["v"], scn["rho"])
        bad = np.array([[0, 10**6]], dtype=np.int32)
        with pytest.raises(_abi.TgError):
            ctx.set_faces(0, bad, scn["faces"][0]["poly"])
    s3 = _scn3()
    with _abi.Context(physics.reference_params(3)) as ctx:
        ctx.upload(s3["tanks"], s3["r"], s3["v"], s3["rho"])
        fv = s3["faces"][0]["face_verts"]
        with pytest.raises(_abi.TgError) as ei:
            ctx.set_faces(0, np.array([[0, 1, 10**6]], dtype=np.int32), s3["faces"][0]["poly"])
        assert ei.value.status == _abi.TG_ERR_INVALID_ARGUMENT
        with pytest.raises(_abi.TgError):
            ctx.set_faces(0, fv, s3["faces"][0]["poly"][:3])


def _scn3(nx_per_H=6):
    return scenarios.dam_break_3d_faces(nx_per_H=nx_per_H, tank=(3.0, 1.5))


@pytest.mark.parametrize("shifting", (False, True))
def test_3d_faces_vs_oracle(gpu_lib, shifting):
    scn = _scn3()
    P = physics.reference_params(3)
    P.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    _compare(scn, P, 1, 1e-11, 1e-9)
    _compare(scn, P, 4, 1e-10)


@pytest.mark.parametrize("kernel", (_abi.TG_KERNEL_WENDLAND_C2, _abi.TG_KERNEL_CUBIC_SPLINE))
def test_3d_faces_other_kernels_and_term_sets(gpu_lib, kernel):
    scn = _scn3()
    _compare(scn, physics.reference_params(3, kernel=kernel), 2, 1e-10)
    _compare(scn, physics.baseline_params(3, kernel=kernel), 2, 1e-10)


@pytest.mark.parametrize("integrator", (_abi.TG_EULER, _abi.TG_VERLET, _abi.TG_SSPRK2))
def test_3d_faces_other_integrators(gpu_lib, integrator):
    scn = _scn3()
    P = physics.reference_params(3)
    P.integrator = integrator
    _compare(scn, P, 3, 1e-10)


def test_3d_faces_survive_autotune(gpu_lib):
    scn = _scn3()
    P = physics.reference_params(3)
    P.post_integrate = _abi.TG_POST_SHIFTING
    f = fluid_mask(scn)
    with gpu_context(scn, P) as ctx, gpu_context(scn, P) as ref:
        ctx.step(1)
        ref.step(1)
        ctx.autotune(2)
        ctx.step(2)
        ref.step(2)
        a, b = gpu_state(ctx), gpu_state(ref)
    assert rel_l2(a["rho"][f], b["rho"][f]) <= 1e-11
    assert rel_l2(a["r"][f], b["r"][f]) <= 1e-11


def test_3d_faces_batched_with_a_particle_wall_tank(gpu_lib):
    a = _scn3()
    b = scenarios.dam_break_3d(nx_per_H=6)
    scn = dict(dim=3, tanks=a["tanks"] + b["tanks"],
               r=np.concatenate([a["r"], b["r"]]), v=np.concatenate([a["v"], b["v"]]),
               rho=np.concatenate([a["rho"], b["rho"]]), faces=[a["faces"][0], None])
    _compare(scn, physics.reference_params(3), 2, 1e-10)


def test_3d_faces_fp32_compensated_vs_fp64_oracle(gpu_lib):
    scn = _scn3()
    P64 = physics.reference_params(3)
    P32 = physics.reference_params(3, precision=_abi.TG_FP32C)
    o = oracle_run(scn, P64, 20)
    f = fluid_mask(scn)
    with gpu_context(scn, P32) as ctx:
        ctx.step(20)
        g = gpu_state(ctx)
    assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-5
    assert rel_l2(g["r"][f], o.r[f]) <= 1e-6


@pytest.mark.parametrize("shifting", (False, True))
def test_faces_fp32_compensated_vs_fp64_oracle(gpu_lib, shifting):
    # The compensated form with face walls: face integrals in FP64 (the
    # default, face_fp32 = 0), pair sums in FP32 with Kahan sums, against the
    # FP64 oracle after 30 steps.
    scn = scenarios.dam_break_2d_faces(nx_per_H=20)
    P64 = physics.reference_params(2)
    P32 = physics.reference_params(2, precision=_abi.TG_FP32C)
    for P in (P64, P32):
        P.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    o = oracle_run(scn, P64, 30)
    f = fluid_mask(scn)
    with gpu_context(scn, P32) as ctx:
        ctx.step(30)
        g = gpu_state(ctx)
    assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-5
    assert rel_l2(g["r"][f], o.r[f]) <= 1e-6


def test_3d_faces_past_the_warp_face_list(gpu_lib):
    # Walls tessellated at dr/3: a particle next to a wall has more faces
    # within its support radius than the per-warp list of k_gamma_faces
    # holds (256), so it takes the list-free path while particles further
    # from the walls take the listed one; both against the oracle.
    scn = scenarios.dam_break_3d_faces(nx_per_H=6, tank=(3.0, 1.5), face_refine=3)
    t = scn["tanks"][0]
    radius = 2.0 * t["h"]
    cent = scn["r"][t["n_fluid"]:][scn["faces"][0]["face_verts"]].mean(axis=1)
    fl = scn["r"][:t["n_fluid"]]
    # A face whose centroid lies within the radius is within reach.
    within = (((fl[:, None, :] - cent[None, :, :]) ** 2).sum(-1) <= radius ** 2).sum(1)
    assert within.max() > 256
    assert within.min() <= 256
    _compare(scn, physics.reference_params(3), 2, 1e-10)


def _fp32_faces_params(dim, shifting, face_fp32, kernel=_abi.TG_KERNEL_WENDLAND_C4):
    P = physics.reference_params(dim, precision=_abi.TG_FP32C, kernel=kernel)
    P.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    P.face_fp32 = face_fp32
    return P


@pytest.mark.parametrize("dim,shifting", ((2, False), (2, True), (3, False), (3, True)))
def test_faces_fp32_integrals_vs_fp64_oracle(gpu_lib, dim, shifting):
    # tg_params.face_fp32: the compensated form with the closed-form face
    # integrals in FP32 too (face selection, frames and the sums over faces
    # stay FP64).  Against the FP64 oracle after 30 (2D) / 20 (3D) steps:
    # rho <= 1e-5 and r <= 5e-6 relative L2 over the fluid.
    scn = scenarios.dam_break_2d_faces(nx_per_H=20) if dim == 2 else _scn3()
    steps = 30 if dim == 2 else 20
    P64 = physics.reference_params(dim)
    P64.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    o = oracle_run(scn, P64, steps)
    f = fluid_mask(scn)
    with gpu_context(scn, _fp32_faces_params(dim, shifting, 1)) as ctx:
        ctx.step(steps)
        g = gpu_state(ctx)
    assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-5
    assert rel_l2(g["r"][f], o.r[f]) <= 5e-6
    # The switch is live: the FP64-integral run of the same form differs.
    with gpu_context(scn, _fp32_faces_params(dim, shifting, 0)) as ctx:
        ctx.step(steps)
        h = gpu_state(ctx)
    assert rel_l2(g["r"][f], h["r"][f]) > 0.0


@pytest.mark.parametrize("kernel", range(6))
def test_faces_fp32_integrals_every_kernel(gpu_lib, kernel):
    # Every kernel's FP32 face integrals (2D segments and 3D triangles)
    # against the FP64 oracle after 4 steps: rho and r <= 1e-6.
    for dim, scn in ((2, scenarios.dam_break_2d_faces(nx_per_H=20)), (3, _scn3())):
        P64 = physics.reference_params(dim, kernel=kernel)
        o = oracle_run(scn, P64, 4)
        f = fluid_mask(scn)
        with gpu_context(scn, _fp32_faces_params(dim, False, 1, kernel)) as ctx:
            ctx.step(4)
            g = gpu_state(ctx)
        assert rel_l2(g["rho"][f], o.rho[f]) <= 1e-6
        assert rel_l2(g["r"][f], o.r[f]) <= 1e-6


# Drift of the compensated form with face walls over 1000 steps, relative
# L2 over the fluid.  The bounds sit 2-3x above the values measured on the
# current build (given per case); shifting's discrete free-surface decisions
# amplify rounding differences, and FP32 face integrals (face_fp32) add
# their own rounding.
_DRIFT_2D = {  # shifting -> face_fp32 -> (rho, r) bounds
    False: {0: (1e-6, 2e-5), 1: (1e-5, 2e-4)},  # measured 2.1e-7 / 9.0e-6; 2.3e-6 / 6.8e-5
    True: {0: (1e-4, 1e-5), 1: (1e-4, 2e-4)},   # measured 4.2e-5 / 2.9e-6; 4.6e-5 / 8.0e-5
}


@pytest.mark.parametrize("shifting", (False, True))
def test_faces_fp32_compensated_1000_steps_vs_fp64_oracle(gpu_lib, shifting):
    # The 2D pool with face walls (800 fluid) against the FP64 oracle after
    # 1000 steps, face integrals in FP64 and in FP32.  With FP64 integrals
    # the drift is within the compensated form's targets (rho <= 1e-4,
    # r <= 1e-5) with shifting; without it r stays below 2e-5.
    scn = scenarios.dam_break_2d_faces(nx_per_H=20)
    P64 = physics.reference_params(2)
    P64.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    o = oracle_run(scn, P64, 1000)
    f = fluid_mask(scn)
    for face_fp32 in (0, 1):
        with gpu_context(scn, _fp32_faces_params(2, shifting, face_fp32, P64.kernel)) as ctx:
            ctx.step(1000)
            g = gpu_state(ctx)
        rho_b, r_b = _DRIFT_2D[shifting][face_fp32]
        assert rel_l2(g["rho"][f], o.rho[f]) <= rho_b
        assert rel_l2(g["r"][f], o.r[f]) <= r_b


def test_3d_faces_fp32_compensated_1000_steps_vs_fp64(gpu_lib):
    # The 3D pool with triangle face walls (432 fluid, 6 particles per H)
    # after 1000 steps against the FP64 form on the GPU (whose short runs
    # match the FP64 oracle to 1e-10 above; 1000 oracle steps of this case
    # take minutes).  At this resolution the drift is sensitive to any
    # change of rounding: with FP32 face integrals rho measured 1.7e-5 and,
    # after the wall pass's lanes per wall changed from 8 to 4, 5.1e-5.
    # Measured with 8 lanes: FP64 integrals rho 9.9e-7, r 5.6e-5; FP32
    # integrals rho 1.7e-5, r 9.1e-4; with shifting, rho 6.7e-5, r 3.7e-3
    # (FP64 integrals): the free-surface decisions of shifting flip between
    # the forms and move particles apart.  The bounds are about 10x those.
    scn = _scn3()
    f = fluid_mask(scn)
    cases = ((False, 0, 1e-5, 5e-4), (False, 1, 2e-4, 1e-2), (True, 0, 1e-3, 3e-2))
    got = []
    for shifting, face_fp32, rho_b, r_b in cases:
        P64 = physics.reference_params(3)
        P64.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
        with gpu_context(scn, P64) as ctx:
            ctx.step(1000)
            ref = gpu_state(ctx)
        with gpu_context(scn, _fp32_faces_params(3, shifting, face_fp32, P64.kernel)) as ctx:
            ctx.step(1000)
            g = gpu_state(ctx)
        got.append((shifting, face_fp32, rel_l2(g["rho"][f], ref["rho"][f]),
                    rel_l2(g["r"][f], ref["r"][f]), rho_b, r_b))
    for shifting, face_fp32, rho, r, rho_b, r_b in got:
        assert rho <= rho_b and r <= r_b, got
