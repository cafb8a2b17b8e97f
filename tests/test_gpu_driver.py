"""The titwcsph-style C++ driver (titsolver_gb300/host/titwcsph_gpu.cpp) on
the GPU through the C++ mirror: its initial state, run through the oracle
(the reference term set, with or without the post-step shifting, with
particle walls or the reference's face walls, as the driver ran), must give
its final state (plain FP64: r and rho 1e-12, v 1e-10 relative L2 after
20 steps, against measured r, rho <= 6e-16 and v <= 1.7e-13 on GB300;
FP32-compensated: rho 1e-5, r 1e-6), and its
.ttdb frames must hold that final state."""

from __future__ import annotations

import sqlite3
import subprocess

import numpy as np
import pytest

from helpers import oracle_run, rel_l2
from test_host_mirror import decode
from titsolver_gb300 import _abi, build as gpu_build, physics

pytestmark = pytest.mark.gpu


def read_dump(path):
    raw = path.read_bytes()
    n, nf, steps = np.frombuffer(raw, "<i8", 3)
    h, m, rho0, cs0, t = np.frombuffer(raw, "<f8", 5, offset=24)
    off = 64

    def state(off):
        r = np.frombuffer(raw, "<f8", 2 * n, offset=off).reshape(n, 2)
        off += 16 * n
        v = np.frombuffer(raw, "<f8", 2 * n, offset=off).reshape(n, 2)
        off += 16 * n
        rho = np.frombuffer(raw, "<f8", n, offset=off)
        return (r, v, rho), off + 8 * n

    init, off = state(off)
    final, off = state(off)
    faces = None
    if off < len(raw):  # --faces: face vertex pairs and containment polygon
        nfaces = int(np.frombuffer(raw, "<i8", 1, offset=off)[0])
        off += 8
        fv = np.frombuffer(raw, "<i4", 2 * nfaces, offset=off).reshape(nfaces, 2)
        off += 8 * nfaces
        npoly = int(np.frombuffer(raw, "<i8", 1, offset=off)[0])
        off += 8
        poly = np.frombuffer(raw, "<f8", 2 * npoly, offset=off).reshape(npoly, 2)
        off += 16 * npoly
        faces = [dict(face_verts=fv.copy(), poly=poly.copy())]
    assert off == len(raw)
    tank = dict(n_fluid=int(nf), n_wall=int(n - nf), h=float(h), m=float(m),
                rho0=float(rho0), cs0=float(cs0))
    return tank, init, final, float(t), int(steps), faces


INTEGRATORS = {"ssprk3": _abi.TG_SSPRK3, "ssprk2": _abi.TG_SSPRK2,
               "euler": _abi.TG_EULER, "verlet": _abi.TG_VERLET}


@pytest.mark.parametrize("fp32c,integrator,shifting,faces", [
    (False, "ssprk3", True, False), (True, "ssprk3", True, False),
    (False, "ssprk3", False, False), (False, "ssprk2", True, False),
    (False, "euler", True, False), (False, "verlet", False, False),
    (False, "ssprk3", True, True), (False, "verlet", True, True), (True, "ssprk3", True, True),
    ("face32", "ssprk3", True, True)])
def test_driver_matches_oracle(gpu_lib, tmp_path, fp32c, integrator, shifting, faces):
    # fp32c = "face32": the compensated form with --face-fp32 (FP32 face
    # integrals), held to the compensated form's tolerances.
    exe = gpu_build.build_host()["titwcsph_gpu"]
    dump, ttdb = tmp_path / "state.bin", tmp_path / "particles.ttdb"
    cmd = [str(exe), "--nx", "20", "--steps", "20", "--dump", str(dump), "--ttdb", str(ttdb),
           "--integrator", integrator]
    if fp32c:
        cmd.append("--fp32c")
    if fp32c == "face32":
        cmd.append("--face-fp32")
    if not shifting:
        cmd.append("--no-shifting")
    if faces:
        cmd.append("--faces")
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    tank, (r0, v0, rho0), (r1, v1, rho1), t, steps, fc = read_dump(dump)
    assert steps == 20
    assert (fc is not None) == faces
    scn = dict(dim=2, tanks=[tank], r=r0.copy(), v=v0.copy(), rho=rho0.copy(), faces=fc)
    # The driver's physics: the reference term set, C4 Wendland, mu = 0.001.
    P = physics.reference_params(2)
    P.integrator = INTEGRATORS[integrator]
    P.post_integrate = _abi.TG_POST_SHIFTING if shifting else _abi.TG_POST_PREPARE
    o = oracle_run(scn, P, steps)
    f = np.arange(r0.shape[0]) < tank["n_fluid"]
    np.testing.assert_allclose(t, o.time[0], rtol=1e-12 if not fp32c else 1e-6)
    if fp32c:
        assert rel_l2(rho1[f], o.rho[f]) <= 1e-5
        assert rel_l2(r1[f], o.r[f]) <= 1e-6
    else:
        assert rel_l2(r1[f], o.r[f]) <= 1e-12
        assert rel_l2(v1[f], o.v[f]) <= 1e-10
        assert rel_l2(rho1[f], o.rho[f]) <= 1e-12
    # The .ttdb: frame 0 is the initial state, the last one the final state.
    con = sqlite3.connect(ttdb)
    frames = con.execute("SELECT id, time FROM DataFrames ORDER BY id").fetchall()
    assert len(frames) == 2 and frames[0][1] == 0.0 and frames[1][1] > 0.0
    arrays = {name: decode(data) for name, data in con.execute(
        "SELECT name, data FROM DataArrays WHERE frame_id = ?", (frames[1][0],))}
    assert {"r", "v", "dv_dt", "rho", "drho_dt", "p", "cs", "m"} <= set(arrays)
    np.testing.assert_array_equal(np.frombuffer(arrays["r"], "<f8").reshape(-1, 2), r1)
    np.testing.assert_array_equal(np.frombuffer(arrays["rho"], "<f8"), rho1)
    r_first = np.frombuffer(decode(con.execute(
        "SELECT data FROM DataArrays WHERE frame_id = ? AND name = 'r'",
        (frames[0][0],)).fetchone()[0]), "<f8").reshape(-1, 2)
    np.testing.assert_array_equal(r_first, r0)
    con.close()


def test_driver_linear_tait_matches_oracle(gpu_lib, tmp_path):
    # titwcsph with LinearTaitEquationOfState{cs_0, rho_0} and face walls.
    exe = gpu_build.build_host()["titwcsph_gpu"]
    dump = tmp_path / "state.bin"
    cmd = [str(exe), "--nx", "20", "--steps", "10", "--faces", "--eos", "linear",
           "--dump", str(dump)]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    tank, (r0, v0, rho0), (r1, v1, rho1), t, steps, fc = read_dump(dump)
    scn = dict(dim=2, tanks=[tank], r=r0.copy(), v=v0.copy(), rho=rho0.copy(), faces=fc)
    P = physics.reference_params(2)
    P.eos = _abi.TG_EOS_LINEAR_TAIT
    P.post_integrate = _abi.TG_POST_SHIFTING
    o = oracle_run(scn, P, steps)
    f = np.arange(r0.shape[0]) < tank["n_fluid"]
    assert rel_l2(r1[f], o.r[f]) <= 1e-9
    assert rel_l2(rho1[f], o.rho[f]) <= 1e-7


def test_titwcsph_full_run_to_the_reference_end_time(gpu_lib, tmp_path):
    # The reference's integration test runs titwcsph to t* = 10
    # (tests/titwcsph/test.cmake:10-16) and compares a platform-specific
    # checksum; here the same run (face walls, dr = H/80, compensated form)
    # must end cleanly with the physics of a collapsed column: every fluid
    # particle finite and inside the pool, the mean height about halved,
    # densities within 2% of rho_0.
    exe = gpu_build.build_host()["titwcsph_gpu"]
    dump = tmp_path / "state.bin"
    cmd = [str(exe), "--faces", "--fp32c", "--nx", "80", "--end-time", "10", "--dump", str(dump)]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    tank, (r0, v0, rho0), (r1, v1, rho1), t, steps, fc = read_dump(dump)
    nf = tank["n_fluid"]
    assert t * np.sqrt(9.81 / 0.6) >= 10.0
    assert np.all(np.isfinite(r1)) and np.all(np.isfinite(v1)) and np.all(np.isfinite(rho1))
    poly = fc[0]["poly"]
    assert np.all((r1[:nf] > poly.min(axis=0)) & (r1[:nf] < poly.max(axis=0)))
    assert 0.4 < r1[:nf, 1].mean() / r0[:nf, 1].mean() < 0.6
    assert r1[:nf, 0].max() > 0.95 * poly[:, 0].max()
    assert np.all(np.abs(rho1[:nf] / 1000.0 - 1.0) < 0.02)
    np.testing.assert_array_equal(r1[nf:], r0[nf:])


def test_driver_log_lines(gpu_lib):
    # --log prints the reference's per-step line (wcsph.cpp:172-176): step,
    # scaled time, and the wall seconds of the previous step and write.
    exe = gpu_build.build_host()["titwcsph_gpu"]
    res = subprocess.run([str(exe), "--nx", "10", "--steps", "3", "--log"],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    rows = [line.split() for line in res.stdout.splitlines() if line.startswith(" ")]
    assert [int(r[0]) for r in rows] == [1, 2, 3]
    times = [float(r[1]) for r in rows]
    assert times[0] == 0.0 and times[0] < times[1] < times[2]
    assert all(len(r) == 4 for r in rows)
