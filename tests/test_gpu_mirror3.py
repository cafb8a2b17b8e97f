"""The C++ mirror in 3D with triangle face walls (tests/cpp/mirror_faces3.cpp):
the extruded titwcsph pool set up through the reference-style API
(geom::tessellate of a box, geom::MakeFastWinding, FluidEquations,
SSPRKIntegrator, ParticleArray) and stepped on the GPU; its initial state,
faces and containment run through the oracle must give its final state
(plain FP64: r 1e-10, v and rho 1e-8 relative L2 over the fluid after 3
steps; FP32-compensated: rho 1e-5, r 1e-6)."""

from __future__ import annotations

import pathlib
import subprocess

import numpy as np
import pytest

from helpers import oracle_run, rel_l2
from titsolver_gb300 import _abi, build as gpu_build, physics

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def mirror_faces3(tmp_path_factory, gpu_lib):
    exe = tmp_path_factory.mktemp("mirror3") / "mirror_faces3"
    lib_dir = gpu_build.OUT_DIR
    cmd = ["g++", "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "mirror_faces3.cpp"),
           "-L", str(lib_dir), "-ltitgpu", f"-Wl,-rpath,{lib_dir}", "-ldl", "-pthread",
           "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def read_dump(path):
    raw = path.read_bytes()
    n, nf, steps = (int(x) for x in np.frombuffer(raw, "<i8", 3))
    h, m, rho0, cs0 = np.frombuffer(raw, "<f8", 4, offset=24)
    off = 56

    def state(off):
        r = np.frombuffer(raw, "<f8", 3 * n, offset=off).reshape(n, 3)
        off += 24 * n
        v = np.frombuffer(raw, "<f8", 3 * n, offset=off).reshape(n, 3)
        off += 24 * n
        rho = np.frombuffer(raw, "<f8", n, offset=off)
        return (r.copy(), v.copy(), rho.copy()), off + 8 * n

    init, off = state(off)
    final, off = state(off)
    nfaces = int(np.frombuffer(raw, "<i8", 1, offset=off)[0])
    off += 8
    fv = np.frombuffer(raw, "<i4", 3 * nfaces, offset=off).reshape(nfaces, 3).copy()
    off += 12 * nfaces
    ntris = int(np.frombuffer(raw, "<i8", 1, offset=off)[0])
    off += 8
    tris = np.frombuffer(raw, "<f8", 9 * ntris, offset=off).reshape(ntris, 3, 3).copy()
    off += 72 * ntris
    assert off == len(raw)
    tank = dict(n_fluid=nf, n_wall=n - nf, h=float(h), m=float(m), rho0=float(rho0),
                cs0=float(cs0))
    return tank, init, final, steps, dict(face_verts=fv, poly=tris)


@pytest.mark.parametrize("fp32c", (False, True))
def test_mirror_3d_faces_match_oracle(mirror_faces3, tmp_path, fp32c):
    out = tmp_path / "state.bin"
    cmd = [str(mirror_faces3), str(out), "--steps", "3"] + (["--fp32c"] if fp32c else [])
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    tank, (r0, v0, rho0), (r1, v1, rho1), steps, faces = read_dump(out)
    # The tessellated walls: every fixed particle is a face vertex and every
    # face edge is at most dr = h / 1.3.
    verts = r0[tank["n_fluid"]:]
    assert np.unique(faces["face_verts"]).size == verts.shape[0]
    tri = verts[faces["face_verts"]]
    edges = np.linalg.norm(tri - np.roll(tri, 1, axis=1), axis=2)
    assert edges.max() <= tank["h"] / 1.3 * (1 + 1e-12)
    scn = dict(dim=3, tanks=[tank], r=r0, v=v0, rho=rho0, faces=[faces])
    P = physics.reference_params(3)  # Ferrari + Morris, Wendland C4, shifting
    P.post_integrate = _abi.TG_POST_SHIFTING
    o = oracle_run(scn, P, steps)
    f = np.arange(r0.shape[0]) < tank["n_fluid"]
    if fp32c:
        assert rel_l2(rho1[f], o.rho[f]) <= 1e-5
        assert rel_l2(r1[f], o.r[f]) <= 1e-6
    else:
        assert rel_l2(r1[f], o.r[f]) <= 1e-10
        assert rel_l2(v1[f], o.v[f]) <= 1e-8
        assert rel_l2(rho1[f], o.rho[f]) <= 1e-8
