"""Generate the committed golden fixtures of tests/golden/ from the oracle.

Run from the repository root:  python tests/golden/make_golden.py

Fixtures (small, seeded, deterministic):
  search_mt19937.npz   the reference's search test inputs (std::mt19937{123},
                       200 uniform points in 2D and 3D) and the naive O(N^2)
                       neighbour lists for radii {0.01, 0.1, 0.5, 1.0}
                       (source/tit/geom/search.test.cpp:130-163)
  kernels.npz          W and grad W of the six kernels at fixed points
  dam_break_small.npz  a 20 x 10 dam break, both term sets: state after 0, 1
                       and 10 SSPRK3 steps
  dam3d_small.npz      a 16 x 8 x 8 3D dam break after 2 steps
  batched_small.npz    4 independent tanks after 3 steps
  cloud_small.npz      a 6,000-point 3D cloud: summation density, neighbour
                       counts and hashes with FP64 and FP32 positions
"""

from __future__ import annotations

import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from titsolver_gb300 import physics, scenarios  # noqa: E402

RADII = (0.01, 0.1, 0.5, 1.0)


def _csr_pack(prefix, off, idx, out):
    out[prefix + "_off"] = off
    out[prefix + "_idx"] = idx


def search_fixture():
    out = {}
    for dim in (2, 3):
        pts = oracle.mt19937_uniform_points(123, 200, dim)
        out[f"points_{dim}d"] = pts
        for r in RADII:
            off, idx = oracle.naive_search(pts, r, inclusive=False)
            _csr_pack(f"naive_{dim}d_{r}", off, idx, out)
    np.savez_compressed(HERE / "search_mt19937.npz", **out)


def kernel_fixture():
    rng = np.random.Generator(np.random.PCG64(7))
    out = {}
    for dim in (2, 3):
        x = rng.uniform(-1.2, 1.2, size=(64, dim)) * 0.1
        out[f"x_{dim}d"] = x
        for k in range(6):
            out[f"W_{k}_{dim}d"] = np.array([oracle.kernel_value(k, xi, 0.1) for xi in x])
            out[f"gW_{k}_{dim}d"] = np.array([oracle.kernel_grad(k, xi, 0.1) for xi in x])
    np.savez_compressed(HERE / "kernels.npz", **out)


def _run(scn, params, steps):
    st = oracle.State(scn)
    snaps = {}
    done = 0
    for s in steps:
        if s > done:
            oracle.step(params, st, s - done, nthreads=1)
            done = s
        snaps[s] = (st.r.copy(), st.v.copy(), st.rho.copy(), st.dv_dt.copy(),
                    st.drho_dt.copy(), st.time.copy())
    return snaps


def _store(prefix, snaps, out):
    for s, (r, v, rho, dv, drho, t) in snaps.items():
        out[f"{prefix}_{s}_r"] = r
        out[f"{prefix}_{s}_v"] = v
        out[f"{prefix}_{s}_rho"] = rho
        out[f"{prefix}_{s}_dv_dt"] = dv
        out[f"{prefix}_{s}_drho_dt"] = drho
        out[f"{prefix}_{s}_time"] = t


def dam_fixture():
    scn = scenarios.dam_break_2d(nx_per_H=10)
    out = {"r0": scn["r"], "rho0": scn["rho"], "n_fluid": scn["tanks"][0]["n_fluid"],
           "n_wall": scn["tanks"][0]["n_wall"]}
    _store("baseline", _run(scn, physics.baseline_params(2), (0, 1, 10)), out)
    _store("reference", _run(scn, physics.reference_params(2), (0, 1, 10)), out)
    np.savez_compressed(HERE / "dam_break_small.npz", **out)


def dam3d_fixture():
    scn = scenarios.dam_break_3d(nx_per_H=8)
    out = {"r0": scn["r"], "rho0": scn["rho"]}
    _store("baseline", _run(scn, physics.baseline_params(3), (0, 2)), out)
    np.savez_compressed(HERE / "dam3d_small.npz", **out)


def batched_fixture():
    scn = scenarios.batched_tanks(n_tanks=4, n_range=(6, 12), seed=11)
    out = {"r0": scn["r"], "rho0": scn["rho"],
           "n_fluid": np.array([t["n_fluid"] for t in scn["tanks"]]),
           "n_wall": np.array([t["n_wall"] for t in scn["tanks"]])}
    _store("baseline", _run(scn, physics.baseline_params(2), (0, 3)), out)
    np.savez_compressed(HERE / "batched_small.npz", **out)


def cloud_fixture():
    scn = scenarios.cloud_3d(n_total=6000, seed=5)
    t = scn["tanks"][0]
    out = {"r": scn["r"], "h": t["h"], "m": t["m"]}
    for prec in (0, 1):
        rho, cnt, hs = oracle.summation_density(scn["r"], t["h"], t["m"], 3, prec, nthreads=1)
        out[f"rho_{prec}"] = rho
        out[f"count_{prec}"] = cnt
        out[f"hash_{prec}"] = hs
    np.savez_compressed(HERE / "cloud_small.npz", **out)


if __name__ == "__main__":
    search_fixture()
    kernel_fixture()
    dam_fixture()
    dam3d_fixture()
    batched_fixture()
    cloud_fixture()
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)
