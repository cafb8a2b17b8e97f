"""Scenario generators: the sizes the benchmark configurations name."""

from __future__ import annotations

import numpy as np
import pytest

from titsolver_gb300 import scenarios


def test_dam_break_2d_counts_and_layout():
    s = scenarios.dam_break_2d()
    t = s["tanks"][0]
    assert t["n_fluid"] == 12_800
    assert 2_600 <= t["n_wall"] <= 2_800
    dx = s["dx"]
    # Fluid at dx * (i + 1, j + 1), i outer (wcsph.cpp:104-109).
    np.testing.assert_array_equal(s["r"][0], [dx, dx])
    np.testing.assert_array_equal(s["r"][1], [dx, 2 * dx])
    np.testing.assert_array_equal(s["r"][80], [2 * dx, dx])
    assert t["h"] == 2 * dx and t["m"] == 1000.0 * dx * dx
    assert t["cs0"] == 10 * np.sqrt(9.81 * 1.0)
    # Hydrostatic: denser at the bottom.
    assert s["rho"][0] > s["rho"][70] > 1000.0 and abs(s["rho"][79] - 1000.0) < 1e-9
    # Walls are three lattice layers and do not overlap the fluid.
    walls = s["r"][t["n_fluid"]:]
    assert walls[:, 1].min() == -2 * dx and walls[:, 0].min() == -2 * dx
    d = np.abs(walls[:, None, :2] - s["r"][None, :50, :]).sum(-1)
    assert d.min() > 0.5 * dx


def test_dam_break_2d_full_size_counts():
    s = scenarios.dam_break_2d(nx_per_H=800)
    t = s["tanks"][0]
    assert t["n_fluid"] == 1_280_000
    assert 26_000 < t["n_wall"] < 28_000


def test_dam_break_3d_small():
    s = scenarios.dam_break_3d(nx_per_H=8)
    t = s["tanks"][0]
    assert t["n_fluid"] == 16 * 8 * 8
    assert t["h"] == 1.3 * s["dx"]
    r = s["r"]
    nf = t["n_fluid"]
    # No wall coincides with a fluid particle.
    wk = {tuple(np.round(x / s["dx"]).astype(int)) for x in r[nf:]}
    fk = {tuple(np.round(x / s["dx"]).astype(int)) for x in r[:nf]}
    assert not (wk & fk)
    assert len(wk) == t["n_wall"]


def test_cloud_3d_deterministic_and_in_box():
    a = scenarios.cloud_3d(n_total=20_000, seed=3)
    b = scenarios.cloud_3d(n_total=20_000, seed=3)
    np.testing.assert_array_equal(a["r"], b["r"])
    assert a["r"].shape[0] == 20_000
    assert a["r"].min() >= 0.0 and a["r"].max() <= 1.0


def test_batched_tanks_sizes():
    s = scenarios.batched_tanks(n_tanks=64, seed=1)
    nf = np.array([t["n_fluid"] for t in s["tanks"]])
    assert nf.min() >= 200 and nf.max() <= 29_000
    assert s["r"].shape[0] == sum(t["n_fluid"] + t["n_wall"] for t in s["tanks"])


def test_batched_tanks_3d_layout():
    scn = scenarios.batched_tanks_3d(n_tanks=5, n_range=(6, 9), seed=3)
    assert scn["dim"] == 3 and len(scn["tanks"]) == 5
    n = sum(t["n_fluid"] + t["n_wall"] for t in scn["tanks"])
    assert scn["r"].shape == (n, 3) and scn["rho"].shape == (n,)
    base = 0
    for t in scn["tanks"]:
        assert t["h"] == pytest.approx(1.3 * scn["dx"])
        assert t["m"] == pytest.approx(1000.0 * scn["dx"] ** 3)
        fl = scn["r"][base:base + t["n_fluid"]]
        # Fluid on the dx lattice from dx, walls after it.
        assert np.all(fl.min(axis=0) == pytest.approx(scn["dx"]))
        base += t["n_fluid"] + t["n_wall"]
