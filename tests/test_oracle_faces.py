"""The oracle's semi-analytical face boundaries (2D), pinned to the
reference's kernel tests: the antigradient flux of a segment is +-1/4 at
its vertices, +-1/2 on its inside and 0 on its line outside
(kernel.test.cpp:362-393), flux and antigradient flux match quadrature of
the kernel and of its antigradient and flip sign with the segment
(kernel.test.cpp:300-356); the winding-number containment; and a few steps
of the titwcsph face scenario."""

from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from titsolver_gb300 import physics, scenarios

KERNELS = range(6)


@pytest.mark.parametrize("kernel", KERNELS)
def test_antigrad_flux_on_the_segment_line(kernel):
    a, b = np.array([0.0, 0.0]), np.array([2.0, 2.0])
    for h in (1.0, 0.1, 0.01):
        assert abs(abs(oracle.kernel_antigrad_flux2(kernel, a, b, a, h)) - 0.25) < 1e-9
        assert abs(abs(oracle.kernel_antigrad_flux2(kernel, a, b, b, h)) - 0.25) < 1e-9
        for o in (0.9, 0.5, 0.1, 0.0, -0.1, -0.5, -0.9):
            x = a + 0.5 * (o + 1.0) * (b - a)
            assert abs(abs(oracle.kernel_antigrad_flux2(kernel, a, b, x, h)) - 0.5) < 1e-9
        for o in (1.0, 0.9, 0.5, 0.1):
            assert abs(oracle.kernel_antigrad_flux2(kernel, a, b, a - o, h)) < 1e-12
            assert abs(oracle.kernel_antigrad_flux2(kernel, a, b, b + o, h)) < 1e-12


def _quadrature(kernel, a, b, x, h, n=4000):
    """n (integral of W(x - y) ds) and -n . (integral of the antigradient),
    antigrad(x) = -x w h^-2 T(q) / q^2 (kernel.hpp:177-190), by the midpoint
    rule; T is the 2D tail moment, from the oracle's kernel values."""
    unit_radius, w = oracle.kernel_info(kernel, 2)
    t = (np.arange(n) + 0.5) / n
    y = a[None, :] + t[:, None] * (b - a)[None, :]
    rvec = x[None, :] - y
    r = np.hypot(rvec[:, 0], rvec[:, 1])
    q = r / h
    W = w / h**2 * np.array([oracle.unit_value(kernel, qi) for qi in q])
    # Tail moment T(q) = int_q^R s w(s) ds, by Gauss-Legendre on [q, R].
    gx, gw = np.polynomial.legendre.leggauss(24)
    T = np.zeros_like(q)
    for i, qi in enumerate(q):
        if qi >= unit_radius:
            continue
        s = 0.5 * (unit_radius - qi) * gx + 0.5 * (unit_radius + qi)
        fs = np.array([oracle.unit_value(kernel, si) for si in s])
        T[i] = 0.5 * (unit_radius - qi) * np.sum(gw * s * fs)
    ba = b - a
    length = float(np.hypot(*ba))
    nrm = np.array([ba[1], -ba[0]]) / length
    flux = nrm * np.sum(W) * length / n
    ag = -rvec * (w / h**2) * (T / q**2)[:, None]
    agf = -float(nrm @ (np.sum(ag, axis=0) * length / n))
    return flux, agf


@pytest.mark.parametrize("kernel", KERNELS)
def test_flux_matches_quadrature_and_flips(kernel):
    for h in (1.0, 0.1):
        a, b = np.array([0.0, 0.0]), np.array([2.0 * h, 0.0])
        for o in (1.0, 0.5, -0.5):
            for s in (1.0, 0.5, 0.1):
                x = np.array([1.0 * h + o * h, s * h])
                f = oracle.kernel_flux2(kernel, a, b, x, h)
                ag = oracle.kernel_antigrad_flux2(kernel, a, b, x, h)
                fq, agq = _quadrature(kernel, a, b, x, h)
                np.testing.assert_allclose(f, fq, rtol=1e-5, atol=1e-7 / h)
                assert abs(ag - agq) <= 1e-5 * max(1.0, abs(agq))
                np.testing.assert_allclose(oracle.kernel_flux2(kernel, b, a, x, h), -f,
                                           rtol=1e-12, atol=1e-14 / h)
                assert abs(oracle.kernel_antigrad_flux2(kernel, b, a, x, h) + ag) <= 1e-12


def test_flux_outside_support_is_zero():
    a, b = np.array([0.0, 0.0]), np.array([2.0, 0.0])
    for kernel in KERNELS:
        for h in (1.0, 0.1, 0.01):
            x = np.array([10.0, 10.0])
            assert np.all(oracle.kernel_flux2(kernel, a, b, x, h) == 0.0)
            assert oracle.kernel_antigrad_flux2(kernel, a, b, x, h) == 0.0


def test_winding_number_of_the_pool():
    poly = np.array([(0.0, 0.0), (2.0, 0.0), (2.0, 1.0), (0.0, 1.0)])
    assert abs(oracle.winding_number2(poly, np.array([1.0, 0.5])) - 1.0) < 1e-12
    assert abs(oracle.winding_number2(poly, np.array([3.0, 0.5]))) < 1e-12
    assert abs(oracle.winding_number2(poly[::-1].copy(), np.array([1.0, 0.5])) + 1.0) < 1e-12


def test_tessellation_matches_the_reference_layout():
    verts, faces = scenarios.rectangle_faces(2.0, 1.0, 0.25)
    # 4 corners + (8 - 1) + (4 - 1) + (8 - 1) + (4 - 1) new vertices.
    assert verts.shape == (24, 2) and faces.shape == (24, 2)
    # Every face joins consecutive points at most dx apart, and the loop
    # visits every vertex once as a start and once as an end.
    seg = verts[faces[:, 1]] - verts[faces[:, 0]]
    assert np.all(np.hypot(seg[:, 0], seg[:, 1]) <= 0.25 + 1e-12)
    assert sorted(faces[:, 0]) == list(range(24)) == sorted(faces[:, 1])


def test_titwcsph_face_scenario_steps():
    scn = scenarios.dam_break_2d_faces(nx_per_H=20)
    st = oracle.State(scn)
    P = physics.reference_params(2)
    P.post_integrate = 1
    nf = scn["tanks"][0]["n_fluid"]
    oracle.step(P, st, 20)
    assert np.all(np.isfinite(st.r)) and np.all(np.isfinite(st.rho))
    poly = scn["faces"][0]["poly"]
    inside = [oracle.winding_number2(poly, x) > 0.5 for x in st.r[:nf]]
    assert all(inside)
    # The column starts to collapse: the front moves right, nothing blows up.
    assert st.r[:nf, 0].max() > scn["r"][:nf, 0].max()
    assert np.abs(st.v[:nf]).max() < 1.0
    # Fixed particles (the face vertices) do not move.
    np.testing.assert_array_equal(st.r[nf:], scn["r"][nf:])
