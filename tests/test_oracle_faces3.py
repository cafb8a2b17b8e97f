"""The oracle's semi-analytical face boundaries in 3D, pinned to the
reference's kernel tests: kernel flux and antigradient flux of a triangle
match quadrature of the kernel and of its antigradient and flip sign with
the triangle's orientation (kernel.test.cpp:237-293, 397-462); on the
triangle's plane the antigradient flux is +-1/12 at the vertices of the
unit-simplex face, +-1/4 on its edges, +-1/2 inside and 0 outside
(kernel.test.cpp:463-533); plus the triangle-sphere overlap of the face
adjacency (geom/triangle.hpp) and the winding-number containment."""

from __future__ import annotations

import functools
import math

import numpy as np
import pytest

import oracle

KERNELS = range(6)


@functools.lru_cache(maxsize=None)
def _radial_tables(kernel: int):
    """Unit kernel values w(q) and the 3D tail moment T(q) = int_q^R s^2 w(s)
    ds on a fine grid (the quadrature's integrand tables)."""
    unit_radius, weight = oracle.kernel_info(kernel, 3)
    q = np.linspace(0.0, unit_radius, 200001)
    w = np.array([oracle.unit_value(kernel, qi) for qi in q])
    f = q * q * w
    seg = 0.5 * (f[1:] + f[:-1]) * np.diff(q)
    tail = np.concatenate([np.cumsum(seg[::-1])[::-1], [0.0]])
    return unit_radius, weight, q, w, tail


def _tri_rule(a, b, c, n=96):
    """Points and weights of the midpoint-of-edges rule (degree 2) on the
    n^2 congruent sub-triangles of a-b-c."""
    pts, wts = [], []
    area = 0.5 * np.linalg.norm(np.cross(b - a, c - a))
    e1, e2 = (b - a) / n, (c - a) / n
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    up = (i + j) < n
    dn = (i + j) < n - 1
    for mask, corners in ((up, ((0, 0), (1, 0), (0, 1))), (dn, ((1, 0), (0, 1), (1, 1)))):
        ii, jj = i[mask], j[mask]
        vs = [a + (ii + ci)[:, None] * e1 + (jj + cj)[:, None] * e2 for ci, cj in corners]
        for p, q in ((0, 1), (1, 2), (2, 0)):
            pts.append(0.5 * (vs[p] + vs[q]))
            wts.append(np.full(len(ii), area / n**2 / 3.0))
    return np.concatenate(pts), np.concatenate(wts)


def _quadrature(kernel, a, b, c, x, h):
    """normal * integral of W(x - y) dA and -normal . integral of
    antigrad(x - y) dA, antigrad(x) = -x w h^-3 T(q)/q^3
    (kernel.hpp:177-190)."""
    unit_radius, weight, qt, wt, tt = _radial_tables(kernel)
    y, dA = _tri_rule(a, b, c)
    rvec = x[None, :] - y
    q = np.linalg.norm(rvec, axis=1) / h
    inside = q < unit_radius
    W = np.where(inside, np.interp(q, qt, wt), 0.0) * weight / h**3
    T = np.where(inside, np.interp(q, qt, tt), 0.0)
    n = np.cross(b - a, c - a)
    n /= np.linalg.norm(n)
    flux = n * np.sum(W * dA)
    with np.errstate(divide="ignore", invalid="ignore"):
        ag = -rvec * (weight / h**3 * T / q**3)[:, None]
    agf = -float(n @ np.sum(ag * dA[:, None], axis=0))
    return flux, agf


@pytest.mark.parametrize("kernel", KERNELS)
def test_triangle_partially_in_support(kernel):
    for h in (1.0, 0.1):
        a, b, c = np.array([3.0 * h, 0, 0]), np.array([0, 3.0 * h, 0]), np.array([0, 0, 3.0 * h])
        for o in (1.0, 0.5, 0.1, -0.5, -1.0):
            for s in (1.0, 0.5, 0.1):
                x = np.array([1.0 * h + o * h, 1.0 * h + s * h, 1.0 * h - s * h])
                f = oracle.kernel_flux3(kernel, a, b, c, x, h)
                ag = oracle.kernel_antigrad_flux3(kernel, a, b, c, x, h)
                fq, agq = _quadrature(kernel, a, b, c, x, h)
                np.testing.assert_allclose(f, fq, rtol=1e-6, atol=1e-9 / h)
                # The antigradient's 1/q^2 peak limits the quadrature near
                # the plane (o = 0.1) to about 1.5e-4.
                assert abs(ag - agq) <= 2e-4 * max(1e-2, abs(agq))
                np.testing.assert_allclose(oracle.kernel_flux3(kernel, c, b, a, x, h), -f,
                                           rtol=1e-10, atol=1e-12 / h)
                assert abs(oracle.kernel_antigrad_flux3(kernel, c, b, a, x, h) + ag) <= 1e-10


@pytest.mark.parametrize("kernel", KERNELS)
def test_triangle_fully_in_support(kernel):
    h = 1.0
    a, b, c = np.array([h / 6, 0, 0]), np.array([0, h / 6, 0]), np.array([0, 0, h / 6])
    for o in (1.0, 0.5, 0.1, -0.5):
        for s in (0.9, 0.1):
            x = np.array([o * h, s * h, -s * h])
            f = oracle.kernel_flux3(kernel, a, b, c, x, h)
            ag = oracle.kernel_antigrad_flux3(kernel, a, b, c, x, h)
            fq, agq = _quadrature(kernel, a, b, c, x, h)
            np.testing.assert_allclose(f, fq, rtol=2e-4, atol=1e-8)
            assert abs(ag - agq) <= 2e-4 * max(1e-3, abs(agq))
            np.testing.assert_allclose(oracle.kernel_flux3(kernel, c, b, a, x, h), -f,
                                       rtol=1e-10, atol=1e-14)


def test_triangle_outside_support():
    a, b, c = np.array([2.0, 0, 0]), np.array([0, 2.0, 0]), np.array([0, 0, 2.0])
    x = np.array([10.0, 10.0, 10.0])
    for kernel in KERNELS:
        for h in (1.0, 0.1, 0.01):
            assert np.all(oracle.kernel_flux3(kernel, a, b, c, x, h) == 0.0)
            assert oracle.kernel_antigrad_flux3(kernel, a, b, c, x, h) == 0.0


@pytest.mark.parametrize("kernel", KERNELS)
def test_antigrad_flux_on_the_triangle_plane(kernel):
    tri = np.eye(3)
    center = tri.mean(axis=0)
    for h in (1.0, 0.1, 0.01):
        for v in tri:
            assert abs(abs(oracle.kernel_antigrad_flux3(kernel, *tri, v, h)) - 1.0 / 12.0) < 1e-9
        for o in (0.9, 0.5, 0.1, 0.0, -0.1, -0.5, -0.9):
            t = 0.5 * (o + 1.0)
            for p, q in ((0, 1), (0, 2), (1, 2)):
                x = tri[p] + t * (tri[q] - tri[p])
                assert abs(abs(oracle.kernel_antigrad_flux3(kernel, *tri, x, h)) - 0.25) < 1e-9
            for p in range(3):
                x = tri[p] + t * (center - tri[p])
                assert abs(abs(oracle.kernel_antigrad_flux3(kernel, *tri, x, h)) - 0.5) < 1e-9
        for o in (1.0, 0.9, 0.5, 0.1):
            for p in range(3):
                d = np.full(3, -o)
                d[p] = 2.0 * o
                assert abs(oracle.kernel_antigrad_flux3(kernel, *tri, tri[p] + d, h)) < 1e-12


def test_triangle_sphere_overlap():
    a, b, c = np.array([0.0, 0, 0]), np.array([1.0, 0, 0]), np.array([0.0, 1, 0])
    # Closest points: the face, an edge, a vertex.
    assert oracle.triangle_in_sphere(a, b, c, np.array([0.2, 0.2, 0.5]), 0.5)
    assert not oracle.triangle_in_sphere(a, b, c, np.array([0.2, 0.2, 0.5]), 0.4999)
    assert oracle.triangle_in_sphere(a, b, c, np.array([0.5, -0.3, 0.4]), 0.5)
    assert not oracle.triangle_in_sphere(a, b, c, np.array([0.5, -0.3, 0.4]), 0.4999)
    assert oracle.triangle_in_sphere(a, b, c, np.array([-0.3, -0.4, 0.0]), 0.5)
    assert not oracle.triangle_in_sphere(a, b, c, np.array([-0.3, -0.4, 0.0]), 0.4999)
    assert oracle.triangle_in_sphere(a, b, c, np.array([0.8, 0.8, 0.0]), 0.5)
    # A degenerate triangle clamps to its longest edge.
    assert oracle.triangle_in_sphere(a, b, 0.5 * b, np.array([0.5, 0.3, 0.0]), 0.3)
    assert not oracle.triangle_in_sphere(a, b, 0.5 * b, np.array([0.5, 0.3, 0.0]), 0.2999)


def _box_mesh(lo, hi):
    """12 outward-oriented triangles of an axis-aligned box."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]])
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]
    tris = []
    for p, q, r, s in quads:
        tris += [(p, q, r), (p, r, s)]
    return v[np.array(tris)]


def test_winding_number_of_a_box():
    tris = _box_mesh((0.0, 0.0, 0.0), (2.0, 1.0, 1.5))
    rng = np.random.default_rng(3)
    for _ in range(200):
        x = rng.uniform(-1.0, 3.0, size=3)
        inside = bool(np.all(x > 0) and x[0] < 2.0 and x[1] < 1.0 and x[2] < 1.5)
        w = oracle.winding_number3(tris, x)
        assert abs(w - (1.0 if inside else 0.0)) < 1e-12
    # Flipping the orientation flips the sign.
    assert abs(oracle.winding_number3(tris[:, ::-1], np.array([1.0, 0.5, 0.5])) + 1.0) < 1e-12


def test_box_faces_close_the_pool():
    from titsolver_gb300 import scenarios
    verts, faces = scenarios.box_faces(2.0, 1.0, 1.5, 0.25)
    tris = verts[faces]
    # Inward normals: the faces wind -1 around interior points.
    assert abs(oracle.winding_number3(tris, np.array([1.0, 0.5, 0.7])) + 1.0) < 1e-12
    assert abs(oracle.winding_number3(tris, np.array([3.0, 0.5, 0.7]))) < 1e-12
    # Every edge is at most dx long and every edge is shared by two faces.
    edges = {}
    for f in faces:
        for p, q in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            assert np.linalg.norm(verts[p] - verts[q]) <= 0.25 * math.sqrt(2) + 1e-12
            edges[(p, q)] = edges.get((p, q), 0) + 1
    assert all(edges.get((q, p)) == 1 for (p, q) in edges)


def test_3d_face_scenario_steps():
    from titsolver_gb300 import physics, scenarios
    scn = scenarios.dam_break_3d_faces(nx_per_H=6, tank=(3.0, 1.5))
    st = oracle.State(scn)
    P = physics.reference_params(3)
    P.post_integrate = 1
    nf = scn["tanks"][0]["n_fluid"]
    oracle.step(P, st, 1)
    # The wall pressure carries most of the column's weight, and the
    # collapse starts towards +x; z is a symmetry plane up to the
    # triangulation's diagonals.
    mean = st.dv_dt[:nf].mean(axis=0)
    assert -0.5 * scenarios.G < mean[1] < 0.0
    assert mean[0] > 0.0
    assert abs(mean[2]) < 1e-3 * scenarios.G
    oracle.step(P, st, 9)
    assert np.all(np.isfinite(st.r)) and np.all(np.isfinite(st.rho))
    poly = scn["faces"][0]["poly"]
    assert all(oracle.winding_number3(poly, x) > 0.5 for x in st.r[:nf])
    assert st.r[:nf, 0].max() > scn["r"][:nf, 0].max()
    np.testing.assert_array_equal(st.r[nf:], scn["r"][nf:])


def test_triangle_geometry_known_answers():
    # geom/triangle.test.cpp: winding number of the unit-simplex face seen
    # from the origin (1/8 of the sphere), its flip, translation and scale;
    # the projection around the face centre; the closest points.
    a, b, c = np.eye(3)
    o = np.zeros(3)
    assert abs(oracle.winding_number3(np.array([[a, b, c]]), o) - 0.125) < 1e-14
    assert abs(oracle.winding_number3(np.array([[c, b, a]]), o) + 0.125) < 1e-14
    off = np.array([3.0, 4.0, 5.0])
    assert abs(oracle.winding_number3(np.array([[a + off, b + off, c + off]]), off) - 0.125) < 1e-14
    assert abs(oracle.winding_number3(np.array([[2 * a, 2 * b, 2 * c]]), o) - 0.125) < 1e-14
    s2, s3 = math.sqrt(2.0), math.sqrt(3.0)
    p = oracle.triangle_project(a, b, c, (a + b + c) / 3.0)
    np.testing.assert_allclose(p, [[-1 / s2, -1 / (s2 * s3)], [1 / s2, -1 / (s2 * s3)],
                                   [0.0, s2 / s3]], atol=1e-14)
    A, B, C = np.array([0.0, 0, 0]), np.array([2.0, 0, 0]), np.array([0.0, 2, 0])
    cases = [((-1, -1, 0), (0, 0, 0)), ((-0.5, -0.5, 5), (0, 0, 0)),
             ((3, -1, 0), (2, 0, 0)), ((2.5, -0.5, -3), (2, 0, 0)),
             ((-1, 3, 0), (0, 2, 0)), ((-0.5, 2.5, 2), (0, 2, 0)),
             ((1, -1, 0), (1, 0, 0)), ((0.5, -2, -1), (0.5, 0, 0)),
             ((-1, 1, 0), (0, 1, 0)), ((-2, 1.5, 4), (0, 1.5, 0)),
             ((2, 2, 0), (1, 1, 0)), ((1.5, 1.5, -2), (1, 1, 0)),
             ((0, 0, 0), (0, 0, 0)), ((2, 0, 0), (2, 0, 0)), ((0, 2, 0), (0, 2, 0)),
             ((0.5, 0.5, 0), (0.5, 0.5, 0)), ((1, 1, 1), (1, 1, 0)), ((1, 1, -1), (1, 1, 0))]
    for x, want in cases:
        np.testing.assert_allclose(oracle.triangle_clamp(A, B, C, np.array(x, float)), want,
                                   atol=1e-14)
    # Degenerate triangles clamp to their longest edge, or their one point.
    z, t = np.zeros(3), np.array([2.0, 2.0, 0.0])
    for tri in ((z, z, t), (z, t, t), (z, t, z), (z, np.array([1.0, 1.0, 0.0]), t)):
        for x, want in (((0, 0, 0), (0, 0, 0)), ((-1, -1, 0), (0, 0, 0)),
                        ((-1, -1, -1), (0, 0, 0)), ((2, 2, 0), (2, 2, 0)),
                        ((3, 3, 0), (2, 2, 0)), ((2, 2, 1), (2, 2, 0)),
                        ((1, 1, 0), (1, 1, 0)), ((0.9, 1.1, 0), (1, 1, 0)),
                        ((1.1, 0.9, 0), (1, 1, 0)), ((1.1, 0.9, 1), (1, 1, 0))):
            np.testing.assert_allclose(oracle.triangle_clamp(*tri, np.array(x, float)), want,
                                       atol=1e-14)
    for x in ((0, 0, 0), (1, 1, 1), (-1, -1, -1)):
        np.testing.assert_allclose(oracle.triangle_clamp(z, z, z, np.array(x, float)), z)
