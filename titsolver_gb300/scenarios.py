"""Seeded synthetic scenarios of the WCSPH hot path.

Each generator returns a dict with ``tanks`` (list of tank dicts: n_fluid,
n_wall, h, m, rho0, cs0) and AoS arrays ``r``, ``v``, ``rho`` in upload
order (tank after tank, fluid then walls), plus descriptive metadata.

* ``dam_break_2d``: the titwcsph setup (source/titwcsph/wcsph.cpp:37-142):
  fluid at dx * (i + 1, j + 1), i outer, j inner; h = 2 dx, m = rho0 dx^2,
  hydrostatic density from the 50-term series of wcsph.cpp:129-141.  The tank
  is W x Ht with three layers of fixed wall particles on the dx lattice
  (bottom and both sides; open top); W is rounded to a whole number of dx.
* ``dam_break_3d``: the same in 3D (y vertical), column L x H x depth, tank
  W x Ht x (depth + dx) with walls on every side but the top, h = 1.3 dx.
* ``cloud_3d``: jittered lattice plus Gaussian clusters in the unit box.
* ``batched_tanks``: many independent 2D dam breaks of random size.
"""

from __future__ import annotations

import math

import numpy as np

G = 9.81
RHO0 = 1000.0


def hydrostatic_pressure(x: np.ndarray, y: np.ndarray, H: float, L: float,
                         g: float = G, rho0: float = RHO0) -> np.ndarray:
    """Dam-break initial pressure of wcsph.cpp:130-138 (odd k < 100).  Each
    term of the series is a function of x times a function of y, so on a
    lattice the series is evaluated once per (distinct x, distinct y) pair
    and gathered: the same arithmetic per point, far fewer evaluations."""
    ux, ix = np.unique(x, return_inverse=True)
    uy, iy = np.unique(y, return_inverse=True)
    if ux.size * uy.size < x.size:
        table = _hydrostatic_series(ux[:, None], uy[None, :], H, L, g, rho0)
        return table[ix.ravel(), iy.ravel()]
    return _hydrostatic_series(x, y, H, L, g, rho0)


def _hydrostatic_series(x, y, H: float, L: float, g: float, rho0: float):
    p = rho0 * g * (H - y)
    for k in range(1, 100, 2):
        k_pi = k * math.pi
        p = p - 8.0 * rho0 * g * H / (k_pi * k_pi) * (
            np.exp(k_pi * (x - L) / (2.0 * H)) * np.cos(k_pi * y / (2.0 * H)))
    return p


def _walls_2d(nW: int, nH: int, layers: int, dx: float) -> np.ndarray:
    """Lattice points (i dx, j dx), -layers < i < nW + layers, -layers < j <= nH,
    that lie in the wall band (i <= 0, i >= nW or j <= 0); ordered by (j, i)."""
    js, is_ = np.meshgrid(np.arange(-(layers - 1), nH + 1),
                          np.arange(-(layers - 1), nW + layers), indexing="ij")
    js = js.ravel()
    is_ = is_.ravel()
    band = (is_ <= 0) | (is_ >= nW) | (js <= 0)
    return np.stack([dx * is_[band].astype(np.float64),
                     dx * js[band].astype(np.float64)], axis=1)


def dam_break_2d(H: float = 1.0, nx_per_H: int = 80, column=(2.0, 1.0),
                 tank=(5.366, 3.0), layers: int = 3, cs0_factor: float = 10.0,
                 g: float = G, rho0: float = RHO0, hydrostatic: bool = True) -> dict:
    dx = H / nx_per_H
    L = column[0] * H
    M = int(round(L / dx))
    N = int(round(column[1] * H / dx))
    i, j = np.meshgrid(np.arange(M), np.arange(N), indexing="ij")  # i outer
    fluid = np.stack([dx * (i.ravel() + 1.0), dx * (j.ravel() + 1.0)], axis=1)
    nW = int(round(tank[0] * H / dx))
    nH = int(round(tank[1] * H / dx))
    walls = _walls_2d(nW, nH, layers, dx)
    cs0 = cs0_factor * math.sqrt(g * H)
    rho_f = np.full(fluid.shape[0], rho0)
    if hydrostatic:
        p = hydrostatic_pressure(fluid[:, 0], fluid[:, 1], H, L, g, rho0)
        rho_f = rho0 + p / (cs0 * cs0)
    r = np.concatenate([fluid, walls])
    rho = np.concatenate([rho_f, np.full(walls.shape[0], rho0)])
    tank_d = dict(n_fluid=fluid.shape[0], n_wall=walls.shape[0], h=2.0 * dx,
                  m=rho0 * dx * dx, rho0=rho0, cs0=cs0)
    return dict(dim=2, tanks=[tank_d], r=r, v=np.zeros_like(r), rho=rho, dx=dx,
                H=H, width=nW * dx, name=f"dam_break_2d_H{H}_dx1/{nx_per_H}")


def rectangle_faces(width: float, height: float, dx: float):
    """The titwcsph domain (source/titwcsph/wcsph.cpp:55-65): a rectangle
    with vertices (0, Ht), (W, Ht), (W, 0), (0, 0) and faces 0-1, 1-2, 2-3,
    3-0, tessellated as geom::tessellate does (geom/tessellation.hpp:30-60:
    the original vertices first, then each face split into
    max(1, ceil(len / dx)) pieces with the new vertices appended in order).
    Returns (vertices (n, 2), faces (m, 2))."""
    verts = [(0.0, height), (width, height), (width, 0.0), (0.0, 0.0)]
    faces_in = [(0, 1), (1, 2), (2, 3), (3, 0)]
    out_v = list(verts)
    out_f = []
    for a, b in faces_in:
        pa, pb = np.array(verts[a]), np.array(verts[b])
        length = float(np.hypot(*(pb - pa)))
        n = max(1, int(math.ceil(length / dx)))
        prev = a
        for i in range(1, n):
            t = i / n
            out_v.append(tuple(pa + t * (pb - pa)))
            out_f.append((prev, len(out_v) - 1))
            prev = len(out_v) - 1
        out_f.append((prev, b))
    return np.array(out_v, dtype=np.float64), np.array(out_f, dtype=np.int32)


def dam_break_2d_faces(nx_per_H: int = 80, H: float = 0.6, g: float = G,
                       rho0: float = RHO0) -> dict:
    """The titwcsph scenario itself (source/titwcsph/wcsph.cpp:37-142):
    H = 0.6, column 2H x H at dr (i + 1, j + 1), pool 5.366H x 4H whose
    tessellated boundary faces carry one fixed particle per vertex,
    cs0 = 20 sqrt(gH), h = 2 dr, m = rho0 dr^2, hydrostatic density; the
    containment polygon is the pool rectangle counter-clockwise (domain2 of
    wcsph.cpp:67-77).  Returns a scenario with "faces"."""
    dx = H / nx_per_H
    L = 2.0 * H
    M = int(round(L / dx))
    N = int(round(H / dx))
    i, j = np.meshgrid(np.arange(M), np.arange(N), indexing="ij")
    fluid = np.stack([dx * (i.ravel() + 1.0), dx * (j.ravel() + 1.0)], axis=1)
    W, Ht = 5.366 * H, 4.0 * H
    walls, faces = rectangle_faces(W, Ht, dx)
    cs0 = 20.0 * math.sqrt(g * H)
    p = hydrostatic_pressure(fluid[:, 0], fluid[:, 1], H, L, g, rho0)
    rho_f = rho0 + p / (cs0 * cs0)
    r = np.concatenate([fluid, walls])
    rho = np.concatenate([rho_f, np.full(walls.shape[0], rho0)])
    tank = dict(n_fluid=fluid.shape[0], n_wall=walls.shape[0], h=2.0 * dx,
                m=rho0 * dx * dx, rho0=rho0, cs0=cs0)
    poly = np.array([(0.0, 0.0), (W, 0.0), (W, Ht), (0.0, Ht)])
    return dict(dim=2, tanks=[tank], r=r, v=np.zeros_like(r), rho=rho, dx=dx, H=H,
                faces=[dict(face_verts=faces, poly=poly)],
                name=f"titwcsph_faces_dx=H/{nx_per_H}")


def dam_break_3d(H: float = 1.0, nx_per_H: int = 200, column=(2.0, 1.0, 1.0),
                 tank=(5.366, 3.0), layers: int = 3, cs0_factor: float = 10.0,
                 h_factor: float = 1.3, g: float = G, rho0: float = RHO0) -> dict:
    dx = H / nx_per_H
    L = column[0] * H
    M = int(round(L / dx))
    N = int(round(column[1] * H / dx))
    K = int(round(column[2] * H / dx))
    i, j, k = np.meshgrid(np.arange(M), np.arange(N), np.arange(K), indexing="ij")
    fluid = np.stack([dx * (i.ravel() + 1.0), dx * (j.ravel() + 1.0),
                      dx * (k.ravel() + 1.0)], axis=1)
    nW = int(round(tank[0] * H / dx))
    nH = int(round(tank[1] * H / dx))
    nZ = K + 1  # side walls at z = 0 and z = (K + 1) dx
    zs = np.arange(-(layers - 1), nZ + layers)
    w2 = _walls_2d(nW, nH, layers, dx)  # (x, y) band of a z-slice
    slices = []
    # Interior z-slices carry the 2D band; the z-side slabs are full planes.
    ys_full, xs_full = np.meshgrid(np.arange(-(layers - 1), nH + 1),
                                   np.arange(-(layers - 1), nW + layers), indexing="ij")
    full = np.stack([dx * xs_full.ravel().astype(np.float64),
                     dx * ys_full.ravel().astype(np.float64)], axis=1)
    for z in zs:
        plane = full if (z <= 0 or z >= nZ) else w2
        slices.append(np.concatenate([plane, np.full((plane.shape[0], 1), dx * z)], axis=1))
    walls = np.concatenate(slices)
    cs0 = cs0_factor * math.sqrt(g * H)
    p = hydrostatic_pressure(fluid[:, 0], fluid[:, 1], H, L, g, rho0)
    rho_f = rho0 + p / (cs0 * cs0)
    r = np.concatenate([fluid, walls])
    rho = np.concatenate([rho_f, np.full(walls.shape[0], rho0)])
    tank_d = dict(n_fluid=fluid.shape[0], n_wall=walls.shape[0], h=h_factor * dx,
                  m=rho0 * dx ** 3, rho0=rho0, cs0=cs0)
    return dict(dim=3, tanks=[tank_d], r=r, v=np.zeros_like(r), rho=rho, dx=dx,
                H=H, name=f"dam_break_3d_H{H}_dx1/{nx_per_H}")


def box_mesh(lo, hi) -> np.ndarray:
    """The 12 outward-oriented triangles (12, 3, 3) of an axis-aligned box:
    a containment surface whose winding number is 1 inside."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], dtype=np.float64)
    quads = [(0, 3, 2, 1), (4, 5, 6, 7), (0, 1, 5, 4), (2, 3, 7, 6), (1, 2, 6, 5), (0, 4, 7, 3)]
    tris = []
    for a, b, c, d in quads:
        tris += [(a, b, c), (a, c, d)]
    return v[np.array(tris)]


def box_faces(width: float, height: float, depth: float, dx: float):
    """Boundary faces of the box [0, W] x [0, Ht] x [0, D]: each side split
    into a grid of max(1, ceil(len / dx)) intervals per axis, each cell into
    two triangles, normals cross(b - a, c - a) pointing into the box (as the
    2D pool's faces do); vertices shared between sides.  Returns
    (vertices (n, 3), faces (m, 3))."""
    ext = (width, height, depth)
    n = [max(1, int(math.ceil(e / dx))) for e in ext]
    index: dict = {}
    verts = []

    def vid(ijk):
        if ijk not in index:
            index[ijk] = len(verts)
            verts.append(tuple(ext[k] * ijk[k] / n[k] for k in range(3)))
        return index[ijk]

    faces = []
    # (fixed axis, fixed side, u axis, v axis) with cross(u, v) inward.
    sides = [(1, 0, 2, 0), (1, 1, 0, 2), (0, 0, 1, 2), (0, 1, 2, 1), (2, 0, 0, 1), (2, 1, 1, 0)]
    for ax, side, u, v in sides:
        for i in range(n[u]):
            for j in range(n[v]):
                def corner(di, dj):
                    ijk = [0, 0, 0]
                    ijk[ax] = side * n[ax]
                    ijk[u] = i + di
                    ijk[v] = j + dj
                    return vid(tuple(ijk))
                p00, p10, p01, p11 = corner(0, 0), corner(1, 0), corner(0, 1), corner(1, 1)
                faces += [(p00, p10, p11), (p00, p11, p01)]
    return np.array(verts, dtype=np.float64), np.array(faces, dtype=np.int32)


def dam_break_3d_faces(nx_per_H: int = 80, H: float = 0.6, column=(2.0, 1.0, 1.0),
                       tank=(5.366, 4.0), h_factor: float = 1.3, g: float = G,
                       rho0: float = RHO0, face_refine: int = 1) -> dict:
    """The titwcsph scenario extruded to 3D with triangle faces: column
    column * H at dr (i + 1, j + 1, k + 1), pool tank[0] H x tank[1] H x
    (K + 1) dr whose triangulated sides (box_faces at dr / face_refine) carry
    one fixed particle per vertex, cs0 = 20 sqrt(gH), h = h_factor dr,
    m = rho0 dr^3, hydrostatic density; the containment is the pool box
    (box_mesh)."""
    dx = H / nx_per_H
    L = column[0] * H
    M = int(round(L / dx))
    N = int(round(column[1] * H / dx))
    K = int(round(column[2] * H / dx))
    i, j, k = np.meshgrid(np.arange(M), np.arange(N), np.arange(K), indexing="ij")
    fluid = np.stack([dx * (i.ravel() + 1.0), dx * (j.ravel() + 1.0),
                      dx * (k.ravel() + 1.0)], axis=1)
    W, Ht, D = tank[0] * H, tank[1] * H, (K + 1) * dx
    walls, faces = box_faces(W, Ht, D, dx / face_refine)
    cs0 = 20.0 * math.sqrt(g * H)
    p = hydrostatic_pressure(fluid[:, 0], fluid[:, 1], H, L, g, rho0)
    rho_f = rho0 + p / (cs0 * cs0)
    r = np.concatenate([fluid, walls])
    rho = np.concatenate([rho_f, np.full(walls.shape[0], rho0)])
    tank_d = dict(n_fluid=fluid.shape[0], n_wall=walls.shape[0], h=h_factor * dx,
                  m=rho0 * dx ** 3, rho0=rho0, cs0=cs0)
    return dict(dim=3, tanks=[tank_d], r=r, v=np.zeros_like(r), rho=rho, dx=dx, H=H,
                faces=[dict(face_verts=faces, poly=box_mesh((0.0, 0.0, 0.0), (W, Ht, D)))],
                name=f"dam_break_3d_faces_dx=H/{nx_per_H}")


def cloud_3d(n_total: int = 4_000_000, lattice_fraction: float = 0.7,
             n_clusters: int = 8, sigma: float = 0.05, jitter: float = 0.25,
             h_factor: float = 1.3, seed: int = 20261203, rho0: float = RHO0) -> dict:
    """Point cloud in [0, 1]^3: a jittered n^3 lattice (n^3 ~ 70% of n_total,
    spacing dx = 1/n, jitter U(-jitter dx, +jitter dx) per axis) plus
    n_clusters isotropic Gaussian clusters (sigma, centres U[0.15, 0.85]^3),
    rejection-sampled into the unit box.  h = 1.3 dx, m = rho0 dx^3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = int(round((lattice_fraction * n_total) ** (1.0 / 3.0)))
    dx = 1.0 / n
    g = (np.arange(n) + 0.5) * dx
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    lat = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    lat += rng.uniform(-jitter * dx, jitter * dx, size=lat.shape)
    n_rest = n_total - lat.shape[0]
    per = n_rest // n_clusters
    parts = [lat]
    for c in range(n_clusters):
        centre = rng.uniform(0.15, 0.85, size=3)
        want = per + (n_rest - per * n_clusters if c == n_clusters - 1 else 0)
        got = []
        have = 0
        while have < want:
            pts = centre + sigma * rng.standard_normal(size=(2 * (want - have) + 16, 3))
            pts = pts[np.all((pts >= 0.0) & (pts <= 1.0), axis=1)]
            got.append(pts[: want - have])
            have += got[-1].shape[0]
        parts.append(np.concatenate(got))
    r = np.ascontiguousarray(np.concatenate(parts))
    tank_d = dict(n_fluid=r.shape[0], n_wall=0, h=h_factor * dx, m=rho0 * dx ** 3,
                  rho0=rho0, cs0=1.0)
    return dict(dim=3, tanks=[tank_d], r=r, v=np.zeros_like(r),
                rho=np.full(r.shape[0], rho0), dx=dx, lattice_n=n, seed=seed,
                name=f"cloud_3d_{r.shape[0]}")


def batched_tanks(n_tanks: int = 512, nx_per_unit: int = 80, n_range=(20, 120),
                  aspect_range=(0.5, 2.0), seed: int = 20261203, layers: int = 3,
                  cs0_factor: float = 10.0, g: float = G, rho0: float = RHO0) -> dict:
    """Independent 2D dam breaks: column height N ~ U{n_range} particles,
    width round(a N) with a ~ U[aspect_range], spacing dx = 1/nx_per_unit,
    H = N dx, tank 5.366 H x 3 H with 3 wall layers, cs0 = 10 sqrt(g H)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dx = 1.0 / nx_per_unit
    tanks, rs, rhos = [], [], []
    for _ in range(n_tanks):
        N = int(rng.integers(n_range[0], n_range[1] + 1))
        a = float(rng.uniform(*aspect_range))
        M = max(1, int(round(a * N)))
        H = N * dx
        i, j = np.meshgrid(np.arange(M), np.arange(N), indexing="ij")
        fluid = np.stack([dx * (i.ravel() + 1.0), dx * (j.ravel() + 1.0)], axis=1)
        nW = max(int(round(5.366 * N)), M + 2)
        nH = 3 * N
        walls = _walls_2d(nW, nH, layers, dx)
        cs0 = cs0_factor * math.sqrt(g * H)
        p = hydrostatic_pressure(fluid[:, 0], fluid[:, 1], H, M * dx, g, rho0)
        rhos.append(np.concatenate([rho0 + p / (cs0 * cs0), np.full(walls.shape[0], rho0)]))
        rs.append(np.concatenate([fluid, walls]))
        tanks.append(dict(n_fluid=fluid.shape[0], n_wall=walls.shape[0], h=2.0 * dx,
                          m=rho0 * dx * dx, rho0=rho0, cs0=cs0))
    r = np.ascontiguousarray(np.concatenate(rs))
    return dict(dim=2, tanks=tanks, r=r, v=np.zeros_like(r), rho=np.concatenate(rhos),
                dx=dx, seed=seed, name=f"batched_{n_tanks}_tanks")


def batched_tanks_3d(n_tanks: int = 64, nx_per_unit: int = 100, n_range=(12, 40),
                     aspect_range=(0.5, 2.0), seed: int = 20261204, layers: int = 3,
                     cs0_factor: float = 10.0, h_factor: float = 1.3, g: float = G,
                     rho0: float = RHO0) -> dict:
    """Independent 3D dam breaks: column height N ~ U{n_range} particles,
    length round(a N) and depth round(b N) with a, b ~ U[aspect_range],
    spacing dx = 1/nx_per_unit, H = N dx; each tank is dam_break_3d's layout
    (tank 5.366 H x 3 H x (depth + dx), 3 wall layers, h = 1.3 dx)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dx = 1.0 / nx_per_unit
    tanks, rs, rhos = [], [], []
    for _ in range(n_tanks):
        N = int(rng.integers(n_range[0], n_range[1] + 1))
        a = float(rng.uniform(*aspect_range))
        b = float(rng.uniform(*aspect_range))
        H = N * dx
        one = dam_break_3d(H=H, nx_per_H=N, column=(max(1, round(a * N)) / N,
                                                    1.0, max(1, round(b * N)) / N),
                           layers=layers, cs0_factor=cs0_factor, h_factor=h_factor,
                           g=g, rho0=rho0)
        tanks.extend(one["tanks"])
        rs.append(one["r"])
        rhos.append(one["rho"])
    r = np.ascontiguousarray(np.concatenate(rs))
    return dict(dim=3, tanks=tanks, r=r, v=np.zeros_like(r), rho=np.concatenate(rhos),
                dx=dx, seed=seed, name=f"batched_3d_{n_tanks}_tanks")


def n_fluid(scn: dict) -> int:
    return int(sum(t["n_fluid"] for t in scn["tanks"]))
