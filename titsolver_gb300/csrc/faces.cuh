// faces.cuh - semi-analytical face boundaries in 2D (FP64 form): the
// reference's wall mode with boundary faces and a containment function
// (FluidEquations with a non-empty domain, fluid_equations.hpp:122-193,
// 241-247, 278-291, 340-349, 491-511).
//
// The tank's fixed particles are the face vertices.  Per prepare, k_gamma
// computes for every particle the kernel flux sum over its adjacent faces
// (grad gamma), the containment (winding number > 1/2, by signed crossings
// of the +x ray with the polygon edges of the particle's grid row), and
// gamma = contains - sum of antigradient fluxes at r + (2 contains - 1)
// n h^2 (fluid_equations.hpp:166-193).  The wall extrapolation, the force
// pass and the post-integration passes then read gamma and grad gamma and
// add the face terms.
//
// Kernel flux and antigradient flux of a segment (kernel.hpp:194-221,
// 286-314) are sums over the kernel's support pieces w_i(q) = sum_p c_p q^p
// (q < cutoff_i) of primitives in the along-segment coordinate z at wall
// distance eta (units of h):
//   flux:     sum_p c_p J_p;   antigrad: t_0 A + t_1 eta L + sum t_p eta J_{p-2}
// with rho^2 = z^2 + eta^2, A = atan2(z, eta), L = asinh(z/eta) (as
// copysign(log1p((|z| + z^2/(rho + eta))/eta), z)), J_0 = z,
// J_1 = (z rho + eta^2 L)/2, J_p = (z rho^p + p eta^2 J_{p-2})/(p + 1), and
// t_p the coefficients of the piece's 2D tail moment.
#pragma once

#include <cstddef>

#include "common.cuh"

namespace tg {

// Device view of the boundary faces of a context (all tanks); on = 0 when
// the tanks have particle walls.
struct FaceArgs {
  const double* seg;          // 4 per face: a.x, a.y, b.x, b.y
  const uint32_t* vert;       // 2 per face: upload indices of the vertices
  const uint32_t* cell_start; // per global cell (+1): its face list
  const uint32_t* cell_face;  // faces within reach of each cell, ascending
  const double* poly_edge;    // 4 per containment edge: x0, y0, x1, y1
  const uint32_t* row_start;  // per global grid row (+1): its edge list
  const uint32_t* row_edge;   // containment edges overlapping each row
  const uint32_t* row_off;    // per tank: first global grid row
  uint32_t* slot_of;          // upload index -> cell-order slot (walls)
  double* gamma;              // per particle, cell order
  double* ggam;               // grad gamma, 2 per particle
  double* face_drho;          // face terms of continuity, per particle
  double* face_dv;            // face terms of momentum, 2 per particle
  const uint32_t* tank_edges; // per tank: containment edges (0: all inside)
  double weight;              // the kernel's 2D weight
  int on;
};

struct FacePiece {
  double cutoff;
  int deg;
  double c[12];
  int tdeg;
  double t[14];
};
struct FacePieces {
  int n;
  FacePiece p[3];
};

// Support pieces of the six kernels (kernel.gen.cpp:520-553), expanded.
static __constant__ FacePieces c_face_pieces[6] = {
  // cubic spline
  {2, {{2.0, 3, {2.0, -3.0, 3.0 / 2.0, -1.0 / 4.0}, 5, {2.0 / 5.0, 0.0, -1.0, 1.0, -3.0 / 8.0, 1.0 / 20.0}},
   {1.0, 3, {-1.0, 3.0, -3.0, 1.0}, 5, {-1.0 / 20.0, 0.0, 1.0 / 2.0, -1.0, 3.0 / 4.0, -1.0 / 5.0}}}},
  // quartic spline
  {3, {{5.0 / 2.0, 4, {625.0 / 16.0, -125.0 / 2.0, 75.0 / 2.0, -10.0, 1.0}, 6, {3125.0 / 384.0, 0.0, -625.0 / 32.0, 125.0 / 6.0, -75.0 / 8.0, 2.0, -1.0 / 6.0}},
   {3.0 / 2.0, 4, {-405.0 / 16.0, 135.0 / 2.0, -135.0 / 2.0, 30.0, -5.0}, 6, {-243.0 / 128.0, 0.0, 405.0 / 32.0, -45.0 / 2.0, 135.0 / 8.0, -6.0, 5.0 / 6.0}},
   {1.0 / 2.0, 4, {5.0 / 8.0, -5.0, 15.0, -20.0, 10.0}, 6, {1.0 / 192.0, 0.0, -5.0 / 16.0, 5.0 / 3.0, -15.0 / 4.0, 4.0, -5.0 / 3.0}}}},
  // quintic spline
  {3, {{3.0, 5, {243.0, -405.0, 270.0, -90.0, 15.0, -1.0}, 7, {729.0 / 14.0, 0.0, -243.0 / 2.0, 135.0, -135.0 / 2.0, 18.0, -5.0 / 2.0, 1.0 / 7.0}},
   {2.0, 5, {-192.0, 480.0, -480.0, 240.0, -60.0, 6.0}, 7, {-128.0 / 7.0, 0.0, 96.0, -160.0, 120.0, -48.0, 10.0, -6.0 / 7.0}},
   {1.0, 5, {15.0, -75.0, 150.0, -150.0, 75.0, -15.0}, 7, {5.0 / 14.0, 0.0, -15.0 / 2.0, 25.0, -75.0 / 2.0, 30.0, -25.0 / 2.0, 15.0 / 7.0}}}},
  // Wendland C2
  {1, {{2.0, 5, {1.0, 0.0, -5.0 / 2.0, 5.0 / 2.0, -15.0 / 16.0, 1.0 / 8.0}, 7, {2.0 / 7.0, 0.0, -1.0 / 2.0, 0.0, 5.0 / 8.0, -1.0 / 2.0, 5.0 / 32.0, -1.0 / 56.0}}}},
  // Wendland C4
  {1, {{2.0, 8, {1.0, 0.0, -7.0 / 3.0, 0.0, 35.0 / 8.0, -14.0 / 3.0, 35.0 / 16.0, -1.0 / 2.0, 35.0 / 768.0}, 10, {2.0 / 9.0, 0.0, -1.0 / 2.0, 0.0, 7.0 / 12.0, 0.0, -35.0 / 48.0, 2.0 / 3.0, -35.0 / 128.0, 1.0 / 18.0, -7.0 / 1536.0}}}},
  // Wendland C6
  {1, {{2.0, 11, {1.0, 0.0, -11.0 / 4.0, 0.0, 33.0 / 8.0, 0.0, -231.0 / 32.0, 33.0 / 4.0, -1155.0 / 256.0, 11.0 / 8.0, -231.0 / 1024.0, 1.0 / 64.0}, 13, {7.0 / 39.0, 0.0, -1.0 / 2.0, 0.0, 11.0 / 16.0, 0.0, -11.0 / 16.0, 0.0, 231.0 / 256.0, -11.0 / 12.0, 231.0 / 512.0, -1.0 / 8.0, 77.0 / 4096.0, -1.0 / 832.0}}}},
};

constexpr double kTiny = 6.0554544523933395e-06;

__device__ __forceinline__ void face_line_integrals(double eta, double z,
                                                    double rho, double L,
                                                    int pmax, double* J) {
  J[0] = z;
  if (pmax >= 1) J[1] = (z * rho + eta * eta * L) / 2.0;
  double rp = rho;
  for (int p = 2; p <= pmax; ++p) {
    rp *= rho;
    J[p] = (z * rp + p * eta * eta * J[p - 2]) / (p + 1);
  }
}

__device__ __forceinline__ double face_primitive(const FacePiece& kp,
                                                 bool antigrad, double eta,
                                                 double z) {
  const double rho = sqrt(z * z + eta * eta);
  const double A = atan2(z, eta);
  const double L = fabs(eta) <= kTiny
                       ? 0.0
                       : copysign(log1p((fabs(z) + z * z / (rho + eta)) / eta), z);
  double J[14];
  double s = 0.0;
  if (!antigrad) {
    face_line_integrals(eta, z, rho, L, kp.deg, J);
    for (int p = 0; p <= kp.deg; ++p) s += kp.c[p] * J[p];
    return s;
  }
  face_line_integrals(eta, z, rho, L, max(kp.tdeg - 2, 0), J);
  for (int p = 0; p <= kp.tdeg; ++p) {
    if (p == 0) s += kp.t[0] * A;
    else if (p == 1) s += kp.t[1] * eta * L;
    else s += kp.t[p] * eta * J[p - 2];
  }
  return s;
}

template<int K>
__device__ __forceinline__ double face_unit_segment(bool antigrad, double eta,
                                                    double zmin, double zmax) {
  const FacePieces& P = c_face_pieces[K];
  double total = 0.0;
  for (int i = 0; i < P.n; ++i) {
    const FacePiece& kp = P.p[i];
    if (eta >= kp.cutoff) continue;
    const double zc = sqrt(kp.cutoff * kp.cutoff - eta * eta);
    const double lo = fmax(zmin, -zc), hi = fmin(zmax, zc);
    if (lo >= hi) continue;
    total += face_primitive(kp, antigrad, eta, hi) -
             face_primitive(kp, antigrad, eta, lo);
  }
  return total;
}

// normalize() with the |a|^2 >= tiny^2 guard (core/_vec/vec.hpp:663-676).
__device__ __forceinline__ void normalize2(const double* a, double* out) {
  const double n2 = a[0] * a[0] + a[1] * a[1];
  const double s = n2 >= kTiny * kTiny ? 1.0 / sqrt(n2) : 0.0;
  out[0] = a[0] * s;
  out[1] = a[1] * s;
}

struct FaceFrame {
  double n[2], d, za, zb;
};

// Segment frame at x: unit normal cross(b - a) = (y, -x) normalised, signed
// distance d and projections of the endpoints (units of h).
__device__ __forceinline__ FaceFrame face_frame(const double* ab,
                                                const double* x, double hinv) {
  const double ba[2] = {ab[2] - ab[0], ab[3] - ab[1]};
  const double cr[2] = {ba[1], -ba[0]};
  FaceFrame F;
  normalize2(cr, F.n);
  double e[2];
  normalize2(ba, e);
  F.d = ((x[0] - ab[0]) * F.n[0] + (x[1] - ab[1]) * F.n[1]) * hinv;
  F.za = ((ab[0] - x[0]) * e[0] + (ab[1] - x[1]) * e[1]) * hinv;
  F.zb = ((ab[2] - x[0]) * e[0] + (ab[3] - x[1]) * e[1]) * hinv;
  return F;
}

// Kernel::flux (kernel.hpp:194-206): n w h^-1 unit_flux(|d|, z_a, z_b);
// wd = the kernel's 2D weight.
template<int K>
__device__ __forceinline__ void face_flux(const double* ab, const double* x,
                                          double h, double wd, double* out) {
  const double hinv = 1.0 / h;
  const FaceFrame F = face_frame(ab, x, hinv);
  const double s = wd * hinv * face_unit_segment<K>(false, fabs(F.d), F.za, F.zb);
  out[0] = F.n[0] * s;
  out[1] = F.n[1] * s;
}

// Kernel::antigrad_flux (kernel.hpp:209-221).
template<int K>
__device__ __forceinline__ double face_antigrad_flux(const double* ab,
                                                     const double* x, double h,
                                                     double wd) {
  const FaceFrame F = face_frame(ab, x, 1.0 / h);
  return copysign(wd, F.d) * face_unit_segment<K>(true, fabs(F.d), F.za, F.zb);
}

// Segment::intersects(BSphere) (geom/segment.hpp:108-112).
__device__ __forceinline__ bool face_in_sphere(const double* ab,
                                               const double* c, double radius) {
  for (int k = 0; k < 2; ++k) {
    const double lo = fmin(ab[k], ab[2 + k]), hi = fmax(ab[k], ab[2 + k]);
    if (!(c[k] - radius <= hi && lo <= c[k] + radius)) return false;
  }
  const double ba[2] = {ab[2] - ab[0], ab[3] - ab[1]};
  const double len2 = ba[0] * ba[0] + ba[1] * ba[1];
  double q[2] = {ab[0], ab[1]};
  if (!(len2 <= kTiny)) {
    const double t = ((c[0] - ab[0]) * ba[0] + (c[1] - ab[1]) * ba[1]) / len2;
    if (t > 1.0) {
      q[0] = ab[2];
      q[1] = ab[3];
    } else if (!(t < 0.0)) {
      q[0] = ab[0] + t * ba[0];
      q[1] = ab[1] + t * ba[1];
    }
  }
  const double d0 = q[0] - c[0], d1 = q[1] - c[1];
  return d0 * d0 + d1 * d1 <= radius * radius;
}

// Faces within the support radius of x, in ascending face order (the
// particle's cell list holds every face within reach of the cell).
template<class Fn>
__device__ __forceinline__ void for_adjacent_faces(const FaceArgs& fc,
                                                   uint32_t gcell,
                                                   const double* x,
                                                   double radius, Fn&& fn) {
  const uint32_t s = fc.cell_start[gcell], e = fc.cell_start[gcell + 1];
  for (uint32_t i = s; i < e; ++i) {
    const uint32_t f = fc.cell_face[i];
    const double* ab = fc.seg + 4 * static_cast<size_t>(f);
    if (face_in_sphere(ab, x, radius)) fn(f, ab);
  }
}

// Winding number > 1/2 by signed crossings of the ray from x towards +x
// with the containment edges that overlap x's grid row.
__device__ __forceinline__ bool face_contains(const FaceArgs& fc, uint32_t tank,
                                              uint32_t grow, const double* x) {
  if (fc.tank_edges[tank] == 0) return true;  // a tank with particle walls
  int w = 0;
  for (uint32_t i = fc.row_start[grow]; i < fc.row_start[grow + 1]; ++i) {
    const double* e = fc.poly_edge + 4 * static_cast<size_t>(fc.row_edge[i]);
    const double y0 = e[1], y1 = e[3];
    if (y0 <= x[1] && x[1] < y1) {
      const double xc = e[0] + (x[1] - y0) * (e[2] - e[0]) / (y1 - y0);
      if (xc > x[0]) ++w;
    } else if (y1 <= x[1] && x[1] < y0) {
      const double xc = e[0] + (x[1] - y0) * (e[2] - e[0]) / (y1 - y0);
      if (xc > x[0]) --w;
    }
  }
  return w >= 1;
}

}  // namespace tg
