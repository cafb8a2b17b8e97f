// faces.cuh - semi-analytical face boundaries: the reference's wall mode with boundary faces and a containment function
// (FluidEquations with a non-empty domain, fluid_equations.hpp:122-193,
// 241-247, 278-291, 340-349, 491-511); segments in 2D, triangles in 3D.
//
// The tank's fixed particles are the face vertices.  Per prepare,
// k_gamma_init / k_gamma_faces compute for every particle the kernel flux
// sum over its adjacent faces (grad gamma), the containment (winding
// number > 1/2: in 2D by signed crossings of the +x ray with the polygon
// edges of the particle's grid row; in 3D from the particle's cell when the
// containment surface does not reach that cell, else by the exact winding
// number of the surface's triangles), and gamma = contains - sum of
// antigradient fluxes at r + (2 contains - 1) n h^2
// (fluid_equations.hpp:166-193).  The wall extrapolation, the force pass
// and the post-integration passes then read gamma and grad gamma and add
// the face terms.
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
//
// Arithmetic: face selection, containment, the face frames and the sums over
// faces are FP64 in both forms.  The closed-form integrals of one face run
// in the type T of their template: FP64 in the plain form and FP32 in the
// compensated form, on the face's vertices already projected into its frame
// around the particle and scaled by 1/h (O(1) values, so FP32 keeps ~1e-7
// relative to h); GB300's FP64 rate is a small fraction of its FP32 rate.
#pragma once

#include <cstddef>
#include <type_traits>

#include "common.cuh"

namespace tg {

// Device view of the boundary faces of a context (all tanks); on = 0 when
// the tanks have particle walls.
struct FaceArgs {
  const double* coords;       // D * D per face: the vertices a, b (, c)
  // Per face its frame (k_face_frames): 2D the unit normal and tangent (4);
  // 3D the unit normal n and the in-plane axes e1, e2 (9).
  const double* frame;
  // Per face the coplanar neighbour across each edge (3D: ab, bc, ca;
  // shares the edge, traversed the other way, same plane and normal) or the
  // collinear neighbour across each end (2D: a, b; the segment ending at a
  // / starting at b on the same line, same direction), or -1.  An edge or
  // end whose neighbour is also within reach cancels against it.
  const int32_t* edge_nbr;
  const uint32_t* vert;       // D per face: upload indices of the vertices
  const uint32_t* cell_start; // per global cell (+1): its face list
  const uint32_t* cell_face;  // faces within reach of each cell, ascending
  // 2D containment: the polygon's edges by grid row.
  const double* poly_edge;    // 4 per containment edge: x0, y0, x1, y1
  const uint32_t* row_start;  // per global grid row (+1): its edge list
  const uint32_t* row_edge;   // containment edges overlapping each row
  const uint32_t* row_off;    // per tank: first global grid row
  // 3D containment: per-cell answers and the surface's triangles.
  const int8_t* cell_state;   // per global cell: 1 inside, 0 outside,
                              // -1 reached by the surface (exact test)
  const double* cont_tri;     // 9 per containment triangle
  const uint32_t* cont_start; // per tank (+1): its containment triangles
  uint32_t* slot_of;          // upload index -> cell-order slot (walls)
  uint32_t* face_list;        // particles (cell order) whose cell lists faces
  uint32_t* face_count;       // entries of face_list (this prepare)
  double* gamma;              // per particle, cell order
  double* ggam;               // grad gamma, D per particle
  double* face_drho;          // face terms of continuity, per particle
  double* face_dv;            // face terms of momentum, D per particle
  double* post_face;          // face terms of the shifting sums per
                              // particle: N, L, grad v, grad rho
  const uint32_t* tank_edges; // per tank: containment edges or triangles
                              // (0: particle walls, all inside)
  double weight;              // the kernel's weight in D dimensions
  int on;
};

// Block size of the warp-per-face-particle passes (their shared queues are
// sized by it).
constexpr int kFaceBlock = 128;

// Doubles per particle in FaceArgs::post_face.
template<int D>
constexpr int kPostFaceSums = 2 * D + 2 * D * D;

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
// Read at compile time only: the face integrals are unrolled per kernel and
// piece, with the coefficients as immediates.
inline constexpr FacePieces kFacePieces[6] = {
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

// 1/k for k = 0..17 (entry 0 unused): the recursions multiply by these
// instead of dividing (FP64 division is a long instruction sequence).
inline constexpr double kFaceInv[18] = {
    0.0, 1.0, 1.0 / 2.0, 1.0 / 3.0, 1.0 / 4.0, 1.0 / 5.0, 1.0 / 6.0, 1.0 / 7.0, 1.0 / 8.0,
    1.0 / 9.0, 1.0 / 10.0, 1.0 / 11.0, 1.0 / 12.0, 1.0 / 13.0, 1.0 / 14.0, 1.0 / 15.0,
    1.0 / 16.0, 1.0 / 17.0};

// x^n at compile time (n >= 0).
constexpr double constexpr_pow(double x, int n) {
  double r = 1.0;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// Compile-time loop: f.template operator()<B>() ... <E - 1>().
template<int B, int E, class Fn>
__device__ __forceinline__ void static_for(Fn&& f) {
  if constexpr (B < E) {
    f.template operator()<B>();
    static_for<B + 1, E>(f);
  }
}

// Scalar maths of the face integrals in their type: the float functions
// for T = float (no silent promotion to FP64), the double ones otherwise.
template<class T>
struct FaceMath;
template<>
struct FaceMath<double> {
  static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
  static __device__ __forceinline__ double abs(double x) { return ::fabs(x); }
  static __device__ __forceinline__ double min(double a, double b) { return ::fmin(a, b); }
  static __device__ __forceinline__ double max(double a, double b) { return ::fmax(a, b); }
  static __device__ __forceinline__ double atan2(double y, double x) { return ::atan2(y, x); }
  static __device__ __forceinline__ double log1p(double x) { return ::log1p(x); }
  static __device__ __forceinline__ double copysign(double a, double b) {
    return ::copysign(a, b);
  }
};
template<>
struct FaceMath<float> {
  static __device__ __forceinline__ float sqrt(float x) { return ::sqrtf(x); }
  static __device__ __forceinline__ float abs(float x) { return ::fabsf(x); }
  static __device__ __forceinline__ float min(float a, float b) { return ::fminf(a, b); }
  static __device__ __forceinline__ float max(float a, float b) { return ::fmaxf(a, b); }
  static __device__ __forceinline__ float atan2(float y, float x) { return ::atan2f(y, x); }
  static __device__ __forceinline__ float log1p(float x) { return ::log1pf(x); }
  static __device__ __forceinline__ float copysign(float a, float b) {
    return ::copysignf(a, b);
  }
};

// Segment line primitive of piece I of kernel K at z (units of h), with the
// J_p recursion and the coefficients unrolled.
template<int K, int I, bool Anti, class T>
__device__ __forceinline__ T face_primitive(T eta, T z) {
  using M = FaceMath<T>;
  constexpr FacePiece kp = kFacePieces[K].p[I];
  constexpr int pmax = Anti ? (kp.tdeg - 2 > 0 ? kp.tdeg - 2 : 0) : kp.deg;
  const T rho = M::sqrt(z * z + eta * eta);
  const T L = M::abs(eta) <= T(kTiny)
                  ? T(0)
                  : M::copysign(M::log1p((M::abs(z) + z * z / (rho + eta)) / eta), z);
  T J[pmax + 1];
  J[0] = z;
  if constexpr (pmax >= 1) J[1] = (z * rho + eta * eta * L) * T(0.5);
  T rp = rho;
  static_for<2, pmax + 1>([&]<int P>() {
    constexpr T inv = T(kFaceInv[P + 1]);
    rp *= rho;
    J[P] = (z * rp + T(P) * eta * eta * J[P - 2]) * inv;
  });
  T s = T(0);
  if constexpr (!Anti) {
    static_for<0, kp.deg + 1>([&]<int P>() {
      constexpr double c = kp.c[P];
      if constexpr (c != 0.0) s += T(c) * J[P];
    });
  } else {
    const T A = M::atan2(z, eta);
    static_for<0, kp.tdeg + 1>([&]<int P>() {
      constexpr double t = kp.t[P];
      if constexpr (t != 0.0) {
        if constexpr (P == 0) s += T(t) * A;
        else if constexpr (P == 1) s += T(t) * eta * L;
        else s += T(t) * eta * J[P - 2];
      }
    });
  }
  return s;
}

// unit_segment_integral (kernel.hpp:286-314) summed over the pieces: per
// piece P(clip(z_max)) - P(clip(z_min)), clip to |z| <= sqrt(cutoff^2 -
// eta^2).  skip bit 0 / 1 leaves out the z_min / z_max end (an end shared
// with an in-range collinear neighbour, whose opposite term cancels it;
// face_skip_edges).
template<int K, bool Anti, class T>
__device__ __forceinline__ T face_unit_segment(T eta, T zmin, T zmax, unsigned skip) {
  using M = FaceMath<T>;
  T total = T(0);
  static_for<0, kFacePieces[K].n>([&]<int I>() {
    constexpr T cutoff = T(kFacePieces[K].p[I].cutoff);
    if (eta >= cutoff) return;
    const T zc = M::sqrt(cutoff * cutoff - eta * eta);
    if (skip == 0) {
      const T lo = M::max(zmin, -zc), hi = M::min(zmax, zc);
      if (lo >= hi) return;
      total += face_primitive<K, I, Anti, T>(eta, hi) - face_primitive<K, I, Anti, T>(eta, lo);
      return;
    }
    // The clipped ends (a segment outside the circle gives P(+-zc) twice,
    // i.e. zero, as the early return above does).
    if (!(skip & 2u)) total += face_primitive<K, I, Anti, T>(eta, M::min(M::max(zmax, -zc), zc));
    if (!(skip & 1u)) total -= face_primitive<K, I, Anti, T>(eta, M::min(M::max(zmin, -zc), zc));
  });
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

// Unit normal cross(b - a) = (y, -x) normalised and unit tangent of a
// segment: its frame (4 doubles), stored once per face.
__device__ __forceinline__ void segment_axes(const double* ab, double* fr) {
  const double ba[2] = {ab[2] - ab[0], ab[3] - ab[1]};
  const double cr[2] = {ba[1], -ba[0]};
  normalize2(cr, fr);
  normalize2(ba, fr + 2);
}

// Segment frame at x from the stored axes fr: signed distance d and
// projections of the endpoints (units of h).
__device__ __forceinline__ FaceFrame face_frame(const double* ab, const double* fr,
                                                const double* x, double hinv) {
  FaceFrame F;
  F.n[0] = fr[0];
  F.n[1] = fr[1];
  const double* e = fr + 2;
  F.d = ((x[0] - ab[0]) * F.n[0] + (x[1] - ab[1]) * F.n[1]) * hinv;
  F.za = ((ab[0] - x[0]) * e[0] + (ab[1] - x[1]) * e[1]) * hinv;
  F.zb = ((ab[2] - x[0]) * e[0] + (ab[3] - x[1]) * e[1]) * hinv;
  return F;
}

// Kernel::flux (kernel.hpp:194-206): n w h^-1 unit_flux(|d|, z_a, z_b);
// wd = the kernel's 2D weight; the integral in type T.
template<int K, class T = double>
__device__ __forceinline__ void face_flux(const double* ab, const double* fr,
                                          const double* x, double h, double wd,
                                          double* out, unsigned skip = 0) {
  const double hinv = 1.0 / h;
  const FaceFrame F = face_frame(ab, fr, x, hinv);
  const double u = static_cast<double>(face_unit_segment<K, false, T>(
      static_cast<T>(fabs(F.d)), static_cast<T>(F.za), static_cast<T>(F.zb), skip));
  const double s = wd * hinv * u;
  out[0] = F.n[0] * s;
  out[1] = F.n[1] * s;
}

// Kernel::antigrad_flux (kernel.hpp:209-221).
template<int K, class T = double>
__device__ __forceinline__ double face_antigrad_flux(const double* ab, const double* fr,
                                                     const double* x, double h,
                                                     double wd, unsigned skip = 0) {
  const FaceFrame F = face_frame(ab, fr, x, 1.0 / h);
  const double u = static_cast<double>(face_unit_segment<K, true, T>(
      static_cast<T>(fabs(F.d)), static_cast<T>(F.za), static_cast<T>(F.zb), skip));
  return copysign(wd, F.d) * u;
}

// Segment::intersects(BSphere) (geom/segment.hpp:108-112).
__device__ __forceinline__ bool segment_in_sphere(const double* ab,
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

// ---------------------------------------------------------------------------
// Triangles (3D): kernel flux and antigradient flux (kernel.hpp:194-221,
// 316-399; kernel.gen.cpp:321-466).  The triangle is projected into its
// plane around x and scaled by 1/h; per support piece at wall distance
// eta < cutoff the integral is a sum over the edges.  Edge p0 -> p1 with
// unit tangent t: delta = det(p0, t), beta^2 = eta^2 + delta^2, z from
// dot(p0, t) over the edge's length, split where the edge crosses the circle
// of radius sqrt(cutoff^2 - eta^2); inside the circle a sub-interval adds
// the line primitive's difference, outside the sector value times the arc
// angle atan2(delta (z_hi - z_lo), z_lo z_hi + delta^2).  Line primitive:
// rho^2 = z^2 + beta^2, A = atan2(delta z (rho - eta), delta^2 rho +
// z^2 eta) (0 for tiny delta), L = asinh(z / beta) (0 for tiny beta),
// J_0 = z, J_1 = (z rho + beta^2 L)/2, J_k = (z rho^k + k beta^2 J_{k-2}) /
// (k + 1), K_0 = A, K_1 = delta L, K_k = delta J_{k-2} + eta^2 K_{k-2};
//   flux line       = sum_p c_p/(p+2) K_{p+2} - K_0 sum_p c_p eta^{p+2}/(p+2)
//   flux sector     = sum_p c_p (cutoff^{p+2} - eta^{p+2})/(p+2)
//   antigrad line   = s_0 K_0 + sum_{p>=3} s_p (eta K_{p-1} - eta^p K_0)/(p-1)
//   antigrad sector = s_0 (1 - eta/cutoff)
//                     + sum_{p>=3} s_p (eta cutoff^{p-1} - eta^p)/(p-1)
// with s_p the coefficients of the piece's 3D tail moment.

struct FaceTail3 {
  int deg;
  double s[15];
};

// 3D tail moments cutoff^3 Q(cutoff) - q^3 Q(q), Q(q) = sum_p c_p q^p/(p+3),
// of the pieces of kFacePieces, in the same order (compile time only).
inline constexpr FaceTail3 kFaceTail3[6][3] = {
  // cubic spline
  {{6, {4.0 / 15.0, 0.0, 0.0, -2.0 / 3.0, 3.0 / 4.0, -3.0 / 10.0, 1.0 / 24.0}},
   {6, {-1.0 / 60.0, 0.0, 0.0, 1.0 / 3.0, -3.0 / 4.0, 3.0 / 5.0, -1.0 / 6.0}}},
  // quartic spline
  {{7, {15625.0 / 2688.0, 0.0, 0.0, -625.0 / 48.0, 125.0 / 8.0, -15.0 / 2.0, 5.0 / 3.0, -1.0 / 7.0}},
   {7, {-729.0 / 896.0, 0.0, 0.0, 135.0 / 16.0, -135.0 / 8.0, 27.0 / 2.0, -5.0, 5.0 / 7.0}},
   {7, {1.0 / 1344.0, 0.0, 0.0, -5.0 / 24.0, 5.0 / 4.0, -3.0, 10.0 / 3.0, -10.0 / 7.0}}},
  // quintic spline
  {{8, {2187.0 / 56.0, 0.0, 0.0, -81.0, 405.0 / 4.0, -54.0, 15.0, -15.0 / 7.0, 1.0 / 8.0}},
   {8, {-64.0 / 7.0, 0.0, 0.0, 64.0, -120.0, 96.0, -40.0, 60.0 / 7.0, -3.0 / 4.0}},
   {8, {5.0 / 56.0, 0.0, 0.0, -5.0, 75.0 / 4.0, -30.0, 25.0, -75.0 / 7.0, 15.0 / 8.0}}},
  // Wendland C2
  {{8, {4.0 / 21.0, 0.0, 0.0, -1.0 / 3.0, 0.0, 1.0 / 2.0, -5.0 / 12.0, 15.0 / 112.0, -1.0 / 64.0}}},
  // Wendland C4
  {{11, {64.0 / 495.0, 0.0, 0.0, -1.0 / 3.0, 0.0, 7.0 / 15.0, 0.0, -5.0 / 8.0, 7.0 / 12.0, -35.0 / 144.0, 1.0 / 20.0, -35.0 / 8448.0}}},
  // Wendland C6
  {{14, {128.0 / 1365.0, 0.0, 0.0, -1.0 / 3.0, 0.0, 11.0 / 20.0, 0.0, -33.0 / 56.0, 0.0, 77.0 / 96.0, -33.0 / 40.0, 105.0 / 256.0, -11.0 / 96.0, 231.0 / 13312.0, -1.0 / 896.0}}},
};

// Per support piece and wall distance eta, the parts of the edge and sector
// values that do not depend on z: with a_p = c_p/(p + 2) and, for the
// antigradient, b_p = s_p/(p - 1),
//   flux:     lead = -sum_p a_p eta^{p+2},
//             sector = sum_p a_p cutoff^{p+2} + lead
//   antigrad: lead = s_0 - sum_{p>=3} b_p eta^p,
//             sector = lead + eta (sum_{p>=3} b_p cutoff^{p-1} - s_0/cutoff)
// so that the line primitive is sum_p a_p K_{p+2} + lead K_0 (flux) or
// lead K_0 + eta sum_{p>=3} b_p K_{p-1} (antigradient).
template<class T>
struct EdgeCoef {
  T lead, sector;
};
template<int K, int I, bool Anti, class T>
__device__ __forceinline__ EdgeCoef<T> face_edge_coef(T eta) {
  constexpr FacePiece kp = kFacePieces[K].p[I];
  constexpr FaceTail3 tp = kFaceTail3[K][I];
  EdgeCoef<T> e{T(0), T(0)};
  T cut = T(0);
  if constexpr (!Anti) {
    T ep = eta * eta;
    static_for<0, kp.deg + 1>([&]<int P>() {
      constexpr double a = kp.c[P] * kFaceInv[P + 2];
      constexpr double ac = a * constexpr_pow(kp.cutoff, P + 2);
      e.lead -= T(a) * ep;
      cut += T(ac);
      ep *= eta;
    });
    e.sector = cut + e.lead;
  } else {
    T ep = eta * eta * eta;
    e.lead = T(tp.s[0]);
    static_for<3, tp.deg + 1>([&]<int P>() {
      constexpr double b = tp.s[P] * kFaceInv[P - 1];
      constexpr double bc = b * constexpr_pow(kp.cutoff, P - 1);
      e.lead -= T(b) * ep;
      cut += T(bc);
      ep *= eta;
    });
    constexpr double s0c = tp.s[0] / kp.cutoff;
    e.sector = e.lead + eta * (cut - T(s0c));
  }
  return e;
}

template<int K, int I, bool Anti, class T>
__device__ __forceinline__ T face_edge_primitive(const EdgeCoef<T>& ec, T eta, T delta,
                                                 T beta2, T beta, T z) {
  using M = FaceMath<T>;
  constexpr FacePiece kp = kFacePieces[K].p[I];
  constexpr FaceTail3 tp = kFaceTail3[K][I];
  constexpr int kmax = Anti ? (tp.deg - 1 > 1 ? tp.deg - 1 : 1) : kp.deg + 2;
  const T rho = M::sqrt(z * z + beta2);
  const T A = M::abs(delta) <= T(kTiny)
                  ? T(0)
                  : M::atan2(delta * z * (rho - eta), delta * delta * rho + z * z * eta);
  const T L = M::abs(beta) <= T(kTiny)
                  ? T(0)
                  : M::copysign(M::log1p((M::abs(z) + z * z / (rho + beta)) / beta), z);
  T J[kmax + 1], Kk[kmax + 1];
  J[0] = z;
  J[1] = (z * rho + beta2 * L) * T(0.5);
  T rp = rho;
  static_for<2, kmax + 1>([&]<int P>() {
    constexpr T inv = T(kFaceInv[P + 1]);
    rp *= rho;
    J[P] = (z * rp + T(P) * beta2 * J[P - 2]) * inv;
  });
  Kk[0] = A;
  Kk[1] = delta * L;
  const T eta2 = eta * eta;
  static_for<2, kmax + 1>([&]<int P>() { Kk[P] = delta * J[P - 2] + eta2 * Kk[P - 2]; });
  T s = T(0);
  if constexpr (!Anti) {
    static_for<0, kp.deg + 1>([&]<int P>() {
      constexpr double a = kp.c[P] * kFaceInv[P + 2];
      if constexpr (a != 0.0) s += T(a) * Kk[P + 2];
    });
    return s + ec.lead * Kk[0];
  } else {
    static_for<3, tp.deg + 1>([&]<int P>() {
      constexpr double b = tp.s[P] * kFaceInv[P - 1];
      if constexpr (b != 0.0) s += T(b) * Kk[P - 1];
    });
    return ec.lead * Kk[0] + eta * s;
  }
}

// unit_triangle_integral (kernel.hpp:316-399) for the triangles of a warp,
// one per lane (inactive lanes pass active = false and get 0); all 32 lanes
// call it together.  Per support piece every lane walks its triangle's
// edges: a sub-interval outside the support circle adds the sector value
// times its arc angle at once, the (at most one) inside sub-interval of an
// edge becomes a task in a per-warp queue; the warp then evaluates the
// queued tasks (each P(z_hi) - P(z_lo) of the line primitive) 32 at a time,
// one per lane, so that the costly primitives run on full warps whatever
// mix of clipped and unclipped edges the lanes hold, and every lane adds up
// its own tasks.  v = the lane's three projected vertices (units of h).
template<class T>
struct EdgeTask {
  T zlo, zhi, delta, eta, lead;
};
constexpr int kTasksPerLane = 3;  // one inside sub-interval per edge

template<int K, int I, bool Anti, class T>
__device__ __forceinline__ T warp_triangle_piece(bool active, T eta, const T* v,
                                                 unsigned skip, EdgeTask<T>* tq, T* tv,
                                                 uint8_t* ti, int lane) {
  using M = FaceMath<T>;
  constexpr T cutoff = T(kFacePieces[K].p[I].cutoff);
  T sector_sum = T(0);
  int nt = 0;
  if (active && eta < cutoff) {
    const T radius2 = cutoff * cutoff - eta * eta;
    const EdgeCoef<T> ec = face_edge_coef<K, I, Anti, T>(eta);
    for (int e = 0; e < 3; ++e) {
      if (skip & (1u << e)) continue;
      const T* p0 = v + 2 * e;
      const T* p1 = v + 2 * (e == 2 ? 0 : e + 1);
      const T ed[2] = {p1[0] - p0[0], p1[1] - p0[1]};
      const T len2 = ed[0] * ed[0] + ed[1] * ed[1];
      if (len2 <= T(kTiny * kTiny)) continue;
      const T len = M::sqrt(len2);
      const T t[2] = {ed[0] / len, ed[1] / len};
      const T delta = p0[0] * t[1] - p0[1] * t[0];
      const T delta2 = delta * delta;
      const T z0 = p0[0] * t[0] + p0[1] * t[1];
      const T z1 = z0 + len;
      T zs[4];
      int nz = 0;
      zs[nz++] = z0;
      if (radius2 > delta2) {
        const T zc = M::sqrt(radius2 - delta2);
        if (z0 < -zc && -zc < z1) zs[nz++] = -zc;
        if (z0 < zc && zc < z1) zs[nz++] = zc;
      }
      zs[nz++] = z1;
      for (int j = 0; j + 1 < nz; ++j) {
        const T lo = zs[j], hi = zs[j + 1];
        if (M::abs(hi - lo) <= T(kTiny)) continue;
        const T mid = (lo + hi) * T(0.5);
        if (mid * mid + delta2 < radius2) {
          if (nt < kTasksPerLane) {
            tq[lane * kTasksPerLane + nt] = EdgeTask<T>{lo, hi, delta, eta, ec.lead};
            ++nt;
          } else {
            // Not reached (an edge has one inside sub-interval); evaluated
            // in place should rounding ever split one.
            const T beta2 = eta * eta + delta2;
            const T beta = M::sqrt(beta2);
            sector_sum += face_edge_primitive<K, I, Anti, T>(ec, eta, delta, beta2, beta, hi) -
                          face_edge_primitive<K, I, Anti, T>(ec, eta, delta, beta2, beta, lo);
          }
        } else {
          sector_sum += ec.sector * M::atan2(delta * (hi - lo), lo * hi + delta2);
        }
      }
    }
  }
  // Dense list of the warp's tasks (inclusive scan of the counts).
  int off = nt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, off, o);
    if (lane >= o) off += y;
  }
  const int total = __shfl_sync(0xffffffffu, off, 31);
  off -= nt;
  for (int k = 0; k < nt; ++k) ti[off + k] = static_cast<uint8_t>(lane * kTasksPerLane + k);
  __syncwarp();
  for (int t = lane; t < total; t += 32) {
    const int slot = ti[t];
    const EdgeTask<T> q = tq[slot];
    const T beta2 = q.eta * q.eta + q.delta * q.delta;
    const T beta = FaceMath<T>::sqrt(beta2);
    const EdgeCoef<T> ec{q.lead, T(0)};
    tv[slot] = face_edge_primitive<K, I, Anti, T>(ec, q.eta, q.delta, beta2, beta, q.zhi) -
               face_edge_primitive<K, I, Anti, T>(ec, q.eta, q.delta, beta2, beta, q.zlo);
  }
  __syncwarp();
  T s = sector_sum;
  for (int k = 0; k < nt; ++k) s += tv[lane * kTasksPerLane + k];
  __syncwarp();
  return s;
}

// The triangle integral summed over the kernel's pieces (all lanes call);
// edges in `skip` (bit e: edge e) are left out.
template<int K, bool Anti, class T>
__device__ __forceinline__ T warp_unit_triangle(bool active, T eta, const T* v,
                                                unsigned skip) {
  __shared__ EdgeTask<T> tq_all[kFaceBlock / 32][32 * kTasksPerLane];
  __shared__ T tv_all[kFaceBlock / 32][32 * kTasksPerLane];
  __shared__ uint8_t ti_all[kFaceBlock / 32][32 * kTasksPerLane];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T total = T(0);
  static_for<0, kFacePieces[K].n>([&]<int I>() {
    total += warp_triangle_piece<K, I, Anti, T>(active, eta, v, skip, tq_all[w], tv_all[w],
                                                ti_all[w], lane);
  });
  return total;
}

__device__ __forceinline__ void face_cross(const double* a, const double* b,
                                           double* out) {
  out[0] = a[1] * b[2] - a[2] * b[1];
  out[1] = a[2] * b[0] - a[0] * b[2];
  out[2] = a[0] * b[1] - a[1] * b[0];
}

// normalize() in 3D with the |a|^2 >= tiny^2 guard; sums left to right.
__device__ __forceinline__ void normalize3(const double* a, double* out) {
  const double n2 = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2];
  const double s = n2 >= kTiny * kTiny ? 1.0 / sqrt(n2) : 0.0;
  out[0] = a[0] * s;
  out[1] = a[1] * s;
  out[2] = a[2] * s;
}

template<int D>
__device__ __forceinline__ void normalize_d(const double* a, double* out) {
  if constexpr (D == 2) normalize2(a, out);
  else normalize3(a, out);
}

template<int D>
__device__ __forceinline__ double dot_d(const double* a, const double* b) {
  double s = a[0] * b[0] + a[1] * b[1];
  if constexpr (D == 3) s += a[2] * b[2];
  return s;
}

// Triangle frame at x (geom/triangle.hpp): normal = normalize(cross(b - a,
// c - a) / 2), signed distance d and the vertices projected on
// e1 = normalize(b - a), e2 = normalize(cross(wnormal, e1)) (units of h).
struct TriFrame {
  double n[3], d, p[6];
};
// The axes n, e1, e2 of a triangle (9 doubles), stored once per face.
__device__ __forceinline__ void triangle_axes(const double* t, double* fr) {
  const double ba[3] = {t[3] - t[0], t[4] - t[1], t[5] - t[2]};
  const double ca[3] = {t[6] - t[0], t[7] - t[1], t[8] - t[2]};
  double wn[3];
  face_cross(ba, ca, wn);
  wn[0] /= 2.0;
  wn[1] /= 2.0;
  wn[2] /= 2.0;
  normalize3(wn, fr);
  double u[3];
  normalize3(ba, fr + 3);
  face_cross(wn, fr + 3, u);
  normalize3(u, fr + 6);
}
// Triangle frame at x from the stored axes fr.
__device__ __forceinline__ TriFrame tri_frame(const double* t, const double* fr,
                                              const double* x, double hinv) {
  TriFrame F;
  F.n[0] = fr[0];
  F.n[1] = fr[1];
  F.n[2] = fr[2];
  const double* e1 = fr + 3;
  const double* e2 = fr + 6;
  const double xa[3] = {x[0] - t[0], x[1] - t[1], x[2] - t[2]};
  F.d = dot_d<3>(xa, F.n) * hinv;
  for (int i = 0; i < 3; ++i) {
    const double vx[3] = {t[3 * i] - x[0], t[3 * i + 1] - x[1], t[3 * i + 2] - x[2]};
    F.p[2 * i] = dot_d<3>(vx, e1) * hinv;
    F.p[2 * i + 1] = dot_d<3>(vx, e2) * hinv;
  }
  return F;
}

// Doubles per face in FaceArgs::frame.
template<int D>
constexpr int kFrameDoubles = D == 2 ? 4 : 9;

template<int D>
__device__ __forceinline__ const double* face_axes(const FaceArgs& fc, uint32_t f) {
  return fc.frame + kFrameDoubles<D> * static_cast<size_t>(f);
}

// The frames of all faces (one thread per face), written once when the
// faces are set.
template<int D>
__global__ void k_face_frames(const double* coords, double* frame, uint32_t nfaces) {
  const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nfaces) return;
  const size_t i = f;
  if constexpr (D == 2) segment_axes(coords + 4 * i, frame + 4 * i);
  else triangle_axes(coords + 9 * i, frame + 9 * i);
}

// Kernel::flux of face g (segment or triangle) at x; wd = the kernel's
// weight in D dimensions.  Called by all lanes of a warp together (the 3D
// integral is warp-cooperative); inactive lanes get zero.  skip: the
// triangle's edges that cancel against in-range coplanar neighbours
// (face_skip_edges).
// fr = the face's stored axes (face_axes).  The integral runs in type T
// (float with tg_params.face_fp32); frame, weights and the result are FP64.
template<int K, int D, class T = double>
__device__ __forceinline__ void face_flux_d(bool active, const double* g, const double* fr,
                                            const double* x, double h, double wd,
                                            double* out, unsigned skip = 0) {
  if constexpr (D == 2) {
    out[0] = out[1] = 0.0;
    if (active) face_flux<K, T>(g, fr, x, h, wd, out, skip);
  } else {
    const double hinv = 1.0 / h;
    const TriFrame F = tri_frame(g, fr, x, hinv);
    T p[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) p[k] = static_cast<T>(F.p[k]);
    const double u = static_cast<double>(
        warp_unit_triangle<K, false, T>(active, static_cast<T>(fabs(F.d)), p, skip));
    const double s = wd * hinv * u;
    out[0] = F.n[0] * s;
    out[1] = F.n[1] * s;
    out[2] = F.n[2] * s;
  }
}

// Kernel::antigrad_flux of face g at x (all lanes together, as above).
template<int K, int D, class T = double>
__device__ __forceinline__ double face_antigrad_flux_d(bool active, const double* g,
                                                       const double* fr, const double* x,
                                                       double h, double wd,
                                                       unsigned skip = 0) {
  if constexpr (D == 2) {
    return active ? face_antigrad_flux<K, T>(g, fr, x, h, wd, skip) : 0.0;
  } else {
    const TriFrame F = tri_frame(g, fr, x, 1.0 / h);
    T p[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) p[k] = static_cast<T>(F.p[k]);
    return copysign(wd, F.d) * static_cast<double>(warp_unit_triangle<K, true, T>(
                                   active, static_cast<T>(fabs(F.d)), p, skip));
  }
}

// Closest point of a segment (Segment::clamp, geom/segment.hpp:91-106).
__device__ __forceinline__ void segment_clamp3(const double* a, const double* b,
                                               const double* x, double* q) {
  const double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double xa[3] = {x[0] - a[0], x[1] - a[1], x[2] - a[2]};
  q[0] = a[0];
  q[1] = a[1];
  q[2] = a[2];
  const double len2 = dot_d<3>(ba, ba);
  if (fabs(len2) <= kTiny) return;
  const double t = dot_d<3>(xa, ba) / len2;
  if (t > 1.0) {
    q[0] = b[0];
    q[1] = b[1];
    q[2] = b[2];
  } else if (!(t < 0.0)) {
    q[0] = a[0] + t * ba[0];
    q[1] = a[1] + t * ba[1];
    q[2] = a[2] + t * ba[2];
  }
}

// Closest point of a triangle (Triangle::clamp, geom/triangle.hpp): the
// Voronoi-region walk of Ericson, Real-Time Collision Detection 5.1.5; a
// degenerate triangle clamps to its longest edge.
__device__ __forceinline__ void triangle_clamp(const double* t, const double* x,
                                               double* q) {
  const double* a = t;
  const double* b = t + 3;
  const double* c = t + 6;
  const double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double ca[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double cb[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
  double wn[3];
  face_cross(ba, ca, wn);
  wn[0] /= 2.0;
  wn[1] /= 2.0;
  wn[2] /= 2.0;
  if (sqrt(dot_d<3>(wn, wn)) <= kTiny) {
    const double l_ab = dot_d<3>(ba, ba), l_bc = dot_d<3>(cb, cb), l_ca = dot_d<3>(ca, ca);
    if (l_ab >= l_bc && l_ab >= l_ca) return segment_clamp3(a, b, x, q);
    if (l_bc >= l_ca) return segment_clamp3(b, c, x, q);
    return segment_clamp3(a, c, x, q);
  }
  const double pa[3] = {x[0] - a[0], x[1] - a[1], x[2] - a[2]};
  const double d1 = dot_d<3>(ba, pa), d2 = dot_d<3>(ca, pa);
  const double* corner = nullptr;
  if (d1 <= 0.0 && d2 <= 0.0) corner = a;
  const double pb[3] = {x[0] - b[0], x[1] - b[1], x[2] - b[2]};
  const double d3 = dot_d<3>(ba, pb), d4 = dot_d<3>(ca, pb);
  if (corner == nullptr && d3 >= 0.0 && d4 <= d3) corner = b;
  const double pc[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
  const double d5 = dot_d<3>(ba, pc), d6 = dot_d<3>(ca, pc);
  if (corner == nullptr && d6 >= 0.0 && d5 <= d6) corner = c;
  if (corner != nullptr) {
    q[0] = corner[0];
    q[1] = corner[1];
    q[2] = corner[2];
    return;
  }
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    const double s = d1 / (d1 - d3);
    for (int k = 0; k < 3; ++k) q[k] = a[k] + s * ba[k];
    return;
  }
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    const double s = d2 / (d2 - d6);
    for (int k = 0; k < 3; ++k) q[k] = a[k] + s * ca[k];
    return;
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && d4 >= d3 && d5 >= d6) {
    const double s = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    for (int k = 0; k < 3; ++k) q[k] = b[k] + s * cb[k];
    return;
  }
  const double v = vb / (va + vb + vc);
  const double w = vc / (va + vb + vc);
  for (int k = 0; k < 3; ++k) q[k] = a[k] + v * ba[k] + w * ca[k];
}

// Triangle::intersects(BSphere): boxes overlap and the closest point of the
// triangle is in the sphere.
__device__ __forceinline__ bool triangle_in_sphere(const double* t,
                                                   const double* x,
                                                   double radius) {
  for (int k = 0; k < 3; ++k) {
    const double lo = fmin(fmin(t[k], t[3 + k]), t[6 + k]);
    const double hi = fmax(fmax(t[k], t[3 + k]), t[6 + k]);
    if (!(x[k] - radius <= hi && lo <= x[k] + radius)) return false;
  }
  double q[3];
  triangle_clamp(t, x, q);
  const double d[3] = {q[0] - x[0], q[1] - x[1], q[2] - x[2]};
  return dot_d<3>(d, d) <= radius * radius;
}

// Edges (3D) or ends (2D) of face f whose coplanar (collinear) neighbour
// across them is also within the support radius of x (a face adjacent to
// the particle).  3D: the two triangles traverse the shared edge in
// opposite directions in the same plane (their frames differ by a rotation
// in it), so its edge integrals (line primitive differences and sector
// arcs, both odd under reversing the edge) cancel.  2D: the shared end is
// the upper end of one segment and the lower end of the other on the same
// line, so its two clipped primitive terms cancel.  Plain sums of the
// particle's face fluxes (grad gamma, the antigradient sum of gamma) are
// the same without them; sums that weight each face differently (the face
// terms) keep every edge.
template<int D>
__device__ __forceinline__ unsigned face_skip_edges(const FaceArgs& fc, uint32_t f,
                                                    const double* x, double radius) {
  unsigned skip = 0;
#pragma unroll
  for (int e = 0; e < (D == 2 ? 2 : 3); ++e) {
    const int32_t nb = fc.edge_nbr[(D == 2 ? 2 : 3) * static_cast<size_t>(f) + e];
    if (nb < 0) continue;
    const double* g = fc.coords + D * D * static_cast<size_t>(nb);
    bool in;
    if constexpr (D == 2) in = segment_in_sphere(g, x, radius);
    else in = triangle_in_sphere(g, x, radius);
    if (in) skip |= 1u << e;
  }
  return skip;
}

// Faces within the support radius of x (the particle's cell list holds
// every face within reach of the cell), shared by the lanes of a warp: the
// lanes test 32 list entries at a time and queue the faces that pass in a
// per-warp shared buffer, and every full batch of 32 queued faces is
// integrated with one face per lane (the rest at the end, with the idle
// lanes inactive), so the costly integrals run on full warps.  fn(active,
// f, coords) is called by all 32 lanes together.  Blocks of kFaceBlock
// threads.

template<int D, class Fn>
__device__ __forceinline__ void for_adjacent_faces(const FaceArgs& fc,
                                                   uint32_t gcell,
                                                   const double* x,
                                                   double radius, int lane,
                                                   Fn&& fn) {
  __shared__ uint32_t queue[kFaceBlock / 32][64];
  uint32_t* q = queue[threadIdx.x >> 5];
  const uint32_t s = fc.cell_start[gcell], e = fc.cell_start[gcell + 1];
  int pending = 0;
  for (uint32_t base = s; base < e; base += 32) {
    const uint32_t i = base + static_cast<uint32_t>(lane);
    bool in = false;
    uint32_t f = 0;
    if (i < e) {
      f = fc.cell_face[i];
      const double* g = fc.coords + D * D * static_cast<size_t>(f);
      if constexpr (D == 2) in = segment_in_sphere(g, x, radius);
      else in = triangle_in_sphere(g, x, radius);
    }
    const unsigned mask = __ballot_sync(0xffffffffu, in);
    if (in) q[pending + __popc(mask & ((1u << lane) - 1u))] = f;
    pending += __popc(mask);
    __syncwarp();
    if (pending >= 32) {
      pending -= 32;
      const uint32_t g = q[pending + lane];
      __syncwarp();
      fn(true, g, fc.coords + D * D * static_cast<size_t>(g));
    }
  }
  if (pending > 0) {
    const bool active = lane < pending;
    const uint32_t g = q[active ? lane : 0];
    fn(active, g, fc.coords + D * D * static_cast<size_t>(g));
  }
  __syncwarp();
}

// Capacity of the per-warp list of a face particle's in-range faces
// (collect_adjacent_faces); a particle with more takes the list-free path.
constexpr int kFaceListCap = 256;

// The faces of the particle's cell list within the support radius of x
// (the for_adjacent_faces predicate), ascending, into the warp's list; all
// lanes call and get the count.  A count above cap means the list holds
// only the first cap faces.
template<int D>
__device__ __forceinline__ int collect_adjacent_faces(const FaceArgs& fc, uint32_t gcell,
                                                      const double* x, double radius,
                                                      int lane, uint32_t* list, int cap) {
  __syncwarp();  // the previous particle's readers are done with the list
  const uint32_t s = fc.cell_start[gcell], e = fc.cell_start[gcell + 1];
  int count = 0;
  for (uint32_t base = s; base < e; base += 32) {
    const uint32_t i = base + static_cast<uint32_t>(lane);
    bool in = false;
    uint32_t f = 0;
    if (i < e) {
      f = fc.cell_face[i];
      const double* g = fc.coords + D * D * static_cast<size_t>(f);
      if constexpr (D == 2) in = segment_in_sphere(g, x, radius);
      else in = triangle_in_sphere(g, x, radius);
    }
    const unsigned mask = __ballot_sync(0xffffffffu, in);
    const int slot = count + __popc(mask & ((1u << lane) - 1u));
    if (in && slot < cap) list[slot] = f;
    count += __popc(mask);
  }
  __syncwarp();
  return count;
}

// Whether face f is in the ascending list of n faces.
__device__ __forceinline__ bool face_listed(const uint32_t* list, int n, uint32_t f) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (list[mid] < f) lo = mid + 1;
    else hi = mid;
  }
  return lo < n && list[lo] == f;
}

// face_skip_edges with the in-range test of the neighbours answered by the
// particle's complete list of in-range faces: a neighbour within the
// support radius is in the particle's cell list (which holds every face
// within reach of the cell), so it is listed exactly when the sphere test
// passes.
template<int D>
__device__ __forceinline__ unsigned face_skip_edges_listed(const FaceArgs& fc, uint32_t f,
                                                           const uint32_t* list, int n) {
  unsigned skip = 0;
#pragma unroll
  for (int e = 0; e < (D == 2 ? 2 : 3); ++e) {
    const int32_t nb = fc.edge_nbr[(D == 2 ? 2 : 3) * static_cast<size_t>(f) + e];
    if (nb >= 0 && face_listed(list, n, static_cast<uint32_t>(nb))) skip |= 1u << e;
  }
  return skip;
}

// Sum over the lanes of a warp (all lanes active), butterfly order.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// 3D containment: the particle's cell answers unless the containment
// surface reaches it; there the exact winding number of the surface
// (Triangle::winding_number, geom/triangle.hpp: per triangle
// atan2(det(a', b', c'), |a'||b'||c'| + (a'.b')|c'| + (b'.c')|a'| +
// (c'.a')|b'|) / (2 pi), primes = vertex - x) decides, > 1/2.
// With lanes = 32 the warp splits the triangles (lane l takes l, l + 32,
// ...) and every lane gets the answer; with lanes = 1 one thread sums them.
__device__ __forceinline__ bool face_contains3(const FaceArgs& fc, uint32_t tank,
                                               uint32_t gcell, const double* x,
                                               int lane, int lanes) {
  const int st = fc.cell_state[gcell];
  if (st >= 0) return st != 0;
  double w = 0.0;
  for (uint32_t i = fc.cont_start[tank] + lane; i < fc.cont_start[tank + 1]; i += lanes) {
    const double* t = fc.cont_tri + 9 * static_cast<size_t>(i);
    const double ap[3] = {t[0] - x[0], t[1] - x[1], t[2] - x[2]};
    const double bp[3] = {t[3] - x[0], t[4] - x[1], t[5] - x[2]};
    const double cp[3] = {t[6] - x[0], t[7] - x[1], t[8] - x[2]};
    const double na = sqrt(dot_d<3>(ap, ap));
    const double nb = sqrt(dot_d<3>(bp, bp));
    const double nc = sqrt(dot_d<3>(cp, cp));
    const double den = na * nb * nc + dot_d<3>(ap, bp) * nc +
                       dot_d<3>(bp, cp) * na + dot_d<3>(cp, ap) * nb;
    double bc[3];
    face_cross(bp, cp, bc);
    w += atan2(dot_d<3>(ap, bc), den) / (2.0 * 3.141592653589793);
  }
  if (lanes == 32) w = warp_sum(w);
  return w > 0.5;
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
