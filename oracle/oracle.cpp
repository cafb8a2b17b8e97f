// oracle.cpp - CPU restatement of TitSolver's WCSPH hot path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h): the checker for the GPU path and
// the timed CPU baseline.  Product code never links or calls it.
//
// Every function states the reference file:line it restates (paths relative
// to the TitSolver source tree).  Compiled with -ffp-contract=off and no
// fast-math, so the arithmetic is plain IEEE double (or float) in the order
// written here.  The pair sums are evaluated in the gather form: for a target
// a, sum over b in N(a) \ {a} in ascending b, of the same term the reference
// scatters to a from the unique pair (a, b) (fluid_equations.hpp:249-259,
// 293-304); the terms are antisymmetric-consistent, so only summation order
// differs from the reference's thread-count-dependent block order.

#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numbers>
#include <random>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Parallel loop (stands in for par::for_each, par/algorithms.hpp:56-80).
// Every index writes only its own outputs, so results do not depend on the
// thread count.

template<class Fn>
void parallel_for(int64_t n, int32_t nthreads, Fn&& fn) {
  if (n <= 0) return;
  int64_t nt = nthreads > 0 ? nthreads : 1;
  if (nt > n) nt = n;
  if (nt <= 1 || n < 256) {
    for (int64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<int64_t> next{0};
  const int64_t chunk = std::max<int64_t>(64, n / (nt * 16));
  auto worker = [&]() {
    for (;;) {
      const int64_t begin = next.fetch_add(chunk);
      if (begin >= n) break;
      const int64_t end = std::min(n, begin + chunk);
      for (int64_t i = begin; i < end; ++i) fn(i);
    }
  };
  std::vector<std::thread> pool;
  pool.reserve(static_cast<size_t>(nt - 1));
  for (int64_t t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// core/math.hpp:84-170 restated.

constexpr double tiny_d = 6.0554544523933395e-06;  // cbrt(DBL_EPSILON)
constexpr float tiny_f = 6.0554544523933395e-06f;

template<class Num>
constexpr Num tiny_v() {
  if constexpr (sizeof(Num) == 4) return tiny_f;
  else return tiny_d;
}
template<class Num>
bool is_tiny(Num a) { return std::abs(a) <= tiny_v<Num>(); }
template<class Num>
Num pow2(Num a) { return a * a; }
// Integer power by squaring, core/math.hpp:92-104.
template<class Num>
Num ipow(Num a, int p) {
  if (p == 0) return Num{1};
  if (p == 1) return a;
  if (p % 2 == 0) return ipow(a * a, p / 2);
  return a * ipow(a * a, p / 2);
}

// Vector helpers of core/_vec/vec.hpp:627-676.  dot() sums left to right:
// (x0*y0 + x1*y1) + x2*y2.  The reference's SIMD ReduceSum is exact for 2D;
// its 3D lane order is a third-party choice, and this fixes it.
template<class Num>
Num dot(const Num* a, const Num* b, int d) {
  Num r = a[0] * b[0];
  for (int i = 1; i < d; ++i) r += a[i] * b[i];
  return r;
}
template<class Num>
Num norm2(const Num* a, int d) { return dot(a, a, d); }
template<class Num>
Num norm(const Num* a, int d) { return std::sqrt(norm2(a, d)); }
// normalize(): multiply by the reciprocal norm when |a|^2 >= tiny^2.
template<class Num>
void normalize(const Num* a, int d, Num* out) {
  const Num n2 = norm2(a, d);
  const Num eps2 = pow2(tiny_v<Num>());
  const Num s = n2 >= eps2 ? Num{1} / std::sqrt(n2) : Num{0};
  for (int i = 0; i < d; ++i) out[i] = a[i] * s;
}

uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// ---------------------------------------------------------------------------
// Kernels: sph/kernel.hpp:126-163 with the support pieces of
// sph/kernel.gen.cpp:520-553, each piece guarded by q < cutoff
// (kernel.gen.cpp:631-636).  Zero moments int_0^R q^(d-1) w(q) dq are the
// exact rationals of those polynomials.

struct KernelTable {
  double unit_radius;
  double moment[3];  // Dim = 1, 2, 3
};

constexpr KernelTable kernel_table[6] = {
    {2.0, {3.0 / 4.0, 7.0 / 20.0, 1.0 / 4.0}},          // cubic spline
    {2.5, {12.0, 1199.0 / 192.0, 5.0}},                 // quartic spline
    {3.0, {60.0, 239.0 / 7.0, 30.0}},                   // quintic spline
    {2.0, {2.0 / 3.0, 2.0 / 7.0, 4.0 / 21.0}},          // Wendland C2
    {2.0, {16.0 / 27.0, 2.0 / 9.0, 64.0 / 495.0}},      // Wendland C4
    {2.0, {8.0 / 15.0, 7.0 / 39.0, 128.0 / 1365.0}},    // Wendland C6
};

template<class Num>
Num unit_value(int k, Num q) {
  const Num one{1};
  switch (k) {
    case TG_KERNEL_CUBIC_SPLINE:
      return (q < Num{2} ? Num{0.25} * ipow(Num{2} - q, 3) : Num{0}) +
             (q < Num{1} ? -ipow(one - q, 3) : Num{0});
    case TG_KERNEL_QUARTIC_SPLINE:
      return (q < Num{2.5} ? ipow(Num{2.5} - q, 4) : Num{0}) +
             (q < Num{1.5} ? Num{-5} * ipow(Num{1.5} - q, 4) : Num{0}) +
             (q < Num{0.5} ? Num{10} * ipow(Num{0.5} - q, 4) : Num{0});
    case TG_KERNEL_QUINTIC_SPLINE:
      return (q < Num{3} ? ipow(Num{3} - q, 5) : Num{0}) +
             (q < Num{2} ? Num{-6} * ipow(Num{2} - q, 5) : Num{0}) +
             (q < Num{1} ? Num{15} * ipow(one - q, 5) : Num{0});
    case TG_KERNEL_WENDLAND_C2:
      return q < Num{2} ? (one + Num{2} * q) * ipow(one - Num{0.5} * q, 4)
                        : Num{0};
    case TG_KERNEL_WENDLAND_C4:
      return q < Num{2} ? (one + Num{3} * q + Num(35.0 / 12.0) * q * q) *
                              ipow(one - Num{0.5} * q, 6)
                        : Num{0};
    case TG_KERNEL_WENDLAND_C6:
      return q < Num{2} ? (one + Num{4} * q + Num{6.25} * q * q +
                           Num{4} * q * q * q) *
                              ipow(one - Num{0.5} * q, 8)
                        : Num{0};
    default: return Num{0};
  }
}

template<class Num>
Num unit_deriv(int k, Num q) {
  const Num one{1};
  switch (k) {
    case TG_KERNEL_CUBIC_SPLINE:
      return (q < Num{2} ? Num{-0.75} * ipow(Num{2} - q, 2) : Num{0}) +
             (q < Num{1} ? Num{3} * ipow(one - q, 2) : Num{0});
    case TG_KERNEL_QUARTIC_SPLINE:
      return (q < Num{2.5} ? Num{-4} * ipow(Num{2.5} - q, 3) : Num{0}) +
             (q < Num{1.5} ? Num{20} * ipow(Num{1.5} - q, 3) : Num{0}) +
             (q < Num{0.5} ? Num{-40} * ipow(Num{0.5} - q, 3) : Num{0});
    case TG_KERNEL_QUINTIC_SPLINE:
      return (q < Num{3} ? Num{-5} * ipow(Num{3} - q, 4) : Num{0}) +
             (q < Num{2} ? Num{30} * ipow(Num{2} - q, 4) : Num{0}) +
             (q < Num{1} ? Num{-75} * ipow(one - q, 4) : Num{0});
    case TG_KERNEL_WENDLAND_C2:
      return q < Num{2} ? Num{-5} * q * ipow(one - Num{0.5} * q, 3) : Num{0};
    case TG_KERNEL_WENDLAND_C4:
      return q < Num{2} ? Num(-14.0 / 3.0) * q * (one + Num{2.5} * q) *
                              ipow(one - Num{0.5} * q, 5)
                        : Num{0};
    case TG_KERNEL_WENDLAND_C6:
      return q < Num{2} ? Num{-2.75} * q *
                              (Num{2} + Num{7} * q + Num{8} * q * q) *
                              ipow(one - Num{0.5} * q, 7)
                        : Num{0};
    default: return Num{0};
  }
}

// Kernel weight, kernel.hpp:126-131: 1 / (zero moment * |S^{d-1}|), with
// unit_sphere_area_v = 2 sqrt(pi^d) / Gamma(d/2) (core/math.hpp:174-180).
double kernel_weight(int k, int d) {
  const double area = 2.0 * std::sqrt(std::pow(std::numbers::pi, d)) /
                      std::tgamma(d / 2.0);
  return 1.0 / (kernel_table[k].moment[d - 1] * area);
}

// ---------------------------------------------------------------------------
// Semi-analytical face boundaries in 2D: kernel flux and antigradient flux
// over a segment (kernel.hpp:194-221, 286-314; kernel.gen.cpp:313-395).
// Each kernel is a sum of support pieces w_i(q) = sum_p c_p q^p for
// q < cutoff_i (the pieces of kernel.gen.cpp:520-553, expanded; t_p are the
// coefficients of the piece's 2D tail moment T(q) = cutoff^2 P(cutoff) -
// q^2 P(q), P(q) = sum_p c_p q^p / (p + 2)).  Over a segment at wall
// distance eta and along-segment coordinates [z_min, z_max] (units of h):
//   unit_flux          = sum over pieces of [sum_p c_p J_p]
//   unit_antigrad_flux = sum over pieces of [t_0 A + t_1 eta L +
//                                            sum_{p>=2} t_p eta J_{p-2}]
// each clipped to |z| <= sqrt(cutoff^2 - eta^2), with rho^2 = z^2 + eta^2,
// A = atan2(z, eta), L = copysign(log1p((|z| + z^2/(rho + eta))/eta), z)
// (0 when eta is tiny), J_0 = z, J_1 = (z rho + eta^2 L)/2,
// J_p = (z rho^p + p eta^2 J_{p-2})/(p + 1).  The reference evaluates A and
// L with Highway's fast_atan2/fast_log1p; this restatement uses the libm
// functions.

struct KernelPiece {
  double cutoff;
  int deg;
  double c[12];
  int tdeg;
  double t[14];
};
struct KernelPieces {
  int n;
  KernelPiece p[3];
};

constexpr KernelPieces kPieces[6] = {
  // cubic
  {2, {{2.0, 3, {2.0, -3.0, 3.0 / 2.0, -1.0 / 4.0}, 5, {2.0 / 5.0, 0.0, -1.0, 1.0, -3.0 / 8.0, 1.0 / 20.0}},
   {1.0, 3, {-1.0, 3.0, -3.0, 1.0}, 5, {-1.0 / 20.0, 0.0, 1.0 / 2.0, -1.0, 3.0 / 4.0, -1.0 / 5.0}}}},
  // quartic
  {3, {{5.0 / 2.0, 4, {625.0 / 16.0, -125.0 / 2.0, 75.0 / 2.0, -10.0, 1.0}, 6, {3125.0 / 384.0, 0.0, -625.0 / 32.0, 125.0 / 6.0, -75.0 / 8.0, 2.0, -1.0 / 6.0}},
   {3.0 / 2.0, 4, {-405.0 / 16.0, 135.0 / 2.0, -135.0 / 2.0, 30.0, -5.0}, 6, {-243.0 / 128.0, 0.0, 405.0 / 32.0, -45.0 / 2.0, 135.0 / 8.0, -6.0, 5.0 / 6.0}},
   {1.0 / 2.0, 4, {5.0 / 8.0, -5.0, 15.0, -20.0, 10.0}, 6, {1.0 / 192.0, 0.0, -5.0 / 16.0, 5.0 / 3.0, -15.0 / 4.0, 4.0, -5.0 / 3.0}}}},
  // quintic
  {3, {{3.0, 5, {243.0, -405.0, 270.0, -90.0, 15.0, -1.0}, 7, {729.0 / 14.0, 0.0, -243.0 / 2.0, 135.0, -135.0 / 2.0, 18.0, -5.0 / 2.0, 1.0 / 7.0}},
   {2.0, 5, {-192.0, 480.0, -480.0, 240.0, -60.0, 6.0}, 7, {-128.0 / 7.0, 0.0, 96.0, -160.0, 120.0, -48.0, 10.0, -6.0 / 7.0}},
   {1.0, 5, {15.0, -75.0, 150.0, -150.0, 75.0, -15.0}, 7, {5.0 / 14.0, 0.0, -15.0 / 2.0, 25.0, -75.0 / 2.0, 30.0, -25.0 / 2.0, 15.0 / 7.0}}}},
  // wc2
  {1, {{2.0, 5, {1.0, 0.0, -5.0 / 2.0, 5.0 / 2.0, -15.0 / 16.0, 1.0 / 8.0}, 7, {2.0 / 7.0, 0.0, -1.0 / 2.0, 0.0, 5.0 / 8.0, -1.0 / 2.0, 5.0 / 32.0, -1.0 / 56.0}}}},
  // wc4
  {1, {{2.0, 8, {1.0, 0.0, -7.0 / 3.0, 0.0, 35.0 / 8.0, -14.0 / 3.0, 35.0 / 16.0, -1.0 / 2.0, 35.0 / 768.0}, 10, {2.0 / 9.0, 0.0, -1.0 / 2.0, 0.0, 7.0 / 12.0, 0.0, -35.0 / 48.0, 2.0 / 3.0, -35.0 / 128.0, 1.0 / 18.0, -7.0 / 1536.0}}}},
  // wc6
  {1, {{2.0, 11, {1.0, 0.0, -11.0 / 4.0, 0.0, 33.0 / 8.0, 0.0, -231.0 / 32.0, 33.0 / 4.0, -1155.0 / 256.0, 11.0 / 8.0, -231.0 / 1024.0, 1.0 / 64.0}, 13, {7.0 / 39.0, 0.0, -1.0 / 2.0, 0.0, 11.0 / 16.0, 0.0, -11.0 / 16.0, 0.0, 231.0 / 256.0, -11.0 / 12.0, 231.0 / 512.0, -1.0 / 8.0, 77.0 / 4096.0, -1.0 / 832.0}}}},
};



// 1/k, k = 0..17 (entry 0 unused): the recursions multiply by these.
constexpr double kInv[18] = {
    0.0, 1.0, 1.0 / 2.0, 1.0 / 3.0, 1.0 / 4.0, 1.0 / 5.0, 1.0 / 6.0, 1.0 / 7.0, 1.0 / 8.0,
    1.0 / 9.0, 1.0 / 10.0, 1.0 / 11.0, 1.0 / 12.0, 1.0 / 13.0, 1.0 / 14.0, 1.0 / 15.0,
    1.0 / 16.0, 1.0 / 17.0};

void line_integrals(double eta, double z, double rho, double L, int pmax,
                    double* J) {
  J[0] = z;
  if (pmax >= 1) J[1] = (z * rho + eta * eta * L) * 0.5;
  double rp = rho;
  for (int p = 2; p <= pmax; ++p) {
    rp *= rho;
    J[p] = (z * rp + p * eta * eta * J[p - 2]) * kInv[p + 1];
  }
}

double piece_primitive(const KernelPiece& kp, bool antigrad, double eta,
                       double z) {
  const double rho = std::sqrt(z * z + eta * eta);
  const double A = std::atan2(z, eta);
  const double L =
      std::abs(eta) <= tiny_d
          ? 0.0
          : std::copysign(std::log1p((std::abs(z) + z * z / (rho + eta)) / eta), z);
  double J[16];
  double s = 0.0;
  if (!antigrad) {
    line_integrals(eta, z, rho, L, kp.deg, J);
    for (int p = 0; p <= kp.deg; ++p) s += kp.c[p] * J[p];
    return s;
  }
  line_integrals(eta, z, rho, L, std::max(kp.tdeg - 2, 0), J);
  for (int p = 0; p <= kp.tdeg; ++p) {
    if (p == 0) s += kp.t[0] * A;
    else if (p == 1) s += kp.t[1] * eta * L;
    else s += kp.t[p] * eta * J[p - 2];
  }
  return s;
}

// unit_segment_integral (kernel.hpp:286-314) summed over the pieces.
double unit_segment(int k, bool antigrad, double eta, double zmin, double zmax) {
  double total = 0.0;
  for (int i = 0; i < kPieces[k].n; ++i) {
    const KernelPiece& kp = kPieces[k].p[i];
    if (eta >= kp.cutoff) continue;
    const double zc = std::sqrt(kp.cutoff * kp.cutoff - eta * eta);
    const double lo = std::max(zmin, -zc), hi = std::min(zmax, zc);
    if (lo >= hi) continue;
    total += piece_primitive(kp, antigrad, eta, hi) -
             piece_primitive(kp, antigrad, eta, lo);
  }
  return total;
}

// Segment geometry (geom/segment.hpp): normal = normalize(cross(b - a)),
// cross((x, y)) = (y, -x) (core/_vec/vec.hpp:692-694); project(x) =
// (dot(a - x, e), dot(b - x, e)), e = normalize(b - a).
struct SegFrame {
  double n[2], d, za, zb;
};
SegFrame seg_frame(const double* a, const double* b, const double* x,
                   double h) {
  const double ba[2] = {b[0] - a[0], b[1] - a[1]};
  const double cr[2] = {ba[1], -ba[0]};
  SegFrame F;
  normalize(cr, 2, F.n);
  double e[2];
  normalize(ba, 2, e);
  const double hinv = 1.0 / h;
  const double xa[2] = {x[0] - a[0], x[1] - a[1]};
  F.d = dot(xa, F.n, 2) * hinv;
  const double ax[2] = {a[0] - x[0], a[1] - x[1]};
  const double bx[2] = {b[0] - x[0], b[1] - x[1]};
  F.za = dot(ax, e, 2) * hinv;
  F.zb = dot(bx, e, 2) * hinv;
  return F;
}

// Kernel::flux (kernel.hpp:194-206): n w h^-1 unit_flux(|d|, z_a, z_b).
void face_flux(int k, const double* a, const double* b, const double* x,
               double h, double* out) {
  const SegFrame F = seg_frame(a, b, x, h);
  const double w = kernel_weight(k, 2) * (1.0 / h);
  const double s = w * unit_segment(k, false, std::abs(F.d), F.za, F.zb);
  out[0] = F.n[0] * s;
  out[1] = F.n[1] * s;
}

// Kernel::antigrad_flux (kernel.hpp:209-221).
double face_antigrad_flux(int k, const double* a, const double* b,
                          const double* x, double h) {
  const SegFrame F = seg_frame(a, b, x, h);
  return std::copysign(kernel_weight(k, 2), F.d) *
         unit_segment(k, true, std::abs(F.d), F.za, F.zb);
}

// Segment::intersects(BSphere) (geom/segment.hpp:108-112): boxes overlap
// and the closest point of the segment (clamp, :91-106) is in the sphere.
bool face_in_sphere(const double* a, const double* b, const double* c,
                    double radius) {
  for (int k = 0; k < 2; ++k) {
    const double lo = std::min(a[k], b[k]), hi = std::max(a[k], b[k]);
    if (!(c[k] - radius <= hi && lo <= c[k] + radius)) return false;
  }
  const double ba[2] = {b[0] - a[0], b[1] - a[1]};
  const double len2 = norm2(ba, 2);
  double q[2] = {a[0], a[1]};
  if (!is_tiny(len2)) {
    const double pa[2] = {c[0] - a[0], c[1] - a[1]};
    const double t = dot(pa, ba, 2) / len2;
    if (t > 1.0) {
      q[0] = b[0];
      q[1] = b[1];
    } else if (!(t < 0.0)) {
      q[0] = a[0] + t * ba[0];
      q[1] = a[1] + t * ba[1];
    }
  }
  const double d[2] = {q[0] - c[0], q[1] - c[1]};
  return norm2(d, 2) <= radius * radius;
}

// Exact generalized winding number of a closed polygon at x
// (Segment::winding_number, geom/segment.hpp:74-79, summed over the loop).
double winding_number(int32_t n_poly, const double* poly, const double* x) {
  double w = 0.0;
  for (int32_t i = 0; i < n_poly; ++i) {
    const double* a = poly + 2 * i;
    const double* b = poly + 2 * ((i + 1) % n_poly);
    const double ap[2] = {a[0] - x[0], a[1] - x[1]};
    const double bp[2] = {b[0] - x[0], b[1] - x[1]};
    w += std::atan2(ap[0] * bp[1] - ap[1] * bp[0], dot(ap, bp, 2)) /
         (2.0 * std::numbers::pi);
  }
  return w;
}

// ---------------------------------------------------------------------------
// Semi-analytical face boundaries in 3D: kernel flux and antigradient flux
// over a triangle (kernel.hpp:194-221, 316-399; kernel.gen.cpp:321-466).
// The triangle is projected into its plane around x (Triangle::project,
// geom/triangle.hpp) and scaled by 1/h; for each support piece at wall
// distance eta < cutoff the integral over the triangle is a sum over its
// edges.  Edge p0 -> p1 with unit tangent t: delta = det(p0, t),
// beta^2 = eta^2 + delta^2, z from dot(p0, t) to dot(p0, t) + |p1 - p0|,
// split where the edge crosses the circle of radius sqrt(cutoff^2 - eta^2);
// a sub-interval inside the circle adds the difference of the line
// primitive, one outside adds the sector value times the arc angle
// atan2(delta (z_hi - z_lo), z_lo z_hi + delta^2).  Line primitive at z:
// rho^2 = z^2 + beta^2, A = atan2(delta z (rho - eta), delta^2 rho +
// z^2 eta) (0 for tiny delta), L = copysign(log1p((|z| + z^2/(rho + beta))
// / beta), z) (0 for tiny beta), J_0 = z, J_1 = (z rho + beta^2 L)/2,
// J_k = (z rho^k + k beta^2 J_{k-2})/(k + 1), K_0 = A, K_1 = delta L,
// K_k = delta J_{k-2} + eta^2 K_{k-2}, and
//   flux line       = sum_p c_p/(p+2) K_{p+2} - K_0 sum_p c_p eta^{p+2}/(p+2)
//   flux sector     = sum_p c_p (cutoff^{p+2} - eta^{p+2})/(p+2)
//   antigrad line   = s_0 K_0 + sum_{p>=3} s_p (eta K_{p-1} - eta^p K_0)/(p-1)
//   antigrad sector = s_0 (1 - eta/cutoff)
//                     + sum_{p>=3} s_p (eta cutoff^{p-1} - eta^p)/(p-1)
// where s_p are the coefficients of the piece's 3D tail moment
// cutoff^3 Q(cutoff) - q^3 Q(q), Q(q) = sum_p c_p q^p/(p + 3) (its q and q^2
// coefficients are zero).

struct TailPiece3 {
  int deg;
  double s[15];
};

// 3D tail moments of the pieces of kPieces, in the same order.
constexpr TailPiece3 kTail3[6][3] = {
  // cubic
  {{6, {4.0 / 15.0, 0.0, 0.0, -2.0 / 3.0, 3.0 / 4.0, -3.0 / 10.0, 1.0 / 24.0}},
   {6, {-1.0 / 60.0, 0.0, 0.0, 1.0 / 3.0, -3.0 / 4.0, 3.0 / 5.0, -1.0 / 6.0}}},
  // quartic
  {{7, {15625.0 / 2688.0, 0.0, 0.0, -625.0 / 48.0, 125.0 / 8.0, -15.0 / 2.0, 5.0 / 3.0, -1.0 / 7.0}},
   {7, {-729.0 / 896.0, 0.0, 0.0, 135.0 / 16.0, -135.0 / 8.0, 27.0 / 2.0, -5.0, 5.0 / 7.0}},
   {7, {1.0 / 1344.0, 0.0, 0.0, -5.0 / 24.0, 5.0 / 4.0, -3.0, 10.0 / 3.0, -10.0 / 7.0}}},
  // quintic
  {{8, {2187.0 / 56.0, 0.0, 0.0, -81.0, 405.0 / 4.0, -54.0, 15.0, -15.0 / 7.0, 1.0 / 8.0}},
   {8, {-64.0 / 7.0, 0.0, 0.0, 64.0, -120.0, 96.0, -40.0, 60.0 / 7.0, -3.0 / 4.0}},
   {8, {5.0 / 56.0, 0.0, 0.0, -5.0, 75.0 / 4.0, -30.0, 25.0, -75.0 / 7.0, 15.0 / 8.0}}},
  // wc2
  {{8, {4.0 / 21.0, 0.0, 0.0, -1.0 / 3.0, 0.0, 1.0 / 2.0, -5.0 / 12.0, 15.0 / 112.0, -1.0 / 64.0}}},
  // wc4
  {{11, {64.0 / 495.0, 0.0, 0.0, -1.0 / 3.0, 0.0, 7.0 / 15.0, 0.0, -5.0 / 8.0, 7.0 / 12.0, -35.0 / 144.0, 1.0 / 20.0, -35.0 / 8448.0}}},
  // wc6
  {{14, {128.0 / 1365.0, 0.0, 0.0, -1.0 / 3.0, 0.0, 11.0 / 20.0, 0.0, -33.0 / 56.0, 0.0, 77.0 / 96.0, -33.0 / 40.0, 105.0 / 256.0, -11.0 / 96.0, 231.0 / 13312.0, -1.0 / 896.0}}},
};

// The parts of the edge and sector values that depend on eta only: with
// a_p = c_p/(p + 2) and b_p = s_p/(p - 1),
//   flux:     lead = -sum_p a_p eta^{p+2}, sector = sum_p a_p cutoff^{p+2} + lead
//   antigrad: lead = s_0 - sum_{p>=3} b_p eta^p,
//             sector = lead + eta (sum_{p>=3} b_p cutoff^{p-1} - s_0/cutoff)
// (the sector formulas above, regrouped); the line primitive is then
// sum_p a_p K_{p+2} + lead K_0 or lead K_0 + eta sum_{p>=3} b_p K_{p-1}.
struct EdgeCoef {
  double lead, sector;
};
EdgeCoef edge_coef(const KernelPiece& kp, const TailPiece3& tp, bool antigrad,
                   double eta) {
  EdgeCoef e{0.0, 0.0};
  if (!antigrad) {
    double ep = eta * eta, cp = kp.cutoff * kp.cutoff, cut = 0.0;
    for (int p = 0; p <= kp.deg; ++p) {
      const double a = kp.c[p] * kInv[p + 2];
      e.lead -= a * ep;
      cut += a * cp;
      ep *= eta;
      cp *= kp.cutoff;
    }
    e.sector = cut + e.lead;
    return e;
  }
  double ep = eta * eta * eta, cp = kp.cutoff * kp.cutoff, cut = 0.0;
  e.lead = tp.s[0];
  for (int p = 3; p <= tp.deg; ++p) {
    const double b = tp.s[p] * kInv[p - 1];
    e.lead -= b * ep;
    cut += b * cp;
    ep *= eta;
    cp *= kp.cutoff;
  }
  e.sector = e.lead + eta * (cut - tp.s[0] / kp.cutoff);
  return e;
}

double edge_primitive(const KernelPiece& kp, const TailPiece3& tp,
                      const EdgeCoef& ec, bool antigrad, double eta,
                      double delta, double beta2, double beta, double z) {
  const double rho = std::sqrt(z * z + beta2);
  const double A =
      is_tiny(delta)
          ? 0.0
          : std::atan2(delta * z * (rho - eta), delta * delta * rho + z * z * eta);
  const double L =
      is_tiny(beta)
          ? 0.0
          : std::copysign(std::log1p((std::abs(z) + z * z / (rho + beta)) / beta), z);
  const int kmax = antigrad ? std::max(tp.deg - 1, 1) : kp.deg + 2;
  double J[16], K[16];
  J[0] = z;
  J[1] = (z * rho + beta2 * L) * 0.5;
  double rp = rho;
  for (int k = 2; k <= kmax; ++k) {
    rp *= rho;
    J[k] = (z * rp + k * beta2 * J[k - 2]) * kInv[k + 1];
  }
  K[0] = A;
  K[1] = delta * L;
  for (int k = 2; k <= kmax; ++k) K[k] = delta * J[k - 2] + eta * eta * K[k - 2];
  double s = 0.0;
  if (!antigrad) {
    for (int p = 0; p <= kp.deg; ++p) s += kp.c[p] * kInv[p + 2] * K[p + 2];
    return s + ec.lead * K[0];
  }
  for (int p = 3; p <= tp.deg; ++p) s += tp.s[p] * kInv[p - 1] * K[p - 1];
  return ec.lead * K[0] + eta * s;
}

// unit_triangle_integral (kernel.hpp:316-399) for one piece; v = the three
// projected vertices (2 doubles each).
double unit_triangle_piece(const KernelPiece& kp, const TailPiece3& tp,
                           bool antigrad, double eta, const double* v) {
  if (eta >= kp.cutoff) return 0.0;
  const double radius2 = kp.cutoff * kp.cutoff - eta * eta;
  const EdgeCoef ec = edge_coef(kp, tp, antigrad, eta);
  double total = 0.0;
  for (int e = 0; e < 3; ++e) {
    const double* p0 = v + 2 * e;
    const double* p1 = v + 2 * ((e + 1) % 3);
    const double edge[2] = {p1[0] - p0[0], p1[1] - p0[1]};
    const double len2 = norm2(edge, 2);
    if (len2 <= tiny_d * tiny_d) continue;
    const double len = std::sqrt(len2);
    const double t[2] = {edge[0] / len, edge[1] / len};
    const double delta = p0[0] * t[1] - p0[1] * t[0];
    const double delta2 = delta * delta;
    const double beta2 = eta * eta + delta2;
    const double beta = std::sqrt(beta2);
    const double z0 = dot(p0, t, 2);
    const double z1 = z0 + len;
    double zs[4];
    int nz = 0;
    zs[nz++] = z0;
    if (radius2 > delta2) {
      const double zc = std::sqrt(radius2 - delta2);
      if (z0 < -zc && -zc < z1) zs[nz++] = -zc;
      if (z0 < zc && zc < z1) zs[nz++] = zc;
    }
    zs[nz++] = z1;
    for (int i = 0; i + 1 < nz; ++i) {
      const double lo = zs[i], hi = zs[i + 1];
      if (is_tiny(hi - lo)) continue;
      const double mid = (lo + hi) * 0.5;
      if (mid * mid + delta2 < radius2) {
        total += edge_primitive(kp, tp, ec, antigrad, eta, delta, beta2, beta, hi) -
                 edge_primitive(kp, tp, ec, antigrad, eta, delta, beta2, beta, lo);
      } else {
        total += ec.sector * std::atan2(delta * (hi - lo), lo * hi + delta2);
      }
    }
  }
  return total;
}

double unit_triangle(int k, bool antigrad, double eta, const double* v) {
  double total = 0.0;
  for (int i = 0; i < kPieces[k].n; ++i) {
    total += unit_triangle_piece(kPieces[k].p[i], kTail3[k][i], antigrad, eta, v);
  }
  return total;
}

void cross3(const double* a, const double* b, double* out) {
  out[0] = a[1] * b[2] - a[2] * b[1];
  out[1] = a[2] * b[0] - a[0] * b[2];
  out[2] = a[0] * b[1] - a[1] * b[0];
}

// Triangle geometry (geom/triangle.hpp): wnormal = cross(b - a, c - a)/2,
// normal = normalize(wnormal); project(x): e1 = normalize(b - a),
// e2 = normalize(cross(wnormal, e1)), p_i = (dot(v_i - x, e1),
// dot(v_i - x, e2)).
struct TriFrame {
  double n[3], d, p[6];
};
TriFrame tri_frame(const double* a, const double* b, const double* c,
                   const double* x, double h) {
  const double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double ca[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  double wn[3];
  cross3(ba, ca, wn);
  for (double& w : wn) w /= 2.0;
  TriFrame F;
  normalize(wn, 3, F.n);
  double e1[3], e2[3], t[3];
  normalize(ba, 3, e1);
  cross3(wn, e1, t);
  normalize(t, 3, e2);
  const double hinv = 1.0 / h;
  const double xa[3] = {x[0] - a[0], x[1] - a[1], x[2] - a[2]};
  F.d = dot(xa, F.n, 3) * hinv;
  const double* vs[3] = {a, b, c};
  for (int i = 0; i < 3; ++i) {
    const double vx[3] = {vs[i][0] - x[0], vs[i][1] - x[1], vs[i][2] - x[2]};
    F.p[2 * i] = dot(vx, e1, 3) * hinv;
    F.p[2 * i + 1] = dot(vx, e2, 3) * hinv;
  }
  return F;
}

// Kernel::flux over a triangle: n w h^-1 unit_flux(|d|, p_a, p_b, p_c).
void tri_flux(int k, const double* a, const double* b, const double* c,
              const double* x, double h, double* out) {
  const TriFrame F = tri_frame(a, b, c, x, h);
  const double w = kernel_weight(k, 3) * (1.0 / h);
  const double s = w * unit_triangle(k, false, std::abs(F.d), F.p);
  for (int i = 0; i < 3; ++i) out[i] = F.n[i] * s;
}

// Kernel::antigrad_flux over a triangle.
double tri_antigrad_flux(int k, const double* a, const double* b,
                         const double* c, const double* x, double h) {
  const TriFrame F = tri_frame(a, b, c, x, h);
  return std::copysign(kernel_weight(k, 3), F.d) *
         unit_triangle(k, true, std::abs(F.d), F.p);
}

// Closest point of a segment to x (Segment::clamp, geom/segment.hpp:91-106).
void seg_clamp(const double* a, const double* b, const double* x, int d,
               double* q) {
  double ba[3], xa[3];
  for (int k = 0; k < d; ++k) {
    ba[k] = b[k] - a[k];
    xa[k] = x[k] - a[k];
    q[k] = a[k];
  }
  const double len2 = norm2(ba, d);
  if (is_tiny(len2)) return;
  const double t = dot(xa, ba, d) / len2;
  if (t > 1.0) {
    for (int k = 0; k < d; ++k) q[k] = b[k];
  } else if (!(t < 0.0)) {
    for (int k = 0; k < d; ++k) q[k] = a[k] + t * ba[k];
  }
}

// Closest point of a triangle to x (Triangle::clamp, geom/triangle.hpp):
// the Voronoi-region walk of Ericson, Real-Time Collision Detection 5.1.5,
// with the degenerate triangle clamped to its longest edge.
void tri_clamp(const double* a, const double* b, const double* c,
               const double* x, double* q) {
  const double ba[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double ca[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double cb[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
  double wn[3];
  cross3(ba, ca, wn);
  for (double& w : wn) w /= 2.0;
  if (is_tiny(norm(wn, 3))) {
    const double l_ab = norm2(ba, 3), l_bc = norm2(cb, 3), l_ca = norm2(ca, 3);
    if (l_ab >= l_bc && l_ab >= l_ca) return seg_clamp(a, b, x, 3, q);
    if (l_bc >= l_ca) return seg_clamp(b, c, x, 3, q);
    return seg_clamp(a, c, x, 3, q);
  }
  auto set = [q](const double* p) { q[0] = p[0]; q[1] = p[1]; q[2] = p[2]; };
  const double pa[3] = {x[0] - a[0], x[1] - a[1], x[2] - a[2]};
  const double d1 = dot(ba, pa, 3), d2 = dot(ca, pa, 3);
  if (d1 <= 0.0 && d2 <= 0.0) return set(a);
  const double pb[3] = {x[0] - b[0], x[1] - b[1], x[2] - b[2]};
  const double d3 = dot(ba, pb, 3), d4 = dot(ca, pb, 3);
  if (d3 >= 0.0 && d4 <= d3) return set(b);
  const double pc[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
  const double d5 = dot(ba, pc, 3), d6 = dot(ca, pc, 3);
  if (d6 >= 0.0 && d5 <= d6) return set(c);
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) {
    const double t = d1 / (d1 - d3);
    for (int k = 0; k < 3; ++k) q[k] = a[k] + t * ba[k];
    return;
  }
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) {
    const double t = d2 / (d2 - d6);
    for (int k = 0; k < 3; ++k) q[k] = a[k] + t * ca[k];
    return;
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0.0 && d4 >= d3 && d5 >= d6) {
    const double t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    for (int k = 0; k < 3; ++k) q[k] = b[k] + t * cb[k];
    return;
  }
  const double v = vb / (va + vb + vc);
  const double w = vc / (va + vb + vc);
  for (int k = 0; k < 3; ++k) q[k] = a[k] + v * ba[k] + w * ca[k];
}

// Triangle::intersects(BSphere): boxes overlap and the closest point of the
// triangle is in the sphere.
bool tri_in_sphere(const double* a, const double* b, const double* c,
                   const double* x, double radius) {
  for (int k = 0; k < 3; ++k) {
    const double lo = std::min(std::min(a[k], b[k]), c[k]);
    const double hi = std::max(std::max(a[k], b[k]), c[k]);
    if (!(x[k] - radius <= hi && lo <= x[k] + radius)) return false;
  }
  double q[3];
  tri_clamp(a, b, c, x, q);
  const double d[3] = {q[0] - x[0], q[1] - x[1], q[2] - x[2]};
  return norm2(d, 3) <= radius * radius;
}

// Exact generalized winding number of a closed triangle mesh at x
// (Triangle::winding_number, geom/triangle.hpp, summed over the mesh):
// per triangle atan2(det(a', b', c'), |a'||b'||c'| + (a'.b')|c'| +
// (b'.c')|a'| + (c'.a')|b'|) / (2 pi), primes = vertex - x (the solid
// angle formula of Van Oosterom and Strackee).  tris: 9 doubles each.
double winding_number3(int32_t n_tris, const double* tris, const double* x) {
  double w = 0.0;
  for (int32_t i = 0; i < n_tris; ++i) {
    const double* t = tris + 9 * static_cast<int64_t>(i);
    const double ap[3] = {t[0] - x[0], t[1] - x[1], t[2] - x[2]};
    const double bp[3] = {t[3] - x[0], t[4] - x[1], t[5] - x[2]};
    const double cp[3] = {t[6] - x[0], t[7] - x[1], t[8] - x[2]};
    const double na = norm(ap, 3), nb = norm(bp, 3), nc = norm(cp, 3);
    const double den = na * nb * nc + dot(ap, bp, 3) * nc +
                       dot(bp, cp, 3) * na + dot(cp, ap, 3) * nb;
    double bc[3];
    cross3(bp, cp, bc);
    w += std::atan2(dot(ap, bc, 3), den) / (2.0 * std::numbers::pi);
  }
  return w;
}

template<class Num>
struct Kern {
  int id;
  int dim;
  Num h;
  Num w;       // weight * h^-d
  Num hinv;
  Num radius;  // unit_radius * h
  Kern(int k, int d, Num h_) : id{k}, dim{d}, h{h_} {
    hinv = Num{1} / h;
    w = static_cast<Num>(kernel_weight(k, d)) * ipow(hinv, d);
    radius = static_cast<Num>(kernel_table[k].unit_radius) * h;
  }
  // kernel.hpp:142-151
  Num value(const Num* x) const {
    const Num q = hinv * norm(x, dim);
    return w * unit_value(id, q);
  }
  // kernel.hpp:154-163
  void grad(const Num* x, Num* out) const {
    const Num q = hinv * norm(x, dim);
    Num n[3];
    normalize(x, dim, n);
    const Num s = w * unit_deriv(id, q);
    for (int i = 0; i < dim; ++i) out[i] = s * (n[i] * hinv);
  }
};

// ---------------------------------------------------------------------------
// Tait EOS, sph/equation_of_state.hpp:37-64.

struct Tait {
  double rho0, cs0, xi;
  // LinearTaitEquationOfState (equation_of_state.hpp:78-122): p = cs0^2
  // (rho - rho0), c = cs0, H = cs0^2 log(rho / rho0).
  bool linear = false;
  double pressure(double rho) const {
    if (linear) return pow2(cs0) * (rho - rho0);
    const double B = rho0 * pow2(cs0) / xi;
    return B * (std::pow(rho / rho0, xi) - 1.0);
  }
  double sound_speed(double rho) const {
    if (linear) return cs0;
    return cs0 * std::pow(rho / rho0, (xi - 1.0) / 2.0);
  }
  double potential(double rho) const {
    if (linear) return pow2(cs0) * std::log(rho / rho0);
    const double xi_1 = xi - 1.0;
    return pow2(cs0) * (std::pow(rho / rho0, xi_1) - 1.0) / xi_1;
  }
  double density_from_potential(double H) const {
    if (linear) return rho0 * std::exp(H / pow2(cs0));
    const double xi_1 = xi - 1.0;
    return rho0 * std::pow(1.0 + xi_1 * H / pow2(cs0), 1.0 / xi_1);
  }
};

// ---------------------------------------------------------------------------
// Uniform grid index, geom/search/grid_search.hpp:45-102 and geom/grid.hpp.

template<class Num>
struct GridIndex {
  int dim = 0;
  int64_t n = 0;
  const Num* pts = nullptr;
  Num low[3]{}, high[3]{};
  Num cell_ext[3]{}, inv_ext[3]{};
  int64_t ncell[3]{1, 1, 1};
  std::vector<int64_t> offsets;
  std::vector<int32_t> points;

  int64_t cell_coord(int i, Num x) const {
    // grid.hpp:105-112: truncation of (point - origin) * inv_extents.
    return static_cast<int64_t>((x - low[i]) * inv_ext[i]);
  }
  int64_t flatten(const int64_t* c) const {
    // grid.hpp:120-128: last coordinate fastest.
    int64_t f = c[0];
    for (int i = 1; i < dim; ++i) f = ncell[i] * f + c[i];
    return f;
  }

  GridIndex(int d, int64_t np, const Num* p, Num size_hint)
      : dim{d}, n{np}, pts{p} {
    if (n == 0) return;
    // bbox, grown by size_hint / 2 (grid_search.hpp:55).
    for (int i = 0; i < dim; ++i) low[i] = high[i] = pts[i];
    for (int64_t a = 1; a < n; ++a) {
      for (int i = 0; i < dim; ++i) {
        low[i] = std::min(low[i], pts[a * dim + i]);
        high[i] = std::max(high[i], pts[a * dim + i]);
      }
    }
    const Num grow = size_hint / Num{2};
    for (int i = 0; i < dim; ++i) {
      low[i] -= grow;
      high[i] += grow;
    }
    // set_cell_extents (grid.hpp:90-98).
    int64_t total = 1;
    for (int i = 0; i < dim; ++i) {
      const Num ext = high[i] - low[i];
      const Num ncf = std::max(std::ceil(ext / size_hint), Num{1});
      ncell[i] = static_cast<int64_t>(ncf);
      cell_ext[i] = ext / ncf;
      inv_ext[i] = Num{1} / cell_ext[i];
      total *= ncell[i];
    }
    // Count, prefix sum, fill (grid_search.hpp:58-84); the fill here is
    // sequential, so each cell lists its points in ascending order.
    offsets.assign(static_cast<size_t>(total + 1), 0);
    std::vector<int64_t> cell_of(static_cast<size_t>(n));
    for (int64_t a = 0; a < n; ++a) {
      int64_t c[3];
      for (int i = 0; i < dim; ++i) c[i] = cell_coord(i, pts[a * dim + i]);
      cell_of[a] = flatten(c);
      offsets[cell_of[a] + 1] += 1;
    }
    for (int64_t c = 0; c < total; ++c) offsets[c + 1] += offsets[c];
    points.resize(static_cast<size_t>(n));
    std::vector<int64_t> fill(offsets.begin(), offsets.end() - 1);
    for (int64_t a = 0; a < n; ++a) {
      points[fill[cell_of[a]]++] = static_cast<int32_t>(a);
    }
  }

  // search() with BSphere::contains (bsphere.hpp:52-54) over
  // cells_intersecting (grid.hpp:160-169).  Appends to out (unsorted).
  void search(const Num* center, Num radius, std::vector<int32_t>& out) const {
    if (n == 0) return;
    int64_t lo[3]{0, 0, 0}, hi[3]{0, 0, 0};
    for (int i = 0; i < dim; ++i) {
      const Num half = cell_ext[i] / Num{2};
      Num bl = center[i] - radius - half;
      Num bh = center[i] + radius + half;
      bl = std::max(bl, low[i]);
      bh = std::min(bh, high[i]);
      bl += half;
      bh -= half;
      lo[i] = cell_coord(i, bl);
      hi[i] = cell_coord(i, bh);
    }
    const Num r2 = pow2(radius);
    int64_t c[3];
    for (c[0] = lo[0]; c[0] <= hi[0]; ++c[0]) {
      for (c[1] = lo[1]; c[1] <= (dim > 1 ? hi[1] : lo[1]); ++c[1]) {
        for (c[2] = lo[2]; c[2] <= (dim > 2 ? hi[2] : lo[2]); ++c[2]) {
          const int64_t f = flatten(c);
          for (int64_t j = offsets[f]; j < offsets[f + 1]; ++j) {
            const int32_t b = points[j];
            Num dvec[3];
            for (int i = 0; i < dim; ++i) {
              dvec[i] = pts[b * dim + i] - center[i];
            }
            if (norm2(dvec, dim) <= r2) out.push_back(b);
          }
        }
      }
    }
  }
};

// Adjacency in CSR form, rows sorted ascending (particle_mesh.hpp:137-147).
struct Adjacency {
  std::vector<int64_t> off;
  std::vector<int32_t> idx;
  int64_t size(int64_t a) const { return off[a + 1] - off[a]; }
};

template<class Num>
void build_adjacency(int dim, int64_t n, const Num* r, Num radius,
                     Num size_hint, int32_t nthreads, Adjacency& adj) {
  adj.off.assign(static_cast<size_t>(n + 1), 0);
  adj.idx.clear();
  if (n == 0) return;
  const GridIndex<Num> grid(dim, n, r, size_hint);
  std::vector<std::vector<int32_t>> rows(static_cast<size_t>(n));
  parallel_for(n, nthreads, [&](int64_t a) {
    auto& row = rows[a];
    grid.search(r + a * dim, radius, row);
    std::sort(row.begin(), row.end());
  });
  for (int64_t a = 0; a < n; ++a) {
    adj.off[a + 1] = adj.off[a] + static_cast<int64_t>(rows[a].size());
  }
  adj.idx.resize(static_cast<size_t>(adj.off[n]));
  parallel_for(n, nthreads, [&](int64_t a) {
    std::copy(rows[a].begin(), rows[a].end(), adj.idx.begin() + adj.off[a]);
  });
}

int64_t export_csr(const Adjacency& adj, int64_t n, int64_t* offsets,
                   int32_t* indices, int64_t capacity) {
  const int64_t total = adj.off[n];
  if (offsets != nullptr) {
    std::memcpy(offsets, adj.off.data(), sizeof(int64_t) * (n + 1));
  }
  if (indices != nullptr && capacity >= total && total > 0) {
    std::memcpy(indices, adj.idx.data(), sizeof(int32_t) * total);
  }
  return total;
}

// ---------------------------------------------------------------------------
// FluidEquations (fluid_equations.hpp:79-512).  With particle walls (no
// boundary faces, an always-true containment) gamma = 1 and grad_gamma = 0
// everywhere (:166-193) and every face term vanishes.  With faces
// (segments in 2D, triangles in 3D) the tank's fixed particles are the face
// vertices; gamma, grad_gamma, the face terms and the gamma-divided pair
// sums follow the reference.

struct TankView {
  int64_t nf = 0, nw = 0, n = 0;
  double h = 0, m = 0;
  Tait eos{};
  double* r = nullptr;
  double* v = nullptr;
  double* rho = nullptr;
  double* drho = nullptr;
  double* dv = nullptr;
  // Boundary faces: dim vertex indices per face into the tank's fixed
  // particles.  Containment: in 2D a closed loop of n_poly vertices, in 3D
  // n_poly triangles (9 doubles each) of a closed, outward-oriented mesh.
  int32_t n_faces = 0;
  const int32_t* face_verts = nullptr;
  int32_t n_poly = 0;
  const double* poly = nullptr;
};

struct Solver {
  const tg_params& P;
  int dim;
  int32_t nthreads;
  TankView& T;
  Kern<double> K;
  Adjacency adj;
  std::vector<double> p, cs;
  std::vector<double> gamma, ggam;           // gamma and grad gamma
  std::vector<std::vector<int32_t>> fadj;    // adjacent faces, ascending

  Solver(const tg_params& params, TankView& tank, int32_t nt)
      : P{params}, dim{params.dim}, nthreads{nt}, T{tank},
        K{params.kernel, params.dim, tank.h} {
    p.assign(static_cast<size_t>(T.n), 0.0);
    cs.assign(static_cast<size_t>(T.n), 0.0);
    gamma.assign(static_cast<size_t>(T.n), 1.0);
    ggam.assign(static_cast<size_t>(T.n * dim), 0.0);
    fadj.assign(static_cast<size_t>(T.n), {});
  }

  bool faces() const { return T.n_faces > 0; }
  const double* vert(int32_t f, int i) const {
    return T.r + (T.nf + T.face_verts[dim * f + i]) * dim;
  }
  int64_t vert_index(int32_t f, int i) const {
    return T.nf + T.face_verts[dim * f + i];
  }
  // Field of a face's vertices: avg (field.hpp:59-64, core/math.hpp:130),
  // (a + b)/2 or (a + b + c)/3.
  double face_avg(const double* fld, int32_t f) const {
    if (dim == 2) return (fld[vert_index(f, 0)] + fld[vert_index(f, 1)]) / 2.0;
    return (fld[vert_index(f, 0)] + fld[vert_index(f, 1)] + fld[vert_index(f, 2)]) / 3.0;
  }
  double face_avg(const std::vector<double>& fld, int32_t f) const {
    return face_avg(fld.data(), f);
  }
  double face_avg_vec(const double* fld, int32_t f, int k) const {
    if (dim == 2) {
      return (fld[vert_index(f, 0) * dim + k] + fld[vert_index(f, 1) * dim + k]) / 2.0;
    }
    return (fld[vert_index(f, 0) * dim + k] + fld[vert_index(f, 1) * dim + k] +
            fld[vert_index(f, 2) * dim + k]) / 3.0;
  }
  // Kernel::flux / antigrad_flux of face f at x, and face-sphere overlap.
  void flux(int32_t f, const double* x, double* out) const {
    if (dim == 2) return face_flux(P.kernel, vert(f, 0), vert(f, 1), x, T.h, out);
    tri_flux(P.kernel, vert(f, 0), vert(f, 1), vert(f, 2), x, T.h, out);
  }
  double antigrad_flux(int32_t f, const double* x) const {
    if (dim == 2) return face_antigrad_flux(P.kernel, vert(f, 0), vert(f, 1), x, T.h);
    return tri_antigrad_flux(P.kernel, vert(f, 0), vert(f, 1), vert(f, 2), x, T.h);
  }
  bool in_sphere(int32_t f, const double* x) const {
    if (dim == 2) return face_in_sphere(vert(f, 0), vert(f, 1), x, K.radius);
    return tri_in_sphere(vert(f, 0), vert(f, 1), vert(f, 2), x, K.radius);
  }
  // FastWindingFunc::contains (fast_winding.hpp:80-95): winding > 1/2, here
  // with the exact winding number.
  bool contains(const double* x) const {
    if (dim == 2) return winding_number(T.n_poly, T.poly, x) > 0.5;
    return winding_number3(T.n_poly, T.poly, x) > 0.5;
  }

  // ParticleMesh face adjacency (particle_mesh.hpp:149-161): faces within
  // the search sphere, sorted.
  void index_faces() {
    parallel_for(T.n, nthreads, [&](int64_t a) {
      auto& out = fadj[a];
      out.clear();
      for (int32_t fi = 0; fi < T.n_faces; ++fi) {
        if (in_sphere(fi, T.r + a * dim)) out.push_back(fi);
      }
    });
  }

  // FluidEquations::compute_gamma (fluid_equations.hpp:166-193).
  void compute_gamma() {
    parallel_for(T.n, nthreads, [&](int64_t a) {
      double* g = &ggam[a * dim];
      for (int k = 0; k < dim; ++k) g[k] = 0.0;
      for (int32_t fi : fadj[a]) {
        double fl[3];
        flux(fi, T.r + a * dim, fl);
        for (int k = 0; k < dim; ++k) g[k] += fl[k];
      }
      double ga = contains(T.r + a * dim) ? 1.0 : 0.0;
      const double ng = norm(g, dim);
      if (!is_tiny(ng)) {
        const double s = (2.0 * ga - 1.0);
        double r_a[3];
        for (int k = 0; k < dim; ++k) {
          r_a[k] = T.r[a * dim + k] + s * (g[k] / ng) * pow2(T.h);
        }
        for (int32_t fi : fadj[a]) ga -= antigrad_flux(fi, r_a);
      }
      gamma[a] = ga;
    });
  }

  bool is_fluid(int64_t a) const { return a < T.nf; }

  // FluidEquations::index (fluid_equations.hpp:112-115) with
  // GridSearch{h} as in wcsph.cpp:147.
  void index() {
    build_adjacency<double>(dim, T.n, T.r, K.radius, T.h, nthreads, adj);
  }

  // FluidEquations::setup_boundary (fluid_equations.hpp:122-164).  With
  // particle walls grad_gamma = 0, so the normal n_e is zero and the
  // hydrostatic term vanishes.
  void setup_boundary() {
    parallel_for(T.nw, nthreads, [&](int64_t i) {
      const int64_t e = T.nf + i;
      for (int k = 0; k < dim; ++k) T.v[e * dim + k] = 0.0;
      double S_e = 0.0, H_e = 0.0;
      double n_e[3] = {0.0, 0.0, 0.0};
      normalize(&ggam[e * dim], dim, n_e);
      for (int64_t j = adj.off[e]; j < adj.off[e + 1]; ++j) {
        const int64_t b = adj.idx[j];
        if (!is_fluid(b)) continue;
        const double V_b = T.m / T.rho[b];
        double r_be[3];
        for (int k = 0; k < dim; ++k) {
          r_be[k] = T.r[b * dim + k] - T.r[e * dim + k];
        }
        const double W_be = K.value(r_be);
        const double H_b = T.eos.potential(T.rho[b]);
        S_e += V_b * W_be;
        H_e += V_b * (H_b + P.g * dot(r_be, n_e, dim) * n_e[1]) * W_be;
      }
      T.rho[e] = T.eos.density_from_potential(is_tiny(S_e) ? 0.0 : H_e / S_e);
    });
  }

  // FluidEquations::prepare (fluid_equations.hpp:99-105).
  void prepare() {
    index();
    if (faces()) {
      index_faces();
      compute_gamma();
    }
    setup_boundary();
  }

  // FluidEquations::compute_time_step (fluid_equations.hpp:199-222).
  double compute_time_step() const {
    double dt = std::numeric_limits<double>::max();
    for (int64_t a = 0; a < T.nf; ++a) {
      const double dt_acoustic =
          P.cfl * T.h /
          (T.eos.sound_speed(T.rho[a]) + norm(T.v + a * dim, dim));
      const double dt_visc = P.c_visc * pow2(T.h) * T.rho[a] / P.mu;
      const double dt_force =
          P.c_force * std::sqrt(T.h / std::max(norm(T.dv + a * dim, dim), P.g));
      dt = std::min({dt, dt_acoustic, dt_visc, dt_force});
    }
    return dt;
  }

  void compute_eos() {
    parallel_for(T.n, nthreads, [&](int64_t a) {
      cs[a] = T.eos.sound_speed(T.rho[a]);
      p[a] = T.eos.pressure(T.rho[a]);
    });
  }

  // FluidEquations::compute_continuity (fluid_equations.hpp:232-260).
  // Ferrari: Psi_ab = max(cs_a, cs_b) (rho_a - rho_b) r_ab / |r_ab|.
  // delta-SPH (Molteni & Colagrossi 2009, restated; no reference code):
  //   2 delta h cs_0 (rho_a - rho_b) (r_ab . grad W_ab) / |r_ab|^2 / rho_b.
  void compute_continuity() {
    compute_eos();
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      double acc = 0.0;
      // Face terms (fluid_equations.hpp:241-247).
      for (int32_t fi : fadj[a]) {
        double gg[3], v_as[3];
        flux(fi, T.r + a * dim, gg);
        for (int k = 0; k < dim; ++k) v_as[k] = T.v[a * dim + k] - face_avg_vec(T.v, fi, k);
        acc -= face_avg(T.rho, fi) * dot(v_as, gg, dim) / gamma[a];
      }
      for (int64_t j = adj.off[a]; j < adj.off[a + 1]; ++j) {
        const int64_t b = adj.idx[j];
        if (b == a) continue;
        double r_ab[3] = {}, v_ab[3] = {}, gW[3] = {};
        for (int k = 0; k < dim; ++k) {
          r_ab[k] = T.r[a * dim + k] - T.r[b * dim + k];
          v_ab[k] = T.v[a * dim + k] - T.v[b * dim + k];
        }
        K.grad(r_ab, gW);
        const double rho_ab = T.rho[a] - T.rho[b];
        if (P.diffusion == TG_DIFF_FERRARI) {
          const double cs_ab = std::max(cs[a], cs[b]);
          const double nr = norm(r_ab, dim);
          double w[3];
          for (int k = 0; k < dim; ++k) {
            const double Psi = cs_ab * rho_ab * r_ab[k] / nr;
            w[k] = v_ab[k] + Psi / T.rho[b];
          }
          acc += T.m / gamma[a] * dot(w, gW, dim);
        } else if (P.diffusion == TG_DIFF_MOLTENI) {
          const double D = 2.0 * P.delta * T.h * T.eos.cs0 * rho_ab / T.rho[b] *
                           dot(r_ab, gW, dim) / norm2(r_ab, dim);
          acc += T.m / gamma[a] * (dot(v_ab, gW, dim) + D);
        } else {
          acc += T.m / gamma[a] * dot(v_ab, gW, dim);
        }
      }
      T.drho[a] = acc;
    });
  }

  // FluidEquations::compute_momentum (fluid_equations.hpp:267-305).
  // Morris: Pi_ab = 2 mu (v_ab . r_ab) / (rho_a rho_b |r_ab|^2).
  // Monaghan (1992, restated; no reference code): for v_ab . r_ab < 0,
  //   Pi_ab = alpha c_ab mu_ab / rho_ab, mu_ab = h v_ab.r_ab/(|r_ab|^2+0.01h^2)
  //   with arithmetic means c_ab, rho_ab; it enters as the reference's Pi.
  void compute_momentum() {
    compute_eos();
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      double acc[3] = {0.0, 0.0, 0.0};
      acc[1] = -P.g;  // unit<1>(r[a], -g)
      // Face terms: wall pressure and wall shear (fluid_equations.hpp:278-291).
      for (int32_t fi : fadj[a]) {
        double gg[3];
        flux(fi, T.r + a * dim, gg);
        const double rho_s = face_avg(T.rho, fi);
        const double p_s = face_avg(p, fi);
        const double P_as =
            rho_s * (p[a] / pow2(T.rho[a]) + p_s / pow2(rho_s));
        double n_s[3], t_as[3], v_as[3], vt[3], r_as[3];
        normalize(gg, dim, n_s);
        for (int k = 0; k < dim; ++k) v_as[k] = T.v[a * dim + k] - face_avg_vec(T.v, fi, k);
        const double vn = dot(v_as, n_s, dim);
        for (int k = 0; k < dim; ++k) vt[k] = v_as[k] - vn * n_s[k];
        normalize(vt, dim, t_as);
        for (int k = 0; k < dim; ++k) r_as[k] = T.r[a * dim + k] - face_avg_vec(T.r, fi, k);
        const double dr_as = std::max(T.h / 2.0, dot(r_as, n_s, dim));
        const double Pi_s =
            2.0 * P.mu / (T.rho[a] * dr_as) * dot(v_as, t_as, dim);
        const double ng = norm(gg, dim);
        for (int k = 0; k < dim; ++k) {
          acc[k] += (P_as * gg[k] - Pi_s * t_as[k] * ng) / gamma[a];
        }
      }
      for (int64_t j = adj.off[a]; j < adj.off[a + 1]; ++j) {
        const int64_t b = adj.idx[j];
        if (b == a) continue;
        double r_ab[3] = {}, v_ab[3] = {}, gW[3] = {};
        for (int k = 0; k < dim; ++k) {
          r_ab[k] = T.r[a * dim + k] - T.r[b * dim + k];
          v_ab[k] = T.v[a * dim + k] - T.v[b * dim + k];
        }
        K.grad(r_ab, gW);
        const double P_ab =
            p[a] / pow2(T.rho[a]) + p[b] / pow2(T.rho[b]);
        double Pi_ab = 0.0;
        if (P.viscosity == TG_VISC_MORRIS) {
          Pi_ab = 2.0 * P.mu * dot(v_ab, r_ab, dim) /
                  (T.rho[a] * T.rho[b] * norm2(r_ab, dim));
        } else {
          const double vr = dot(v_ab, r_ab, dim);
          if (vr < 0.0) {
            const double mu_ab =
                T.h * vr / (norm2(r_ab, dim) + 0.01 * pow2(T.h));
            const double c_ab = 0.5 * (cs[a] + cs[b]);
            const double rho_m = 0.5 * (T.rho[a] + T.rho[b]);
            Pi_ab = P.alpha * c_ab * mu_ab / rho_m;
          }
        }
        const double s = T.m / gamma[a] * (Pi_ab - P_ab);
        for (int k = 0; k < dim; ++k) acc[k] += s * gW[k];
      }
      for (int k = 0; k < dim; ++k) T.dv[a * dim + k] = acc[k];
    });
  }

  // ---- post-integration (fluid_equations.hpp:315-512) ---------------------
  static constexpr double phi_max = 1.0;
  static constexpr double phi_min = std::numeric_limits<double>::min();

  static bool bits_equal(double a, double b) {
    uint64_t x, y;
    std::memcpy(&x, &a, 8);
    std::memcpy(&y, &b, 8);
    return x == y;
  }

  // LU without pivoting with the is_tiny pivot test (core/_mat/fact.hpp),
  // then inverse by forward/backward substitution of the identity.
  static bool lu_inverse(const double* A, int d, double* inv) {
    double LU[9];
    for (int i = 0; i < d; ++i) {
      for (int j = 0; j < i; ++j) {
        double s = A[i * d + j];
        for (int k = 0; k < j; ++k) s -= LU[i * d + k] * LU[k * d + j];
        LU[i * d + j] = s / LU[j * d + j];
      }
      for (int j = i; j < d; ++j) {
        double s = A[i * d + j];
        for (int k = 0; k < i; ++k) s -= LU[i * d + k] * LU[k * d + j];
        LU[i * d + j] = s;
      }
      if (is_tiny(LU[i * d + i])) return false;
    }
    for (int c = 0; c < d; ++c) {
      double x[3];
      for (int i = 0; i < d; ++i) x[i] = (i == c) ? 1.0 : 0.0;
      for (int i = 0; i < d; ++i) {
        for (int k = 0; k < i; ++k) x[i] -= LU[i * d + k] * x[k];
      }
      for (int i = d - 1; i >= 0; --i) {
        for (int k = i + 1; k < d; ++k) x[i] -= LU[i * d + k] * x[k];
        x[i] /= LU[i * d + i];
      }
      for (int i = 0; i < d; ++i) inv[i * d + c] = x[i];
    }
    return true;
  }

  // apply_shifts (fluid_equations.hpp:331-471) restricted to fluid targets;
  // the fixed particles' N, L, grad_v, grad_rho are never read.
  void apply_shifts() {
    const int64_t n = T.n;
    const int d = dim;
    std::vector<double> N(n * d, 0.0), L(n * d * d, 0.0), gv(n * d * d, 0.0),
        gr(n * d, 0.0), dr(n * d, 0.0), phi(n, 0.0);
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      double* Na = &N[a * d];
      double* La = &L[a * d * d];
      double* gva = &gv[a * d * d];
      double* gra = &gr[a * d];
      // Face terms (fluid_equations.hpp:340-349).
      for (int32_t fi : fadj[a]) {
        double gg[3];
        flux(fi, T.r + a * d, gg);
        double r_sa[3], v_sa[3];
        for (int k = 0; k < d; ++k) {
          r_sa[k] = face_avg_vec(T.r, fi, k) - T.r[a * d + k];
          v_sa[k] = face_avg_vec(T.v, fi, k) - T.v[a * d + k];
        }
        const double rho_sa = face_avg(T.rho, fi) - T.rho[a];
        for (int i = 0; i < d; ++i) {
          Na[i] -= gg[i] / gamma[a];
          for (int k = 0; k < d; ++k) {
            La[i * d + k] -= r_sa[i] * gg[k] / gamma[a];
            gva[i * d + k] -= v_sa[i] * gg[k] / gamma[a];
          }
          gra[i] -= rho_sa * gg[i] / gamma[a];
        }
      }
      for (int64_t j = adj.off[a]; j < adj.off[a + 1]; ++j) {
        const int64_t b = adj.idx[j];
        if (b == a) continue;
        double r_ab[3] = {}, r_ba[3] = {}, v_ba[3] = {}, gW[3] = {};
        for (int k = 0; k < d; ++k) {
          r_ab[k] = T.r[a * d + k] - T.r[b * d + k];
          r_ba[k] = T.r[b * d + k] - T.r[a * d + k];
          v_ba[k] = T.v[b * d + k] - T.v[a * d + k];
        }
        K.grad(r_ab, gW);
        const double V_b = T.m / T.rho[b];
        const double s = V_b / gamma[a];
        const double rho_ba = T.rho[b] - T.rho[a];
        for (int i = 0; i < d; ++i) {
          Na[i] += s * gW[i];
          for (int k = 0; k < d; ++k) {
            La[i * d + k] += s * (r_ba[i] * gW[k]);
            gva[i * d + k] += s * (v_ba[i] * gW[k]);
          }
          gra[i] += s * rho_ba * gW[i];
        }
      }
      // dr = N; renormalise with inverse(transpose(L)) (:366-377).
      for (int i = 0; i < d; ++i) dr[a * d + i] = Na[i];
      double LT[9], Li[9];
      for (int i = 0; i < d; ++i) {
        for (int k = 0; k < d; ++k) LT[i * d + k] = La[k * d + i];
      }
      if (lu_inverse(LT, d, Li)) {
        double tN[3], tg[3], tgv[9];
        for (int i = 0; i < d; ++i) {
          tN[i] = 0.0;
          tg[i] = 0.0;
          for (int k = 0; k < d; ++k) {
            tN[i] += Li[i * d + k] * Na[k];
            tg[i] += Li[i * d + k] * gra[k];
          }
        }
        // grad_v * transpose(Li)
        for (int i = 0; i < d; ++i) {
          for (int k = 0; k < d; ++k) {
            double s2 = 0.0;
            for (int l = 0; l < d; ++l) s2 += gva[i * d + l] * Li[k * d + l];
            tgv[i * d + k] = s2;
          }
        }
        for (int i = 0; i < d; ++i) {
          Na[i] = tN[i];
          gra[i] = tg[i];
        }
        for (int i = 0; i < d * d; ++i) gva[i] = tgv[i];
      }
      double nn[3];
      normalize(Na, d, nn);
      for (int i = 0; i < d; ++i) Na[i] = nn[i];
    });

    // Free-surface classification (:387-416): a fluid particle leaves
    // phi_min when some neighbour lies in its 45-degree "outside" cone.
    parallel_for(T.n, nthreads, [&](int64_t a) {
      phi[a] = is_fluid(a) ? phi_min : phi_max;
    });
    const double cos_fov = std::cos(std::numbers::pi / 4.0);
    std::vector<double> phi_c(phi);
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      bool visible = false;
      for (int64_t j = adj.off[a]; j < adj.off[a + 1] && !visible; ++j) {
        const int64_t b = adj.idx[j];
        if (b == a) continue;
        double r_ab[3] = {};
        for (int k = 0; k < d; ++k) {
          r_ab[k] = T.r[a * d + k] - T.r[b * d + k];
        }
        const double r2_ab = norm2(r_ab, d);
        const double thr = (K.radius + K.radius) / 2.0;
        if (r2_ab > pow2(thr)) continue;
        const double fov_threshold = pow2(cos_fov) * r2_ab;
        const double n_a = dot(&N[a * d], r_ab, d);
        if (n_a > 0.0 && pow2(n_a) >= fov_threshold) visible = true;
      }
      if (visible) phi_c[a] = phi_max;
    });
    phi.swap(phi_c);
    // Splashes (:419-426).
    const int64_t cutoff = d == 2 ? 8 : 26;
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      if (adj.size(a) <= cutoff) phi[a] = phi_min;
    });
    // Near-surface scaling (:440-452); reads only phi == phi_min.
    phi_c = phi;
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      if (!bits_equal(phi[a], phi_max)) return;
      int64_t best = -1;
      double best_d2 = 0.0;
      for (int64_t j = adj.off[a]; j < adj.off[a + 1]; ++j) {
        const int64_t b = adj.idx[j];
        if (!bits_equal(phi[b], phi_min)) continue;
        double r_ab[3] = {};
        for (int k = 0; k < d; ++k) {
          r_ab[k] = T.r[a * d + k] - T.r[b * d + k];
        }
        const double d2 = norm2(r_ab, d);
        if (best < 0 || d2 < best_d2) {
          best = b;
          best_d2 = d2;
        }
      }
      if (best >= 0) {
        double r_ab[3] = {};
        for (int k = 0; k < d; ++k) {
          r_ab[k] = T.r[a * d + k] - T.r[best * d + k];
        }
        phi_c[a] = phi[a] * (std::abs(dot(&N[best * d], r_ab, d)) / K.radius);
      }
    });
    phi.swap(phi_c);
    // Shift the far particles (:455-470).
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      double* dra = &dr[a * d];
      if (!bits_equal(phi[a], phi_max)) {
        for (int i = 0; i < d; ++i) dra[i] = 0.0;
        return;
      }
      const double c = -P.cfl * 0.2 * pow2(T.h);
      for (int i = 0; i < d; ++i) dra[i] *= c;
      for (int i = 0; i < d; ++i) T.r[a * d + i] += dra[i];
      // Velocity correction only where gamma ~ 1 (:465-467).
      if (is_tiny(gamma[a] - 1.0)) {
        double dv[3];
        for (int i = 0; i < d; ++i) {
          dv[i] = dot(&gv[a * d * d + i * d], dra, d);
        }
        for (int i = 0; i < d; ++i) T.v[a * d + i] += dv[i];
      }
      T.rho[a] += dot(&gr[a * d], dra, d);
    });
    phi_.swap(phi);
  }

  // apply_free_surface_correction (fluid_equations.hpp:484-512), on the
  // adjacency of the last prepare() and the shifted positions.
  void apply_free_surface_correction() {
    std::vector<double> rho_raw(T.rho, T.rho + T.n);
    const double K_fs = -std::log(0.05) / pow2(0.01);
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      if (bits_equal(phi_[a], phi_max)) return;
      double alpha = 0.0, rho_t = 0.0;
      for (int64_t j = adj.off[a]; j < adj.off[a + 1]; ++j) {
        const int64_t b = adj.idx[j];
        double r_ab[3] = {};
        for (int k = 0; k < dim; ++k) {
          r_ab[k] = T.r[a * dim + k] - T.r[b * dim + k];
        }
        const double W_ab = K.value(r_ab);
        alpha += T.m / rho_raw[b] * W_ab;
        rho_t += T.m * W_ab;
      }
      const double ratio = std::min(1.0, alpha / gamma[a]);
      if (ratio > 0.99) return;
      const double beta = std::exp(-K_fs * pow2(ratio - 1.0));
      const double corr = beta * gamma[a] + (1.0 - beta) * alpha;
      if (!is_tiny(corr)) T.rho[a] = rho_t / corr;
    });
  }

  std::vector<double> phi_;

  void post_integrate() {
    prepare();
    if (P.post_integrate == TG_POST_SHIFTING) {
      apply_shifts();
      apply_free_surface_correction();
    }
  }

  // ---- integrators (time_integrator.hpp) ----------------------------------
  void euler_update(double dt) {
    // time_integrator.hpp:203-207: r uses the velocity before its update.
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      for (int k = 0; k < dim; ++k) T.r[a * dim + k] += dt * T.v[a * dim + k];
      for (int k = 0; k < dim; ++k) T.v[a * dim + k] += dt * T.dv[a * dim + k];
      T.rho[a] += dt * T.drho[a];
    });
  }

  double substep(double dt_in, bool have_dt) {
    prepare();
    const double dt = have_dt ? dt_in : compute_time_step();
    compute_continuity();
    compute_momentum();
    euler_update(dt);
    return dt;
  }

  void lincomb(const std::vector<double>& r0, const std::vector<double>& v0,
               const std::vector<double>& rho0, double w) {
    // time_integrator.hpp:212-223
    parallel_for(T.nf, nthreads, [&](int64_t a) {
      for (int k = 0; k < dim; ++k) {
        const size_t i = static_cast<size_t>(a * dim + k);
        T.r[i] = (1.0 - w) * r0[i] + w * T.r[i];
        T.v[i] = (1.0 - w) * v0[i] + w * T.v[i];
      }
      T.rho[a] = (1.0 - w) * rho0[a] + w * T.rho[a];
    });
  }

  double step() {
    switch (P.integrator) {
      case TG_SSPRK2:
      case TG_SSPRK3: {
        // SSPRKIntegrator::step (time_integrator.hpp:161-185).
        std::vector<double> r0(T.r, T.r + T.n * dim);
        std::vector<double> v0(T.v, T.v + T.n * dim);
        std::vector<double> rho0(T.rho, T.rho + T.n);
        const double dt = substep(0.0, false);
        if (P.integrator == TG_SSPRK2) {
          substep(dt, true);
          lincomb(r0, v0, rho0, 1.0 / 2.0);
        } else {
          substep(dt, true);
          lincomb(r0, v0, rho0, 1.0 / 4.0);
          substep(dt, true);
          lincomb(r0, v0, rho0, 2.0 / 3.0);
        }
        post_integrate();
        return dt;
      }
      case TG_EULER: {
        // SymplecticEulerIntegrator::step (time_integrator.hpp:50-69).
        prepare();
        const double dt = compute_time_step();
        compute_continuity();
        parallel_for(T.nf, nthreads,
                     [&](int64_t a) { T.rho[a] += dt * T.drho[a]; });
        compute_momentum();
        parallel_for(T.nf, nthreads, [&](int64_t a) {
          for (int k = 0; k < dim; ++k) {
            T.v[a * dim + k] += dt * T.dv[a * dim + k];
            T.r[a * dim + k] += dt * T.v[a * dim + k];
          }
        });
        post_integrate();
        return dt;
      }
      case TG_VERLET: {
        // VelocityVerletIntegrator::step (time_integrator.hpp:99-123).
        prepare();
        const double dt = compute_time_step();
        const double dt_2 = dt / 2.0;
        compute_momentum();
        parallel_for(T.nf, nthreads, [&](int64_t a) {
          for (int k = 0; k < dim; ++k) {
            T.v[a * dim + k] += dt_2 * T.dv[a * dim + k];
            T.r[a * dim + k] += dt * T.v[a * dim + k];
          }
        });
        prepare();
        compute_continuity();
        parallel_for(T.nf, nthreads,
                     [&](int64_t a) { T.rho[a] += dt * T.drho[a]; });
        compute_momentum();
        parallel_for(T.nf, nthreads, [&](int64_t a) {
          for (int k = 0; k < dim; ++k) {
            T.v[a * dim + k] += dt_2 * T.dv[a * dim + k];
          }
        });
        post_integrate();
        return dt;
      }
      default: return 0.0;
    }
  }
};

bool valid_params(const tg_params* P) {
  if (P == nullptr) return false;
  if (P->dim != 2 && P->dim != 3) return false;
  if (P->kernel < 0 || P->kernel > 5) return false;
  if (P->integrator < 0 || P->integrator > 3) return false;
  if (P->eos != TG_EOS_TAIT && P->eos != TG_EOS_LINEAR_TAIT) return false;
  return true;
}

}  // namespace

extern "C" {

void or_kernel_info(int32_t kernel, int32_t dim, double* unit_radius,
                    double* weight) {
  if (unit_radius) *unit_radius = kernel_table[kernel].unit_radius;
  if (weight) *weight = kernel_weight(kernel, dim);
}

double or_kernel_value(int32_t kernel, int32_t dim, const double* x,
                       double h) {
  return Kern<double>(kernel, dim, h).value(x);
}

void or_kernel_grad(int32_t kernel, int32_t dim, const double* x, double h,
                    double* out) {
  Kern<double>(kernel, dim, h).grad(x, out);
}

double or_kernel_unit_value(int32_t kernel, double q) {
  return unit_value<double>(kernel, q);
}

double or_kernel_unit_deriv(int32_t kernel, double q) {
  return unit_deriv<double>(kernel, q);
}

void or_eos(int32_t eos, double rho, double rho0, double cs0, double xi,
            double* p, double* cs, double* potential, double* rho_back) {
  const Tait E{rho0, cs0, xi, eos == TG_EOS_LINEAR_TAIT};
  const double H = E.potential(rho);
  if (p) *p = E.pressure(rho);
  if (cs) *cs = E.sound_speed(rho);
  if (potential) *potential = H;
  if (rho_back) *rho_back = E.density_from_potential(H);
}

void or_tait(double rho, double rho0, double cs0, double xi, double* p,
             double* cs, double* potential) {
  const Tait eos{rho0, cs0, xi};
  if (p) *p = eos.pressure(rho);
  if (cs) *cs = eos.sound_speed(rho);
  if (potential) *potential = eos.potential(rho);
}

double or_tait_density_from_potential(double H, double rho0, double cs0,
                                      double xi) {
  return Tait{rho0, cs0, xi}.density_from_potential(H);
}

uint64_t or_splitmix64(uint64_t x) { return splitmix64(x); }

int64_t or_grid_search(int32_t dim, int64_t n, const double* r, double radius,
                       double size_hint, int64_t* offsets, int32_t* indices,
                       int64_t capacity, int32_t nthreads) {
  Adjacency adj;
  build_adjacency<double>(dim, n, r, radius, size_hint, nthreads, adj);
  return export_csr(adj, n, offsets, indices, capacity);
}

int64_t or_grid_search_f32(int32_t dim, int64_t n, const float* r,
                           float radius, float size_hint, int64_t* offsets,
                           int32_t* indices, int64_t capacity,
                           int32_t nthreads) {
  Adjacency adj;
  build_adjacency<float>(dim, n, r, radius, size_hint, nthreads, adj);
  return export_csr(adj, n, offsets, indices, capacity);
}

int64_t or_naive_search(int32_t dim, int64_t n, const double* r,
                        double radius, int32_t inclusive, int64_t* offsets,
                        int32_t* indices, int64_t capacity) {
  // search.test.cpp:40-55, rows then sorted ascending.
  const double r2 = pow2(radius);
  std::vector<std::vector<int32_t>> rows(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) {
    rows[i].push_back(static_cast<int32_t>(i));
    for (int64_t j = 0; j < i; ++j) {
      double d[3];
      for (int k = 0; k < dim; ++k) d[k] = r[i * dim + k] - r[j * dim + k];
      const double s = norm2(d, dim);
      if (inclusive ? s <= r2 : s < r2) {
        rows[i].push_back(static_cast<int32_t>(j));
        rows[j].push_back(static_cast<int32_t>(i));
      }
    }
  }
  Adjacency adj;
  adj.off.assign(static_cast<size_t>(n + 1), 0);
  for (int64_t i = 0; i < n; ++i) {
    std::sort(rows[i].begin(), rows[i].end());
    adj.off[i + 1] = adj.off[i] + static_cast<int64_t>(rows[i].size());
  }
  for (auto& row : rows) adj.idx.insert(adj.idx.end(), row.begin(), row.end());
  return export_csr(adj, n, offsets, indices, capacity);
}

void or_mt19937_uniform_points(uint32_t seed, int64_t count, double* out) {
  std::mt19937 engine{seed};
  std::uniform_real_distribution<double> dist{0.0, 1.0};
  for (int64_t i = 0; i < count; ++i) out[i] = dist(engine);
}

int32_t or_summation_density(int32_t dim, int32_t kernel,
                             int32_t pos_precision, int64_t n,
                             const double* r, double h, double m,
                             double* rho, int32_t* counts, uint64_t* hashes,
                             int32_t nthreads) {
  if ((dim != 2 && dim != 3) || kernel < 0 || kernel > 5 || n < 0) {
    return TG_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return TG_OK;
  auto run = [&]<class Num>(const Num* pts) {
    const Kern<Num> K(kernel, dim, static_cast<Num>(h));
    const GridIndex<Num> grid(dim, n, pts, K.h);
    const Num mm = static_cast<Num>(m);
    parallel_for(n, nthreads, [&](int64_t a) {
      std::vector<int32_t> row;
      grid.search(pts + a * dim, K.radius, row);
      std::sort(row.begin(), row.end());
      Num acc{0};
      uint64_t hs = 0;
      for (const int32_t b : row) {
        Num d[3];
        for (int k = 0; k < dim; ++k) d[k] = pts[a * dim + k] - pts[b * dim + k];
        acc += mm * K.value(d);
        hs += splitmix64(static_cast<uint64_t>(b) + 1u);
      }
      if (rho) rho[a] = static_cast<double>(acc);
      if (counts) counts[a] = static_cast<int32_t>(row.size());
      if (hashes) hashes[a] = hs;
    });
  };
  if (pos_precision == TG_POS_FP32) {
    std::vector<float> pf(static_cast<size_t>(n * dim));
    for (size_t i = 0; i < pf.size(); ++i) pf[i] = static_cast<float>(r[i]);
    run(pf.data());
  } else {
    run(r);
  }
  return TG_OK;
}

int32_t or_wcsph_step(const tg_params* params, int32_t n_tanks,
                      const tg_tank* tanks, double* r, double* v, double* rho,
                      double* drho_dt, double* dv_dt, int32_t n_steps,
                      double* dt_out, double* time_io, int32_t nthreads) {
  return or_wcsph_step_faces(params, n_tanks, tanks, r, v, rho, drho_dt, dv_dt,
                             n_steps, dt_out, time_io, nthreads, nullptr);
}

int32_t or_wcsph_step_faces(const tg_params* params, int32_t n_tanks,
                            const tg_tank* tanks, double* r, double* v,
                            double* rho, double* drho_dt, double* dv_dt,
                            int32_t n_steps, double* dt_out, double* time_io,
                            int32_t nthreads, const or_tank_faces* faces) {
  if (!valid_params(params) || n_tanks < 0 || n_steps < 0) {
    return TG_ERR_INVALID_ARGUMENT;
  }
  if (faces != nullptr) {
    for (int32_t t = 0; t < n_tanks; ++t) {
      const or_tank_faces& F = faces[t];
      if (F.n_faces == 0) continue;
      const int32_t min_poly = params->dim == 2 ? 3 : 4;
      if (F.n_faces < 0 || F.face_verts == nullptr || F.n_poly < min_poly ||
          F.poly == nullptr) {
        return TG_ERR_INVALID_ARGUMENT;
      }
      for (int32_t i = 0; i < params->dim * F.n_faces; ++i) {
        if (F.face_verts[i] < 0 || F.face_verts[i] >= tanks[t].n_wall) {
          return TG_ERR_INVALID_ARGUMENT;
        }
      }
    }
  }
  const int dim = params->dim;
  int64_t base = 0;
  for (int32_t t = 0; t < n_tanks; ++t) {
    TankView T;
    T.nf = tanks[t].n_fluid;
    T.nw = tanks[t].n_wall;
    T.n = T.nf + T.nw;
    T.h = tanks[t].h;
    T.m = tanks[t].m;
    T.eos = Tait{tanks[t].rho0, tanks[t].cs0, params->xi, params->eos == TG_EOS_LINEAR_TAIT};
    T.r = r + base * dim;
    T.v = v + base * dim;
    T.rho = rho + base;
    T.drho = drho_dt + base;
    T.dv = dv_dt + base * dim;
    if (faces != nullptr) {
      T.n_faces = faces[t].n_faces;
      T.face_verts = faces[t].face_verts;
      T.n_poly = faces[t].n_poly;
      T.poly = faces[t].poly;
    }
    Solver S(*params, T, nthreads);
    double dt = 0.0;
    for (int32_t s = 0; s < n_steps; ++s) {
      dt = S.step();
      if (time_io) time_io[t] += dt;
    }
    if (dt_out) dt_out[t] = dt;
    base += T.n;
  }
  return TG_OK;
}

void or_kernel_flux2(int32_t kernel, const double* a, const double* b,
                     const double* x, double h, double* out) {
  face_flux(kernel, a, b, x, h, out);
}

double or_kernel_antigrad_flux2(int32_t kernel, const double* a,
                                const double* b, const double* x, double h) {
  return face_antigrad_flux(kernel, a, b, x, h);
}

double or_winding_number2(int32_t n_poly, const double* poly, const double* x) {
  return winding_number(n_poly, poly, x);
}

void or_kernel_flux3(int32_t kernel, const double* a, const double* b,
                     const double* c, const double* x, double h, double* out) {
  tri_flux(kernel, a, b, c, x, h, out);
}

double or_kernel_antigrad_flux3(int32_t kernel, const double* a,
                                const double* b, const double* c,
                                const double* x, double h) {
  return tri_antigrad_flux(kernel, a, b, c, x, h);
}

double or_winding_number3(int32_t n_tris, const double* tris, const double* x) {
  return winding_number3(n_tris, tris, x);
}

int32_t or_triangle_in_sphere(const double* a, const double* b, const double* c,
                              const double* x, double radius) {
  return tri_in_sphere(a, b, c, x, radius) ? 1 : 0;
}

void or_triangle_clamp(const double* a, const double* b, const double* c,
                       const double* x, double* out) {
  tri_clamp(a, b, c, x, out);
}

void or_triangle_project(const double* a, const double* b, const double* c,
                         const double* origin, double* out) {
  const TriFrame F = tri_frame(a, b, c, origin, 1.0);
  for (int i = 0; i < 6; ++i) out[i] = F.p[i];
}

int32_t or_tank_neighbour_counts(const tg_params* params, int32_t n_tanks,
                                 const tg_tank* tanks, const double* r,
                                 int32_t* counts, uint64_t* hashes,
                                 int32_t nthreads) {
  if (!valid_params(params)) return TG_ERR_INVALID_ARGUMENT;
  const int dim = params->dim;
  int64_t base = 0;
  for (int32_t t = 0; t < n_tanks; ++t) {
    const int64_t n = tanks[t].n_fluid + tanks[t].n_wall;
    const double radius = kernel_table[params->kernel].unit_radius * tanks[t].h;
    Adjacency adj;
    build_adjacency<double>(dim, n, r + base * dim, radius, tanks[t].h,
                            nthreads, adj);
    parallel_for(n, nthreads, [&](int64_t a) {
      uint64_t hs = 0;
      for (int64_t j = adj.off[a]; j < adj.off[a + 1]; ++j) {
        hs += splitmix64(static_cast<uint64_t>(adj.idx[j]) + 1u);
      }
      counts[base + a] = static_cast<int32_t>(adj.size(a));
      hashes[base + a] = hs;
    });
    base += n;
  }
  return TG_OK;
}

}  // extern "C"
