// common.cuh - device-side building blocks of the GB300 WCSPH path: smoothing
// kernels, Tait EOS, cell grid addressing and per-tank constants.
//
// Layout in HBM (per context, all arrays in "cell order", i.e. particles
// sorted by global cell key, ties kept in the order of the previous sort):
//   state X      positions (FP64, SoA per axis), velocity, density
//                (FP64, or FP32 deviation rho - rho0 in the compensated
//                form), dv/dt, drho/dt, id (upload index, bit 31 = wall),
//                cell key, and in the compensated form the FP32 offset of
//                the position from its cell corner
//   state Y      positions and ids gathered into the new cell order of a
//                stage (all fields when a prepare pass commits them back)
//   pos records  neighbour positions packed per particle (FP64 absolute, or
//                the FP32 cell offsets)
//   data records v, rho, P = p / rho^2, cs, 1 / rho packed per particle
//   step start   positions, velocity, density at the step start (two
//                buffers, permuted along with every re-sort)
//   cell table   first sorted index of every cell of every tank (+1 end)
// The tank of a particle is implied by its cell key (tanks own disjoint,
// consecutive key ranges).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/titgpu.h"

namespace tg {

constexpr uint32_t kWallBit = 0x80000000u;
constexpr uint32_t kIdMask = 0x7fffffffu;

// ---------------------------------------------------------------------------
// Per-tank constants (read-only in kernels; one entry per tank).
struct TankDev {
  double lo[3];        // grid origin
  double cs;           // cell size
  double inv_cs;       // 1 / cell size
  int32_t nc[3];       // cells per axis (nc[2] = 1 in 2D)
  uint32_t cell_off;   // first global cell of the tank
  double h, hinv;      // kernel width
  double radius2;      // (unit_radius * h)^2 in FP64
  float radius2_f;     // the same rounded from FP32 operands
  float cs_f;          // cell size in FP32
  float inv_cs_f;      // 1 / cell size in FP32 (row clipping)
  double w;            // kernel weight * h^-d
  double wg;           // w * h^-1 (gradient prefactor)
  double m;            // particle mass
  double rho0, cs0;    // Tait reference values
  double B;            // rho0 cs0^2 / xi
  double diff_k;       // 2 delta h cs0 (delta-SPH)
  double visc_eps2;    // 0.01 h^2 (Monaghan)
  uint32_t n_fluid;    // for bookkeeping
  uint32_t pad;
  // FP32 copies for the compensated form (no FP64 conversions in kernels).
  float h_f, hinv_f, w_f, wg_f, m_f, rho0_f, cs0_f, B_f, diff_k_f;
  float visc_eps2_f, c02_f;
  float cull_r2_f;  // (R (1 + 2^-12))^2: cell clipping radius, squared
  // (R (1 + 2^-12) + 2^-19 extent)^2: the wall pass's fluid-box test radius
  // in tank-local FP32 coordinates (extent = the grid's largest side).
  float wall_skip_r2_f;
  // The compensated form's neighbour band: an FP32 squared distance below
  // band_lo_f is a neighbour and one above band_hi_f is not (R^2 (1 -+ 2^-14),
  // far outside the FP32 error of the cell-relative offsets); between them
  // the pair is decided by the FP64 predicate on the FP64 positions.
  float band_lo_f, band_hi_f;
};

struct PhysDev {
  double xi;
  double g;
  double mu;
  double alpha;
  double cfl, c_force, c_visc;
  int32_t xi_is_7;
  int32_t eos;  // TG_EOS_*
  int32_t viscosity;
  int32_t diffusion;
  int32_t kernel;
  float xi_f, g_f, mu_f, alpha_f, cfl_f, c_force_f, c_visc_f, pad_f;
};

// ---------------------------------------------------------------------------
// Smoothing kernels (source/tit/sph/kernel.gen.cpp:520-553): unit value f(q)
// and g(q) = f'(q) / q for the Wendland kernels (a polynomial, so the
// gradient needs no 1/r), or f'(q) for the B-splines.
template<int K>
struct KernelPoly;

template<>
struct KernelPoly<TG_KERNEL_WENDLAND_C2> {
  static constexpr bool deriv_over_q = true;
  static constexpr double unit_radius = 2.0;
  template<class T>
  __device__ __forceinline__ static T value(T q) {
    const T t = T(1) - T(0.5) * q;
    const T t2 = t * t;
    return q < T(2) ? (T(1) + T(2) * q) * (t2 * t2) : T(0);
  }
  template<class T>
  __device__ __forceinline__ static T dq(T q) {  // f'(q) / q
    const T t = T(1) - T(0.5) * q;
    return q < T(2) ? T(-5) * (t * t * t) : T(0);
  }
};

template<>
struct KernelPoly<TG_KERNEL_WENDLAND_C4> {
  static constexpr bool deriv_over_q = true;
  static constexpr double unit_radius = 2.0;
  template<class T>
  __device__ __forceinline__ static T value(T q) {
    const T t = T(1) - T(0.5) * q;
    const T t2 = t * t;
    return q < T(2) ? (T(1) + T(3) * q + T(35.0 / 12.0) * q * q) *
                          (t2 * t2 * t2)
                    : T(0);
  }
  template<class T>
  __device__ __forceinline__ static T dq(T q) {
    const T t = T(1) - T(0.5) * q;
    const T t2 = t * t;
    return q < T(2) ? T(-14.0 / 3.0) * (T(1) + T(2.5) * q) * (t2 * t2 * t)
                    : T(0);
  }
};

template<>
struct KernelPoly<TG_KERNEL_WENDLAND_C6> {
  static constexpr bool deriv_over_q = true;
  static constexpr double unit_radius = 2.0;
  template<class T>
  __device__ __forceinline__ static T value(T q) {
    const T t = T(1) - T(0.5) * q;
    const T t2 = t * t;
    const T t4 = t2 * t2;
    return q < T(2) ? (T(1) + T(4) * q + T(6.25) * q * q + T(4) * q * q * q) *
                          (t4 * t4)
                    : T(0);
  }
  template<class T>
  __device__ __forceinline__ static T dq(T q) {
    const T t = T(1) - T(0.5) * q;
    const T t2 = t * t;
    const T t4 = t2 * t2;
    return q < T(2) ? T(-2.75) * (T(2) + T(7) * q + T(8) * q * q) *
                          (t4 * t2 * t)
                    : T(0);
  }
};

template<>
struct KernelPoly<TG_KERNEL_CUBIC_SPLINE> {
  static constexpr bool deriv_over_q = false;
  static constexpr double unit_radius = 2.0;
  template<class T>
  __device__ __forceinline__ static T value(T q) {
    const T a = T(2) - q, b = T(1) - q;
    return (q < T(2) ? T(0.25) * a * a * a : T(0)) +
           (q < T(1) ? -(b * b * b) : T(0));
  }
  template<class T>
  __device__ __forceinline__ static T deriv(T q) {
    const T a = T(2) - q, b = T(1) - q;
    return (q < T(2) ? T(-0.75) * a * a : T(0)) +
           (q < T(1) ? T(3) * b * b : T(0));
  }
};

template<>
struct KernelPoly<TG_KERNEL_QUARTIC_SPLINE> {
  static constexpr bool deriv_over_q = false;
  static constexpr double unit_radius = 2.5;
  template<class T>
  __device__ __forceinline__ static T value(T q) {
    const T a = T(2.5) - q, b = T(1.5) - q, c = T(0.5) - q;
    const T a2 = a * a, b2 = b * b, c2 = c * c;
    return (q < T(2.5) ? a2 * a2 : T(0)) +
           (q < T(1.5) ? T(-5) * (b2 * b2) : T(0)) +
           (q < T(0.5) ? T(10) * (c2 * c2) : T(0));
  }
  template<class T>
  __device__ __forceinline__ static T deriv(T q) {
    const T a = T(2.5) - q, b = T(1.5) - q, c = T(0.5) - q;
    return (q < T(2.5) ? T(-4) * a * a * a : T(0)) +
           (q < T(1.5) ? T(20) * b * b * b : T(0)) +
           (q < T(0.5) ? T(-40) * c * c * c : T(0));
  }
};

template<>
struct KernelPoly<TG_KERNEL_QUINTIC_SPLINE> {
  static constexpr bool deriv_over_q = false;
  static constexpr double unit_radius = 3.0;
  template<class T>
  __device__ __forceinline__ static T value(T q) {
    const T a = T(3) - q, b = T(2) - q, c = T(1) - q;
    const T a2 = a * a, b2 = b * b, c2 = c * c;
    return (q < T(3) ? a2 * a2 * a : T(0)) +
           (q < T(2) ? T(-6) * (b2 * b2 * b) : T(0)) +
           (q < T(1) ? T(15) * (c2 * c2 * c) : T(0));
  }
  template<class T>
  __device__ __forceinline__ static T deriv(T q) {
    const T a = T(3) - q, b = T(2) - q, c = T(1) - q;
    const T a2 = a * a, b2 = b * b, c2 = c * c;
    return (q < T(3) ? T(-5) * (a2 * a2) : T(0)) +
           (q < T(2) ? T(30) * (b2 * b2) : T(0)) +
           (q < T(1) ? T(-75) * (c2 * c2) : T(0));
  }
};

// Gradient factor F with grad W_ab = F * (r_a - r_b):
//   F = w h^-1 f'(q) / r.  For the Wendland kernels f'(q)/r = h^-1 f'(q)/q.
template<int K, class T>
__device__ __forceinline__ T grad_factor(T q, T rinv, T wg, T hinv) {
  if constexpr (KernelPoly<K>::deriv_over_q) {
    return wg * hinv * KernelPoly<K>::dq(q);
  } else {
    return wg * KernelPoly<K>::deriv(q) * rinv;
  }
}

// Host-side kernel normalisation tables (zero moments of the unit kernels,
// kernel.hpp:126-131; exact rationals of the kernel.gen.cpp polynomials).
inline double kernel_unit_radius(int k) {
  switch (k) {
    case TG_KERNEL_QUARTIC_SPLINE: return 2.5;
    case TG_KERNEL_QUINTIC_SPLINE: return 3.0;
    default: return 2.0;
  }
}
inline double kernel_zero_moment(int k, int dim) {
  static const double m[6][3] = {
      {3.0 / 4.0, 7.0 / 20.0, 1.0 / 4.0},
      {12.0, 1199.0 / 192.0, 5.0},
      {60.0, 239.0 / 7.0, 30.0},
      {2.0 / 3.0, 2.0 / 7.0, 4.0 / 21.0},
      {16.0 / 27.0, 2.0 / 9.0, 64.0 / 495.0},
      {8.0 / 15.0, 7.0 / 39.0, 128.0 / 1365.0},
  };
  return m[k][dim - 1];
}

// ---------------------------------------------------------------------------
// Cell addressing.  All cell coordinates are computed in FP64 from FP64 (or
// FP32-widened) positions, clamped to the tank grid.  Clamping is a per-axis
// 1-Lipschitz projection, so two points within the support radius still land
// at most cells_per_radius cells apart.
template<int D>
__device__ __forceinline__ void cell_of(const TankDev& T, const double* x,
                                        int* c, bool& outside) {
#pragma unroll
  for (int i = 0; i < D; ++i) {
    const double f = (x[i] - T.lo[i]) * T.inv_cs;
    int ci;
    if (!(f >= 0.0)) {  // also catches NaN
      ci = 0;
      outside = true;
    } else if (f >= static_cast<double>(T.nc[i])) {
      ci = T.nc[i] - 1;
      outside = true;
    } else {
      ci = static_cast<int>(f);
    }
    c[i] = ci;
  }
}

// Keys: every cell owns two consecutive keys, 2 * cell for its fluid
// particles and 2 * cell + 1 for its wall particles, so in key order a
// cell's fluid particles precede its walls and a row of cells is still one
// contiguous key range.
__device__ __forceinline__ uint32_t key_of(uint32_t cell, bool wall) {
  return (cell << 1) | (wall ? 1u : 0u);
}

// Tank of a global key: the last tank whose first key is <= key (off holds
// each tank's first key, 2 * cell_off).
__device__ __forceinline__ uint32_t tank_of_key(uint32_t key,
                                                const uint32_t* __restrict__ off,
                                                int ntanks) {
  int lo = 0, hi = ntanks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(off + mid) <= key) {
      lo = mid;
    } else {
      hi = mid - 1;
    }
  }
  return static_cast<uint32_t>(lo);
}

// Cell coordinates of a key of tank T (inverse of key_of(flat_cell)).
template<int D>
__device__ __forceinline__ void cell_from_key(const TankDev& T, uint32_t key,
                                              int* c) {
  const uint32_t f = (key >> 1) - T.cell_off;
  const uint32_t nx = static_cast<uint32_t>(T.nc[0]);
  c[0] = static_cast<int>(f % nx);
  const uint32_t rest = f / nx;
  if constexpr (D == 2) {
    c[1] = static_cast<int>(rest);
    c[2] = 0;
  } else {
    const uint32_t ny = static_cast<uint32_t>(T.nc[1]);
    c[1] = static_cast<int>(rest % ny);
    c[2] = static_cast<int>(rest / ny);
  }
}

template<int D>
__device__ __forceinline__ uint32_t flat_cell(const TankDev& T, const int* c) {
  uint32_t f = static_cast<uint32_t>(c[0]);
  if constexpr (D >= 2) f += static_cast<uint32_t>(c[1]) * T.nc[0];
  if constexpr (D == 3) {
    f += static_cast<uint32_t>(c[2]) * static_cast<uint32_t>(T.nc[0]) *
         static_cast<uint32_t>(T.nc[1]);
  }
  return T.cell_off + f;
}

// ---------------------------------------------------------------------------
// Tait EOS (source/tit/sph/equation_of_state.hpp:37-64).
//   p = B ((rho/rho0)^xi - 1), cs = cs0 (rho/rho0)^((xi-1)/2),
//   H = cs0^2 ((rho/rho0)^(xi-1) - 1) / (xi - 1).
// FP64 form works on rho; the compensated form works on the deviation
// d = (rho - rho0) / rho0 and expands (1+d)^n - 1 = d * sum C(n,k) d^(k-1)
// for xi = 7 (log1p/expm1 otherwise), so no cancellation occurs.
struct EosOut {
  double p, c;
};

__device__ __forceinline__ void tait_f64(const PhysDev& P, const TankDev& T,
                                         double rho, double& p, double& c) {
  if (P.eos == TG_EOS_LINEAR_TAIT) {
    // LinearTaitEquationOfState (equation_of_state.hpp:91-105).
    p = T.cs0 * T.cs0 * (rho - T.rho0);
    c = T.cs0;
    return;
  }
  const double x = rho / T.rho0;
  if (P.xi_is_7) {
    const double x2 = x * x;
    const double x3 = x2 * x;
    p = T.B * (x3 * x3 * x - 1.0);
    c = T.cs0 * x3;
  } else {
    p = T.B * (pow(x, P.xi) - 1.0);
    c = T.cs0 * pow(x, 0.5 * (P.xi - 1.0));
  }
}

__device__ __forceinline__ double potential_f64(const PhysDev& P,
                                                const TankDev& T, double rho) {
  if (P.eos == TG_EOS_LINEAR_TAIT) return T.cs0 * T.cs0 * log(rho / T.rho0);
  const double x = rho / T.rho0;
  if (P.xi_is_7) {
    const double x2 = x * x;
    const double x6 = x2 * x2 * x2;
    return T.cs0 * T.cs0 * (x6 - 1.0) / 6.0;
  }
  return T.cs0 * T.cs0 * (pow(x, P.xi - 1.0) - 1.0) / (P.xi - 1.0);
}

__device__ __forceinline__ double density_from_potential_f64(
    const PhysDev& P, const TankDev& T, double H) {
  if (P.eos == TG_EOS_LINEAR_TAIT) return T.rho0 * exp(H / (T.cs0 * T.cs0));
  const double xi_1 = P.xi - 1.0;
  return T.rho0 * pow(1.0 + xi_1 * H / (T.cs0 * T.cs0), 1.0 / xi_1);
}

// Compensated form: d = drho / rho0 in FP32.
__device__ __forceinline__ void tait_f32(const PhysDev& P, const TankDev& T,
                                         float drho, float& p, float& c) {
  if (P.eos == TG_EOS_LINEAR_TAIT) {
    p = T.c02_f * drho;
    c = T.cs0_f;
    return;
  }
  const float d = __fdividef(drho, T.rho0_f);
  const float B = T.B_f;
  const float c0 = T.cs0_f;
  if (P.xi_is_7) {
    const float poly =
        7.f + d * (21.f + d * (35.f + d * (35.f + d * (21.f + d * (7.f + d)))));
    p = B * d * poly;
    const float x = 1.f + d;
    c = c0 * (x * x * x);
  } else {
    const float l = log1pf(d);
    p = B * expm1f(P.xi_f * l);
    c = c0 * expf(0.5f * (P.xi_f - 1.f) * l);
  }
}

__device__ __forceinline__ float potential_f32(const PhysDev& P,
                                               const TankDev& T, float drho) {
  const float d = __fdividef(drho, T.rho0_f);
  const float c02 = T.c02_f;
  if (P.eos == TG_EOS_LINEAR_TAIT) return c02 * log1pf(d);
  if (P.xi_is_7) {
    const float poly =
        6.f + d * (15.f + d * (20.f + d * (15.f + d * (6.f + d))));
    return c02 * d * poly * (1.f / 6.f);
  }
  const float xi_1 = P.xi_f - 1.f;
  return c02 * expm1f(xi_1 * log1pf(d)) / xi_1;
}

// Returns the density deviation rho - rho0.
__device__ __forceinline__ float deviation_from_potential_f32(
    const PhysDev& P, const TankDev& T, float H) {
  if (P.eos == TG_EOS_LINEAR_TAIT) return T.rho0_f * expm1f(H / T.c02_f);
  const float xi_1 = P.xi_f - 1.f;
  const float u = xi_1 * H / T.c02_f;
  return T.rho0_f * expm1f(log1pf(u) / xi_1);
}

// ---------------------------------------------------------------------------
// Misc helpers.
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Positive doubles order like their bit patterns.
__device__ __forceinline__ void atomic_min_pos(double* addr, double v) {
  atomicMin(reinterpret_cast<unsigned long long*>(addr),
            static_cast<unsigned long long>(__double_as_longlong(v)));
}

// Kahan-Babuska compensated accumulation in FP32 with explicit round-to-
// nearest operations so nothing is contracted or reassociated.
struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ float value() const { return s; }
  // Fold in another accumulator's sum s2 - c2 (two compensated adds).
  __device__ __forceinline__ void merge(float s2, float c2) {
    add(s2);
    add(-c2);
  }
};

}  // namespace tg
