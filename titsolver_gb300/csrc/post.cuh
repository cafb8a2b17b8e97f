// post.cuh - the post-integration stage with particle shifting and the
// free-surface density correction (FluidEquations::post_integrate,
// apply_shifts and apply_free_surface_correction,
// source/tit/sph/fluid_equations.hpp:315-512), in gather form on the cell
// order of a fresh prepare (sort + reorder + wall extrapolation).
//
// Arithmetic is FP64 in both forms (the compensated form converts its FP32
// fields on load and rounds the results back); the decisions the reference
// takes by exact comparison (the 45-degree visibility cone, the splash
// neighbour count, phi == phi_max / phi_min bit tests, the nearest
// free-surface neighbour with the lowest index on ties) use the same
// uncontracted operation order as the oracle's restatement.
//
//   k_post_sums   N, L, grad v, grad rho (pair sums over the prepare's
//                 neighbours), L^T inverse by unpivoted LU, neighbour count
//   k_post_phi    free-surface flag: visibility cone, then splashes
//   k_post_near   near-surface scaling of phi by the closest surface
//                 neighbour's normal
//   k_post_shift  r += dr, v += grad v dr, rho += grad rho . dr for the far
//                 particles; new home keys
//   k_post_fs     Shepard-corrected summation density for the others, on
//                 the prepare's neighbours at the shifted positions
#pragma once

#include "faces.cuh"
#include "fluid.cuh"

namespace tg {

constexpr double kPhiMax = 1.0;
constexpr double kPhiMin = 2.2250738585072014e-308;  // smallest normal double

template<int D, int F>
struct PostArgs {
  StageArgs<D, F> S;  // Y: the state in cell order; X: the home output
  double* N;          // D per particle: renormalised unit normal
  double* dr;         // D: raw N (the shift direction)
  double* gv;         // D x D: renormalised velocity gradient
  double* grho;       // D: renormalised density gradient
  int32_t* count;     // neighbours including self
  double* phi;        // free-surface flag after the cone and splash tests
  double* phi2;       // after the near-surface scaling
  double* rho_raw;    // densities after shifting (walls: extrapolated)
  double cos2_fov;    // cos(pi/4)^2
  double k_fs;        // -log(0.05) / 0.01^2
  double shift;       // -CFL * 0.2
};

// f'(q) of the unit kernel.
template<int K>
__device__ __forceinline__ double kernel_deriv(double q) {
  if constexpr (KernelPoly<K>::deriv_over_q) {
    return KernelPoly<K>::dq(q) * q;
  } else {
    return KernelPoly<K>::deriv(q);
  }
}

__device__ __forceinline__ double dot_rn(const double* a, const double* b,
                                         int d) {
  double r = __dmul_rn(a[0], b[0]);
  for (int i = 1; i < d; ++i) r = __dadd_rn(r, __dmul_rn(a[i], b[i]));
  return r;
}

// Density, velocity and volume of neighbour j from the prepare's records
// (walls: extrapolated density, zero velocity).
template<int D>
__device__ __forceinline__ void post_neighbour(const Dat64* dat, uint32_t j,
                                               const TankDev&, double& rho,
                                               double* v) {
  const Dat64 b = load_dat(dat, j);
  rho = b.rho;
  v[0] = b.vx;
  v[1] = b.vy;
  v[2] = b.vz;
}
template<int D>
__device__ __forceinline__ void post_neighbour(const Dat32* dat, uint32_t j,
                                               const TankDev& T, double& rho,
                                               double* v) {
  const Dat32 b = load_dat(dat, j);
  rho = T.rho0 + static_cast<double>(b.drho);
  v[0] = b.vx;
  v[1] = b.vy;
  v[2] = b.vz;
}

// Unpivoted LU inverse with the |pivot| <= tiny test (core/_mat/fact.hpp);
// false when a pivot is tiny.
template<int D>
__device__ __forceinline__ bool lu_inverse(const double* A, double* inv) {
  constexpr double tiny = 6.0554544523933395e-06;
  double LU[D * D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
#pragma unroll
    for (int j = 0; j < i; ++j) {
      double s = A[i * D + j];
#pragma unroll
      for (int k = 0; k < j; ++k) s = __dsub_rn(s, __dmul_rn(LU[i * D + k], LU[k * D + j]));
      LU[i * D + j] = __ddiv_rn(s, LU[j * D + j]);
    }
#pragma unroll
    for (int j = i; j < D; ++j) {
      double s = A[i * D + j];
#pragma unroll
      for (int k = 0; k < i; ++k) s = __dsub_rn(s, __dmul_rn(LU[i * D + k], LU[k * D + j]));
      LU[i * D + j] = s;
    }
    if (fabs(LU[i * D + i]) <= tiny) return false;
  }
#pragma unroll
  for (int c = 0; c < D; ++c) {
    double x[D];
#pragma unroll
    for (int i = 0; i < D; ++i) x[i] = i == c ? 1.0 : 0.0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
#pragma unroll
      for (int k = 0; k < i; ++k) x[i] = __dsub_rn(x[i], __dmul_rn(LU[i * D + k], x[k]));
    }
#pragma unroll
    for (int i = D - 1; i >= 0; --i) {
#pragma unroll
      for (int k = i + 1; k < D; ++k) x[i] = __dsub_rn(x[i], __dmul_rn(LU[i * D + k], x[k]));
      x[i] = __ddiv_rn(x[i], LU[i * D + i]);
    }
#pragma unroll
    for (int i = 0; i < D; ++i) inv[i * D + c] = x[i];
  }
  return true;
}

template<int D, int F>
__device__ __forceinline__ bool post_target(const PostArgs<D, F>& A, int64_t& i,
                                            uint32_t& id, const TankDev*& T,
                                            int* c) {
  i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.S.n) return false;
  id = A.S.Y.id[i];
  const uint32_t key = A.S.skey[i];
  T = &A.S.tanks[tank_of_key(key, A.S.tank_off, A.S.ntanks)];
  cell_from_key<D>(*T, key, c);
  return true;
}

// Face terms of the shifting sums of the fluid face particles (N, L,
// grad v, grad rho; fluid_equations.hpp:340-349), divided by gamma_a, one
// warp per particle with the lanes splitting its faces; k_post_sums starts
// its pair sums from them (zero for particles whose cell lists no faces).
// A pass of its own keeps the face integrals' registers out of the pair
// loop.
template<int D, int F, int K, class FT>
__global__ void __launch_bounds__(128) k_post_faces(PostArgs<D, F> A) {
  const FaceArgs& fc = A.S.fc;
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  const uint32_t count = *fc.face_count;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += nwarps) {
    const uint32_t i = fc.face_list[w];
    if (A.S.Y.id[i] & kWallBit) continue;
    const uint32_t key = A.S.skey[i];
    const TankDev& T = A.S.tanks[tank_of_key(key, A.S.tank_off, A.S.ntanks)];
    int c[3] = {0, 0, 0};
    cell_from_key<D>(T, key, c);
    double rho_a, va[3];
    post_neighbour<D>(A.S.datrec, i, T, rho_a, va);
    double pa[3];
#pragma unroll
    for (int k = 0; k < D; ++k) pa[k] = A.S.Y.pos[k][i];
    double sums[kPostFaceSums<D>] = {};
    double* N = sums;
    double* L = sums + D;
    double* gv = sums + D + D * D;
    double* gr = sums + D + 2 * D * D;
    const double gam = fc.gamma[i];
    const double radius = KernelPoly<K>::unit_radius * T.h;
    for_adjacent_faces<D>(fc, global_cell<D>(T, c), pa, radius, lane,
                          [&](bool active, uint32_t f, const double* g) {
      // Per-face weights (vertex density, face centre): no edges cancel.
      double gg[3], rv[3], r_sa[3];
      face_flux_d<K, D, FT>(active, g, face_axes<D>(fc, f), pa, T.h, fc.weight, gg);
      if (!active) return;
#pragma unroll
      for (int j = 0; j < D; ++j) rv[j] = vertex_rho(A.S.datrec, fc.slot_of[fc.vert[D * f + j]], T);
#pragma unroll
      for (int k = 0; k < D; ++k) {
        double xk[3];
#pragma unroll
        for (int j = 0; j < D; ++j) xk[j] = g[D * j + k];
        r_sa[k] = face_avg<D>(xk) - pa[k];
      }
      // The face vertices' velocities are zero: v_sa = -v_a.
      const double rho_sa = face_avg<D>(rv) - rho_a;
#pragma unroll
      for (int a2 = 0; a2 < D; ++a2) {
        N[a2] -= gg[a2] / gam;
#pragma unroll
        for (int b2 = 0; b2 < D; ++b2) {
          L[a2 * D + b2] -= r_sa[a2] * gg[b2] / gam;
          gv[a2 * D + b2] -= -va[a2] * gg[b2] / gam;
        }
        gr[a2] -= rho_sa * gg[a2] / gam;
      }
    });
    double* out = fc.post_face + kPostFaceSums<D> * static_cast<size_t>(i);
#pragma unroll
    for (int k = 0; k < kPostFaceSums<D>; ++k) {
      const double v = warp_sum(sums[k]);
      if (lane == 0) out[k] = v;
    }
  }
}

template<int D, int F, int K>
__global__ void __launch_bounds__(128) k_post_sums(PostArgs<D, F> A) {
  int64_t i;
  uint32_t id;
  const TankDev* Tp;
  int c[3] = {0, 0, 0};
  if (!post_target(A, i, id, Tp, c)) return;
  const TankDev& T = *Tp;
  double rho_a, va[3];
  post_neighbour<D>(A.S.datrec, static_cast<uint32_t>(i), T, rho_a, va);
  if (id & kWallBit) {
    A.rho_raw[i] = rho_a;
    A.phi[i] = kPhiMax;
    return;
  }
  double pa[3];
#pragma unroll
  for (int k = 0; k < D; ++k) pa[k] = A.S.Y.pos[k][i];
  double N[D] = {}, L[D * D] = {}, gv[D * D] = {}, gr[D] = {};
  int32_t count = 0;
  const double tiny2 = 6.0554544523933395e-06 * 6.0554544523933395e-06;
  // Face boundaries (fluid_equations.hpp:335-349): face terms first, and
  // every sum divided by gamma_a.
  // Face boundaries (fluid_equations.hpp:335-349): the face terms come
  // first (k_post_faces), and every sum is divided by gamma_a.
  double gam = 1.0;
  const uint32_t gcell = A.S.fc.on ? global_cell<D>(T, c) : 0u;
  if (A.S.fc.on) gam = A.S.fc.gamma[i];
  if (A.S.fc.on && A.S.fc.cell_start[gcell + 1] > A.S.fc.cell_start[gcell]) {
    const double* f0 = A.S.fc.post_face + kPostFaceSums<D> * static_cast<size_t>(i);
#pragma unroll
    for (int k = 0; k < D; ++k) {
      N[k] = f0[k];
      gr[k] = f0[D + 2 * D * D + k];
    }
#pragma unroll
    for (int k = 0; k < D * D; ++k) {
      L[k] = f0[D + k];
      gv[k] = f0[D + D * D + k];
    }
  }
  for_cells<D, false>(T, c, A.S.k, A.S.cell_start,
                      [&](uint32_t s, uint32_t en, int, int, int) {
    for (uint32_t j = s; j < en; ++j) {
      double pb[3], d[3];
#pragma unroll
      for (int k = 0; k < D; ++k) pb[k] = A.S.Y.pos[k][j];
      const double s2 = dist2_exact<D>(pa, pb, d);
      if (s2 > T.radius2) continue;
      ++count;
      if (j == static_cast<uint32_t>(i)) continue;
      // grad W(r_ab) = w f'(q) / h * normalize(r_ab) (kernel.hpp:154-163).
      const double r = sqrt(s2);
      const double sc = s2 >= tiny2 ? 1.0 / r : 0.0;
      const double q = T.hinv * r;
      const double f = T.w * kernel_deriv<K>(q);
      double gW[3];
#pragma unroll
      for (int k = 0; k < D; ++k) gW[k] = f * ((d[k] * sc) * T.hinv);
      double rho_b, vb[3];
      post_neighbour<D>(A.S.datrec, j, T, rho_b, vb);
      const double V = T.m / rho_b / gam;
      const double drb = rho_b - rho_a;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        N[a] += V * gW[a];
#pragma unroll
        for (int b = 0; b < D; ++b) {
          L[a * D + b] += V * (-d[a] * gW[b]);
          gv[a * D + b] += V * ((vb[a] - va[a]) * gW[b]);
        }
        gr[a] += V * drb * gW[a];
      }
    }
  });
  double* dr = A.dr + i * D;
#pragma unroll
  for (int a = 0; a < D; ++a) dr[a] = N[a];
  double LT[D * D], Li[D * D];
#pragma unroll
  for (int a = 0; a < D; ++a) {
#pragma unroll
    for (int b = 0; b < D; ++b) LT[a * D + b] = L[b * D + a];
  }
  if (lu_inverse<D>(LT, Li)) {
    double tN[D], tg[D], tgv[D * D];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      tN[a] = 0.0;
      tg[a] = 0.0;
#pragma unroll
      for (int b = 0; b < D; ++b) {
        tN[a] += Li[a * D + b] * N[b];
        tg[a] += Li[a * D + b] * gr[b];
      }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
#pragma unroll
      for (int b = 0; b < D; ++b) {
        double s = 0.0;
#pragma unroll
        for (int l = 0; l < D; ++l) s += gv[a * D + l] * Li[b * D + l];
        tgv[a * D + b] = s;
      }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
      N[a] = tN[a];
      gr[a] = tg[a];
    }
#pragma unroll
    for (int a = 0; a < D * D; ++a) gv[a] = tgv[a];
  }
  // normalize() with the |N|^2 >= tiny^2 guard (core/_vec/vec.hpp:663-676).
  const double n2 = dot_rn(N, N, D);
  const double sN = n2 >= tiny2 ? 1.0 / sqrt(n2) : 0.0;
#pragma unroll
  for (int a = 0; a < D; ++a) A.N[i * D + a] = N[a] * sN;
#pragma unroll
  for (int a = 0; a < D * D; ++a) A.gv[i * D * D + a] = gv[a];
#pragma unroll
  for (int a = 0; a < D; ++a) A.grho[i * D + a] = gr[a];
  A.count[i] = count;
}

template<int D, int F>
__global__ void __launch_bounds__(128) k_post_phi(PostArgs<D, F> A) {
  int64_t i;
  uint32_t id;
  const TankDev* Tp;
  int c[3] = {0, 0, 0};
  if (!post_target(A, i, id, Tp, c)) return;
  if (id & kWallBit) return;  // phi_max, set by k_post_sums
  const TankDev& T = *Tp;
  double pa[3], Na[3];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    pa[k] = A.S.Y.pos[k][i];
    Na[k] = A.N[i * D + k];
  }
  bool visible = false;
  for_cells<D, false>(T, c, A.S.k, A.S.cell_start,
                      [&](uint32_t s, uint32_t en, int, int, int) {
    for (uint32_t j = s; j < en && !visible; ++j) {
      if (j == static_cast<uint32_t>(i)) continue;
      double pb[3], d[3];
#pragma unroll
      for (int k = 0; k < D; ++k) pb[k] = A.S.Y.pos[k][j];
      const double s2 = dist2_exact<D>(pa, pb, d);
      if (s2 > T.radius2) continue;
      const double fov = __dmul_rn(A.cos2_fov, s2);
      const double na = dot_rn(Na, d, D);
      if (na > 0.0 && __dmul_rn(na, na) >= fov) visible = true;
    }
  });
  const int cutoff = D == 2 ? 8 : 26;
  double phi = visible ? kPhiMax : kPhiMin;
  if (A.count[i] <= cutoff) phi = kPhiMin;
  A.phi[i] = phi;
}

__device__ __forceinline__ bool bits_eq(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}

template<int D, int F, int K>
__global__ void __launch_bounds__(128) k_post_near(PostArgs<D, F> A) {
  int64_t i;
  uint32_t id;
  const TankDev* Tp;
  int c[3] = {0, 0, 0};
  if (!post_target(A, i, id, Tp, c)) return;
  const double phi = A.phi[i];
  if ((id & kWallBit) || !bits_eq(phi, kPhiMax)) {
    A.phi2[i] = phi;
    return;
  }
  const TankDev& T = *Tp;
  double pa[3];
#pragma unroll
  for (int k = 0; k < D; ++k) pa[k] = A.S.Y.pos[k][i];
  int64_t best = -1;
  uint32_t best_id = 0;
  double best_d2 = 0.0;
  for_cells<D, false>(T, c, A.S.k, A.S.cell_start,
                      [&](uint32_t s, uint32_t en, int, int, int) {
    for (uint32_t j = s; j < en; ++j) {
      if (!bits_eq(A.phi[j], kPhiMin)) continue;
      double pb[3], d[3];
#pragma unroll
      for (int k = 0; k < D; ++k) pb[k] = A.S.Y.pos[k][j];
      const double s2 = dist2_exact<D>(pa, pb, d);
      if (s2 > T.radius2) continue;
      // The reference takes the first minimum in index order.
      const uint32_t jid = A.S.Y.id[j] & kIdMask;
      if (best < 0 || s2 < best_d2 || (s2 == best_d2 && jid < best_id)) {
        best = j;
        best_id = jid;
        best_d2 = s2;
      }
    }
  });
  double out = phi;
  if (best >= 0) {
    double d[3], Nb[3];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      d[k] = __dsub_rn(pa[k], A.S.Y.pos[k][best]);
      Nb[k] = A.N[best * D + k];
    }
    const double R = KernelPoly<K>::unit_radius * T.h;
    out = phi * (fabs(dot_rn(Nb, d, D)) / R);
  }
  A.phi2[i] = out;
}

template<int D, int F>
__global__ void __launch_bounds__(128) k_post_shift(PostArgs<D, F> A) {
  using R = typename StageArgs<D, F>::R;
  int64_t i;
  uint32_t id;
  const TankDev* Tp;
  int c[3] = {0, 0, 0};
  if (!post_target(A, i, id, Tp, c)) return;
  if (id & kWallBit) {
    commit_wall(A.S, i, id);
    return;
  }
  const TankDev& T = *Tp;
  const StateBuf<R>& Y = A.S.Y;
  const StateBuf<R>& X = A.S.X;
  double p[3] = {0.0, 0.0, 0.0}, v[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < D; ++k) {
    p[k] = Y.pos[k][i];
    v[k] = static_cast<double>(Y.vel[k][i]);
  }
  double rho = static_cast<double>(Y.rho[i]);
  if constexpr (F == TG_FP32C) rho += T.rho0;
  if (bits_eq(A.phi2[i], kPhiMax)) {
    const double sc = A.shift * (T.h * T.h);
    double dr[D];
#pragma unroll
    for (int k = 0; k < D; ++k) dr[k] = A.dr[i * D + k] * sc;
#pragma unroll
    for (int k = 0; k < D; ++k) p[k] += dr[k];
    // The velocity correction applies where gamma ~ 1 (:465-467).
    const double gam = A.S.fc.on ? A.S.fc.gamma[i] : 1.0;
    if (fabs(gam - 1.0) <= 6.0554544523933395e-06) {
      double dv[D];
#pragma unroll
      for (int a = 0; a < D; ++a) dv[a] = dot_rn(A.gv + (i * D + a) * D, dr, D);
#pragma unroll
      for (int k = 0; k < D; ++k) v[k] += dv[k];
    }
    rho += dot_rn(A.grho + i * D, dr, D);
  }
  A.rho_raw[i] = rho;
  // Home state with the key (and FP32 offset) of the new position.
  int cn[3] = {0, 0, 0};
  bool outside = false;
  cell_of<D>(T, p, cn, outside);
  if (outside) atomicOr(A.S.err, static_cast<uint32_t>(TG_DEV_OUTSIDE_GRID));
  bool finite = true;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    X.pos[k][i] = p[k];
    if constexpr (F == TG_FP64) {
      X.vel[k][i] = v[k];
    } else {
      X.vel[k][i] = __double2float_rn(v[k]);
      X.off[k][i] = __double2float_rn(p[k] - fma(static_cast<double>(cn[k]), T.cs, T.lo[k]));
    }
    X.dv[k][i] = Y.dv[k][i];
    finite = finite && finite_bits(p[k]) && finite_bits(v[k]);
  }
  if constexpr (F == TG_FP64) {
    X.rho[i] = rho;
  } else {
    X.rho[i] = __double2float_rn(rho - T.rho0);
  }
  X.drho[i] = Y.drho[i];
  X.id[i] = id;
  X.pkey[i] = A.S.skey[i];  // read before the key write: the buffers may alias
  X.key[i] = key_of(flat_cell<D>(T, cn), false);
  if (!(finite && finite_bits(rho))) {
    atomicOr(A.S.err, static_cast<uint32_t>(TG_DEV_NONFINITE_STATE));
  }
}

template<int D, int F, int K>
__global__ void __launch_bounds__(128) k_post_fs(PostArgs<D, F> A) {
  int64_t i;
  uint32_t id;
  const TankDev* Tp;
  int c[3] = {0, 0, 0};
  if (!post_target(A, i, id, Tp, c)) return;
  if ((id & kWallBit) || bits_eq(A.phi2[i], kPhiMax)) return;
  const TankDev& T = *Tp;
  double pa[3], xa[3];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    pa[k] = A.S.Y.pos[k][i];  // prepare positions: the neighbour set
    xa[k] = A.S.X.pos[k][i];  // shifted positions: the kernel values
  }
  double alpha = 0.0, rho_t = 0.0;
  for_cells<D, false>(T, c, A.S.k, A.S.cell_start,
                      [&](uint32_t s, uint32_t en, int, int, int) {
    for (uint32_t j = s; j < en; ++j) {
      double pb[3], d[3];
#pragma unroll
      for (int k = 0; k < D; ++k) pb[k] = A.S.Y.pos[k][j];
      if (dist2_exact<D>(pa, pb, d) > T.radius2) continue;
      double x[3];
#pragma unroll
      for (int k = 0; k < D; ++k) x[k] = xa[k] - A.S.X.pos[k][j];
      const double q = T.hinv * sqrt(dot_rn(x, x, D));
      const double W = T.w * KernelPoly<K>::value(q);
      alpha += T.m / A.rho_raw[j] * W;
      rho_t += T.m * W;
    }
  });
  const double gam = A.S.fc.on ? A.S.fc.gamma[i] : 1.0;
  const double ratio = fmin(1.0, alpha / gam);
  if (ratio > 0.99) return;
  const double beta = exp(-A.k_fs * ((ratio - 1.0) * (ratio - 1.0)));
  const double corr = beta * gam + (1.0 - beta) * alpha;
  if (fabs(corr) <= 6.0554544523933395e-06) return;
  const double rho = rho_t / corr;
  if constexpr (F == TG_FP64) {
    A.S.X.rho[i] = rho;
  } else {
    A.S.X.rho[i] = __double2float_rn(rho - T.rho0);
  }
}

}  // namespace tg
