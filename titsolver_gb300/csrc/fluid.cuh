// fluid.cuh - stage kernels of the GB300 WCSPH step, templated on dimension
// (D = 2, 3), arithmetic form (TG_FP64, TG_FP32C) and smoothing kernel K.
//
// One stage of the reference's SSPRK substep (time_integrator.hpp:190-210:
// prepare, [dt], continuity, momentum, Euler update; then lincomb) runs as:
//   radix sort  stable sort of the cell keys (sort.cu)
//   k_cell_table
//   k_reorder   gather the state into cell order, pack neighbour records,
//               Tait p, cs (+ the dt min-reduction in the first stage)
//   k_walls     Shepard extrapolation of the wall density
//               (FluidEquations::setup_boundary, fluid_equations.hpp:122-164)
//   k_forces    fused continuity + momentum sums in gather form, Euler
//               update, SSPRK linear combination, and the cell key (and
//               FP32 cell offset) of the new position for the next sort
//               (fluid_equations.hpp:232-305, time_integrator.hpp:203-223)
// Keys come from FP64 positions in k_keys only after an upload; afterwards
// k_forces and k_walls write them, so no kernel recomputes cells from FP64
// positions (FP64 issue is scarce on GB300).
#pragma once

#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "faces.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// Records.
struct alignas(16) Pos64_2 { double x, y; };
struct alignas(32) Pos64_3 { double x, y, z, w; };
struct alignas(32) Dat64 { double vx, vy, vz, rho, P, c, invrho, pad; };
struct alignas(8) Pos32_2 { float x, y; };

struct alignas(16) Pos32_3 { float x, y, z, w; };
struct alignas(32) Dat32 { float vx, vy, vz, drho, P, c, invrho, pad; };

template<int D, int F>
struct Layout;
template<int D>
struct Layout<D, TG_FP64> {
  using R = double;
  using PosRec = std::conditional_t<D == 2, Pos64_2, Pos64_3>;
  using DatRec = Dat64;
};
template<int D>
struct Layout<D, TG_FP32C> {
  using R = float;
  using PosRec = std::conditional_t<D == 2, Pos32_2, Pos32_3>;
  using DatRec = Dat32;
};

__device__ __forceinline__ void load_pos(const Pos64_2* p, uint32_t j,
                                         double* x) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p + j));
  x[0] = a.x;
  x[1] = a.y;
}
__device__ __forceinline__ void load_pos(const Pos64_3* p, uint32_t j,
                                         double* x) {
  const double2* q = reinterpret_cast<const double2*>(p + j);
  const double2 a = __ldg(q), b = __ldg(q + 1);
  x[0] = a.x;
  x[1] = a.y;
  x[2] = b.x;
}
__device__ __forceinline__ void load_pos(const Pos32_2* p, uint32_t j,
                                         float* x) {
  const float2 a = __ldg(reinterpret_cast<const float2*>(p + j));
  x[0] = a.x;
  x[1] = a.y;
}
__device__ __forceinline__ void load_pos(const Pos32_3* p, uint32_t j,
                                         float* x) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p + j));
  x[0] = a.x;
  x[1] = a.y;
  x[2] = a.z;
}
__device__ __forceinline__ Dat64 load_dat(const Dat64* p, uint32_t j) {
  const double2* q = reinterpret_cast<const double2*>(p + j);
  const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2),
                d = __ldg(q + 3);
  return Dat64{a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y};
}
__device__ __forceinline__ Dat32 load_dat(const Dat32* p, uint32_t j) {
  const float4* q = reinterpret_cast<const float4*>(p + j);
  const float4 a = __ldg(q), b = __ldg(q + 1);
  return Dat32{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}
// Coherent (non-__ldg) loads for kernels that also write the record array.
__device__ __forceinline__ Dat64 load_dat_coherent(const Dat64* p,
                                                   uint32_t j) {
  return p[j];
}
__device__ __forceinline__ Dat32 load_dat_coherent(const Dat32* p,
                                                   uint32_t j) {
  return p[j];
}

// ---------------------------------------------------------------------------
// Buffers.
template<class R>
struct StateBuf {
  double* pos[3];
  R* vel[3];
  R* rho;  // FP64: rho; FP32C: rho - rho0
  R* dv[3];
  R* drho;
  uint32_t* id;   // upload index | kWallBit for walls
  uint32_t* key;  // global cell key (home state only)
  uint32_t* pkey;  // key of each slot at the sort that set the home order
                   // (home state only; the re-sort's previous keys)
  float* off[3];  // FP32C: offset from the cell corner (home state only)
};

template<class R>
struct StartBuf {
  double* pos[3];
  R* vel[3];
  R* rho;
};

template<int D, int F>
struct StageArgs {
  using L = Layout<D, F>;
  using R = typename L::R;
  StateBuf<R> X, Y;
  StartBuf<R> Usrc, Udst;
  const uint32_t* perm;
  const uint32_t* skey;  // sorted keys (cell order)
  typename L::PosRec* posrec;
  typename L::DatRec* datrec;
  const uint32_t* cell_start;
  const TankDev* tanks;
  const uint32_t* tank_off;  // first global cell of each tank
  int ntanks;
  PhysDev phys;
  double* dt;
  uint32_t* wall_list;
  uint32_t* wall_count;   // [0] walls listed, [1] walls near fluid
  uint32_t* wall_active;  // the walls near fluid (k_wall_select)
  uint32_t* err;
  int64_t n;
  int k;             // cells per radius
  int copy_start;    // stage 0: Udst = current state
  int compute_dt;    // stage 0: min-reduce dt
  int lincomb;       // apply (1 - w) Udst + w new
  double w_new;
  int kahan;
  int carry;         // gather every field into Y (prepare and split passes)
  int mode;          // update rule of the force pass (kPass*)
  int walls_keep;    // k_walls: keep the carried wall densities
  unsigned* fbox;     // per-tank fluid bounding box (k_reorder)
  FaceArgs fc;        // boundary faces (fc.on = 0: particle walls)
};

// Order-preserving map of floats to unsigned 32-bit integers (and back),
// for atomic min/max of coordinates of either sign.
__device__ __forceinline__ unsigned order_enc(float x) {
  const unsigned b = __float_as_uint(x);
  return (b >> 31) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float order_dec(unsigned e) {
  return __uint_as_float((e >> 31) ? (e & 0x7fffffffu) : ~e);
}

// Fold a lane's fluid position (tank-local FP32 coordinates, x - lo) into
// its tank's bounding box.  Each warp reduces its lanes (one instruction
// per bound) when they share a tank; the block then merges its warps and
// issues at most one atomic per bound and tank run, and only when it would
// move the box (cell order makes the slowest axis grow block after block,
// so per-warp atomics would queue on one address).  Warps that straddle
// tanks fold lane by lane.  Called by every thread of the block.
template<int D>
__device__ __forceinline__ void fold_fluid_box(unsigned* box, int ntanks,
                                               uint32_t tk, bool fluid,
                                               const float* xl) {
  constexpr uint32_t kEmpty = 0xffffffffu, kMixed = 0xfffffffeu;
  __shared__ unsigned s_lo[32][3], s_hi[32][3];
  __shared__ uint32_t s_tk[32];
  unsigned lo[3], hi[3];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    lo[k] = fluid ? order_enc(xl[k]) : 0xffffffffu;
    hi[k] = fluid ? order_enc(xl[k]) : 0u;
  }
  const uint32_t key_tk = fluid ? tk : kEmpty;
  const uint32_t t0 = __reduce_min_sync(0xffffffffu, key_tk);
  const bool one_tank = __all_sync(0xffffffffu, key_tk == t0 || key_tk == kEmpty);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto push = [&](uint32_t t, const unsigned* l, const unsigned* h) {
    unsigned* mins = box + 3 * t;
    unsigned* maxs = box + 3 * (ntanks + t);
#pragma unroll
    for (int k = 0; k < D; ++k) {
      if (l[k] < *reinterpret_cast<volatile unsigned*>(mins + k)) atomicMin(mins + k, l[k]);
      if (h[k] > *reinterpret_cast<volatile unsigned*>(maxs + k)) atomicMax(maxs + k, h[k]);
    }
  };
  if (one_tank) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      lo[k] = __reduce_min_sync(0xffffffffu, lo[k]);
      hi[k] = __reduce_max_sync(0xffffffffu, hi[k]);
    }
  } else if (fluid) {
    push(tk, lo, hi);
  }
  if (lane == 0) {
    s_tk[warp] = one_tank ? t0 : kMixed;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      s_lo[warp][k] = lo[k];
      s_hi[warp][k] = hi[k];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    uint32_t cur = kEmpty;
    unsigned clo[3] = {0u, 0u, 0u}, chi[3] = {0u, 0u, 0u};
    for (int w = 0; w < nw; ++w) {
      const uint32_t t = s_tk[w];
      if (t == kEmpty || t == kMixed) continue;
      if (t != cur) {
        if (cur != kEmpty) push(cur, clo, chi);
        cur = t;
#pragma unroll
        for (int k = 0; k < D; ++k) {
          clo[k] = s_lo[w][k];
          chi[k] = s_hi[w][k];
        }
      } else {
#pragma unroll
        for (int k = 0; k < D; ++k) {
          clo[k] = min(clo[k], s_lo[w][k]);
          chi[k] = max(chi[k], s_hi[w][k]);
        }
      }
    }
    if (cur != kEmpty) push(cur, clo, chi);
  }
}

// True when no fluid particle of the tank can lie within the support radius
// of a point with tank-local FP32 coordinates xl: its distance to the
// tank's fluid bounding box exceeds R plus a margin that covers the FP32
// rounding of both coordinates (wall_skip_r2_f), or the tank has no fluid
// this stage.
template<int D>
__device__ __forceinline__ bool beyond_fluid(const unsigned* box, int ntanks,
                                             uint32_t tk, const TankDev& T,
                                             const float* xl) {
  if (box == nullptr) return false;  // no box this stage: walk every wall
  float g2 = 0.f;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const unsigned elo = box[3 * tk + k];
    const unsigned ehi = box[3 * (ntanks + tk) + k];
    if (elo > ehi) return true;  // empty box
    const float g = fmaxf(fmaxf(order_dec(elo) - xl[k], xl[k] - order_dec(ehi)), 0.f);
    g2 += g * g;
  }
  return g2 > T.wall_skip_r2_f;
}

// Tank-local FP32 coordinates: from the FP64 position (FP64 form) or from
// the cell index and the FP32 offset from the cell corner (compensated
// form, FP32 only).
template<int D>
__device__ __forceinline__ void local_coords(const TankDev& T, const double* p,
                                             float* xl) {
#pragma unroll
  for (int k = 0; k < D; ++k) xl[k] = __double2float_rn(p[k] - T.lo[k]);
}
template<int D>
__device__ __forceinline__ void local_coords(const TankDev& T, const int* c,
                                             const float* o, float* xl) {
#pragma unroll
  for (int k = 0; k < D; ++k) xl[k] = fmaf(static_cast<float>(c[k]), T.cs_f, o[k]);
}

// Update rules of a force pass.  The SSPRK stage uses both sums; the split
// passes of the symplectic Euler and velocity Verlet integrators
// (time_integrator.hpp:50-69, 99-123) use one sum each and carry the other
// field through unchanged.
enum {
  kPassRK = 0,         // r += dt v, v += dt dv, rho += dt drho (+ lincomb)
  kPassContinuity,     // rho += dt drho
  kPassKickDrift,      // v += dt dv, then r += dt v
  kPassHalfKickDrift,  // v += dt/2 dv, then r += dt v
  kPassHalfKick        // v += dt/2 dv
};

// ---------------------------------------------------------------------------
// Neighbour-cell traversal over the (2k+1)^D block of cells around c,
// clipped to the tank grid.  cstart is indexed by key (2 per cell).
// Merged: one [begin, end) range per row of cells (rows are contiguous in
// key order), fluid and walls, with the row offset (0, dy, dz).  Per cell: one range per cell with its cell
// offset (dx, dy, dz) relative to c; FluidOnly restricts each cell's range
// to its fluid particles.
//
// With the target's offset o from its own cell's corner (o == nullptr: no
// clipping), rows and cells that cannot hold a point within the cull radius
// (the support radius widened by 2^-12, far above the FP32 rounding of the
// offsets) are skipped: a row whose y/z gap to the target exceeds it, and
// cells beyond the row's half-width.  Skipped cells hold no neighbour, so
// every sum is bit-identical to the unclipped traversal.  Rows and columns
// on the grid border are never clipped (particles clamped into border
// cells may lie outside their cell's box).

// Distance from offset o to the cell box [d cs, (d + 1) cs) along one axis.
__device__ __forceinline__ float cell_gap(int d, float o, float cs) {
  if (d > 0) return fmaxf(static_cast<float>(d) * cs - o, 0.f);
  if (d < 0) return fmaxf(o - static_cast<float>(d + 1) * cs, 0.f);
  return 0.f;
}

// FP32 offset of an FP64 position from the corner of its cell c.
template<int D>
__device__ __forceinline__ void cell_offset(const TankDev& T, const int* c,
                                            const double* p, float* o) {
#pragma unroll
  for (int k = 0; k < D; ++k) {
    o[k] = __double2float_rn(p[k] - fma(static_cast<double>(c[k]), T.cs, T.lo[k]));
  }
}

// Clipped x-range of one row: [x0, x1] within [xlo, xhi]; false when the
// row holds no reachable cell.
template<int D>
__device__ __forceinline__ bool clip_row(const TankDev& T, const int* c,
                                         const float* o, int y, int z,
                                         int xlo, int xhi, int& x0, int& x1) {
  x0 = xlo;
  x1 = xhi;
  if (o == nullptr) return true;
  const float cs = T.cs_f;
  const float gy = (y == 0 || y == T.nc[1] - 1) ? 0.f : cell_gap(y - c[1], o[1], cs);
  float gz = 0.f;
  if constexpr (D == 3) {
    gz = (z == 0 || z == T.nc[2] - 1) ? 0.f : cell_gap(z - c[2], o[2], cs);
  }
  const float rem = T.cull_r2_f - gy * gy - gz * gz;
  if (rem < 0.f) return false;
  if (xlo == 0 || xhi == T.nc[0] - 1) return true;
  const float w = sqrtf(rem);
  // dx > 0 reachable iff dx cs - o0 <= w; dx < 0 iff o0 - (dx + 1) cs <= w.
  // The cull radius exceeds R by R / 4096, so w exceeds the half-width of
  // the support in this row by at least R / 4096, far beyond the rounding
  // of a multiplication by 1 / cs: no cell holding a neighbour is clipped.
  const float hi = floorf((o[0] + w) * T.inv_cs_f);
  const float lo = ceilf((o[0] - w) * T.inv_cs_f) - 1.f;
  x1 = min(xhi, c[0] + static_cast<int>(fminf(fmaxf(hi, 0.f), 64.f)));
  x0 = max(xlo, c[0] + static_cast<int>(fmaxf(fminf(lo, 0.f), -64.f)));
  return true;
}

template<int D, bool PerCell, class Fn, bool FluidOnly = false>
__device__ __forceinline__ void for_cells(const TankDev& T, const int* c,
                                          int k,
                                          const uint32_t* __restrict__ cstart,
                                          Fn&& fn, const float* o = nullptr) {
  const int nx = T.nc[0], ny = T.nc[1];
  const int zlo = D == 3 ? max(c[2] - k, 0) : 0;
  const int zhi = D == 3 ? min(c[2] + k, T.nc[2] - 1) : 0;
  const int ylo = max(c[1] - k, 0), yhi = min(c[1] + k, ny - 1);
  const int xlo = max(c[0] - k, 0), xhi = min(c[0] + k, nx - 1);
  for (int z = zlo; z <= zhi; ++z) {
    for (int y = ylo; y <= yhi; ++y) {
      int x0, x1;
      if (!clip_row<D>(T, c, o, y, z, xlo, xhi, x0, x1)) continue;
      const uint32_t row =
          T.cell_off + (static_cast<uint32_t>(z) * ny + y) * nx;
      if constexpr (!PerCell) {
        fn(__ldg(cstart + 2 * (row + x0)), __ldg(cstart + 2 * (row + x1 + 1)),
           0, y - c[1], D == 3 ? z - c[2] : 0);
      } else if constexpr (FluidOnly) {
        for (int x = x0; x <= x1; ++x) {
          const uint32_t kc = 2 * (row + x);
          fn(__ldg(cstart + kc), __ldg(cstart + kc + 1), x - c[0], y - c[1],
             D == 3 ? z - c[2] : 0);
        }
      } else {
        // The next cell's end is loaded before this cell is walked (2D
        // compensated force pass: 1.2% faster per step; loading the next
        // row's range ahead in the row mode measured 4% slower in 3D).
        uint32_t s = __ldg(cstart + 2 * (row + x0));
        uint32_t e = __ldg(cstart + 2 * (row + x0 + 1));
        for (int x = x0; x <= x1; ++x) {
          const uint32_t en = x < x1 ? __ldg(cstart + 2 * (row + x + 2)) : 0u;
          fn(s, e, x - c[0], y - c[1], D == 3 ? z - c[2] : 0);
          s = e;
          e = en;
        }
      }
    }
  }
}

// The (2k+1)^D cell block around c, dealt out to the lanes of a team: lane
// l of a team of `team` lanes visits cells l, l + team, ... of the block
// (cells, not particles, are split, so no lane repeats another lane's
// cell-table reads).  Each visit gets the cell's fluid range (FluidOnly) or
// its whole range, fluid then walls, with the cell offset (dx, dy, dz).
template<int D, bool FluidOnly, class Fn>
__device__ __forceinline__ void for_cells_team(
    const TankDev& T, const int* c, int k,
    const uint32_t* __restrict__ cstart, int lane, int team, Fn&& fn,
    const float* o = nullptr) {
  const int nx = T.nc[0], ny = T.nc[1];
  const int zlo = D == 3 ? max(c[2] - k, 0) : 0;
  const int zhi = D == 3 ? min(c[2] + k, T.nc[2] - 1) : 0;
  const int ylo = max(c[1] - k, 0), yhi = min(c[1] + k, ny - 1);
  const int xlo = max(c[0] - k, 0), xhi = min(c[0] + k, nx - 1);
  const int wx = xhi - xlo + 1, wy = yhi - ylo + 1, wz = zhi - zlo + 1;
  const int total = wx * wy * wz;
  for (int t = lane; t < total; t += team) {
    const int x = xlo + t % wx;
    const int rest = t / wx;
    const int y = ylo + rest % wy;
    const int z = zlo + rest / wy;
    if (o != nullptr) {
      // Skip a cell whose box lies beyond the cull radius (border cells
      // are always visited; see for_cells).
      const float cs = T.cs_f;
      const float gx = (x == 0 || x == nx - 1) ? 0.f : cell_gap(x - c[0], o[0], cs);
      const float gy = (y == 0 || y == ny - 1) ? 0.f : cell_gap(y - c[1], o[1], cs);
      float g2 = gx * gx + gy * gy;
      if constexpr (D == 3) {
        const float gz =
            (z == 0 || z == T.nc[2] - 1) ? 0.f : cell_gap(z - c[2], o[2], cs);
        g2 += gz * gz;
      }
      if (g2 > T.cull_r2_f) continue;
    }
    const uint32_t kc =
        2 * (T.cell_off + (static_cast<uint32_t>(z) * ny + y) * nx + x);
    fn(__ldg(cstart + kc), __ldg(cstart + kc + (FluidOnly ? 1 : 2)),
       x - c[0], y - c[1], D == 3 ? z - c[2] : 0);
  }
}

// Rows of the (2k+1)^D cell block around c (3D), dealt out to the lanes of
// a team: lane l visits rows l, l + team, ...; each visit gets the row's
// whole record range (fluid and walls, clipped as in for_cells) and its
// offset (0, dy, dz).
template<int D, class Fn>
__device__ __forceinline__ void for_rows_team(
    const TankDev& T, const int* c, int k,
    const uint32_t* __restrict__ cstart, int lane, int team, Fn&& fn,
    const float* o) {
  const int nx = T.nc[0], ny = T.nc[1];
  const int zlo = D == 3 ? max(c[2] - k, 0) : 0;
  const int zhi = D == 3 ? min(c[2] + k, T.nc[2] - 1) : 0;
  const int ylo = max(c[1] - k, 0), yhi = min(c[1] + k, ny - 1);
  const int xlo = max(c[0] - k, 0), xhi = min(c[0] + k, nx - 1);
  const int wy = yhi - ylo + 1;
  const int rows = wy * (zhi - zlo + 1);
  for (int t = lane; t < rows; t += team) {
    const int y = ylo + t % wy;
    const int z = zlo + t / wy;
    int x0, x1;
    if (!clip_row<D>(T, c, o, y, z, xlo, xhi, x0, x1)) continue;
    const uint32_t row = T.cell_off + (static_cast<uint32_t>(z) * ny + y) * nx;
    fn(__ldg(cstart + 2 * (row + x0)), __ldg(cstart + 2 * (row + x1 + 1)), 0,
       y - c[1], D == 3 ? z - c[2] : 0);
  }
}

// Mask of the `team` lanes (aligned, a power of two) that hold this lane.
template<int Team>
__device__ __forceinline__ unsigned team_mask() {
  if constexpr (Team >= 32) {
    return 0xffffffffu;
  } else {
    const unsigned base = (threadIdx.x & 31u) & ~static_cast<unsigned>(Team - 1);
    return ((1u << Team) - 1u) << base;
  }
}

// Bit-exact squared distance: d = a - b per axis, then
// (d0*d0 + d1*d1) + d2*d2, every operation rounded (no FMA contraction),
// as the oracle's BSphere::contains restatement.
template<int D>
__device__ __forceinline__ double dist2_exact(const double* a,
                                              const double* b, double* d) {
#pragma unroll
  for (int k = 0; k < D; ++k) d[k] = __dsub_rn(a[k], b[k]);
  double s = __dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1]));
  if constexpr (D == 3) s = __dadd_rn(s, __dmul_rn(d[2], d[2]));
  return s;
}
template<int D>
__device__ __forceinline__ float dist2_exact(const float* a, const float* b,
                                             float* d) {
#pragma unroll
  for (int k = 0; k < D; ++k) d[k] = __fsub_rn(a[k], b[k]);
  float s = __fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1]));
  if constexpr (D == 3) s = __fadd_rn(s, __fmul_rn(d[2], d[2]));
  return s;
}

// The compensated form's neighbour predicate.  Its FP32 squared distance
// s2_f comes from cell-relative offsets, each rounded once from an exact
// FP64 difference.  With u = 2^-24, offsets within a cell size cs (plus a
// few ulps) of their cell corner and the candidate's cell within k cells of
// the target's (cs = R / k), each FP32 component of r_ab is within
// (3k + 3) u cs + u |r_ab| <= 7 u R of the exact one (the FP64 cell corners
// add 2^-52 of the coordinates, negligible within 2^20 cells of the
// origin), so |s2_f - s2| < 32 u R^2: far inside the band R^2 (1 -+ 2^-14)
// = R^2 (1 -+ 1024 u).  Below the band the pair is a neighbour, above it is
// not; inside it the reference's own predicate decides (dist2_exact on the
// cell-ordered FP64 positions against the FP64 R^2), so the set is exactly
// the reference's.  A particle clamped into a border cell may carry an
// offset of any size, so a target whose block of cells reaches a border
// cell decides every candidate in FP64 (the grid's margins keep every
// particle more than k cells from its border unless it left the grid).
struct Band {
  float lo, hi;
};

// Band of a target in cell c whose traversal covers cells c -+ k: the
// tank's band, or (lo, hi) = (-1, inf), every candidate decided in FP64,
// when that block of cells reaches a border cell.
template<int D>
__device__ __forceinline__ Band target_band(const TankDev& T, const int* c, int k) {
  bool b = c[0] - k <= 0 || c[0] + k >= T.nc[0] - 1 || c[1] - k <= 0 ||
           c[1] + k >= T.nc[1] - 1;
  if constexpr (D == 3) b = b || c[2] - k <= 0 || c[2] + k >= T.nc[2] - 1;
  return b ? Band{-1.f, __int_as_float(0x7f800000)} : Band{T.band_lo_f, T.band_hi_f};
}

// The reference predicate |r_a - r_b|^2 <= R^2 on the FP64 positions of
// cell-order slots a and b.
template<int D>
__device__ __forceinline__ bool within_fp64(double* const* pos, uint32_t a,
                                            uint32_t b, double R2) {
  // (d0^2 + d1^2) + d2^2 axis by axis, rounded as dist2_exact.
  double d = __dsub_rn(pos[0][a], pos[0][b]);
  double s = __dmul_rn(d, d);
#pragma unroll
  for (int k = 1; k < D; ++k) {
    d = __dsub_rn(pos[k][a], pos[k][b]);
    s = __dadd_rn(s, __dmul_rn(d, d));
  }
  return s <= R2;
}

__device__ __forceinline__ bool finite_bits(double x) {
  return (static_cast<unsigned long long>(__double_as_longlong(x)) &
          0x7ff0000000000000ull) != 0x7ff0000000000000ull;
}

// ---------------------------------------------------------------------------
// Cell key (and FP32 offset) of every home particle from its FP64 position;
// runs after an upload.  The tank comes from the upload index.
template<int D, int F>
__global__ void __launch_bounds__(256)
    k_keys(StateBuf<typename Layout<D, F>::R> X,
           const uint32_t* __restrict__ tank_of,
           const TankDev* __restrict__ tanks, int64_t n, uint32_t* err) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const TankDev& T = tanks[tank_of[X.id[i] & kIdMask]];
  double p[3] = {X.pos[0][i], X.pos[1][i], D == 3 ? X.pos[2][i] : 0.0};
  int c[3] = {0, 0, 0};
  bool outside = false;
  cell_of<D>(T, p, c, outside);
  X.key[i] = key_of(flat_cell<D>(T, c), (X.id[i] & kWallBit) != 0);
  if constexpr (F == TG_FP32C) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      X.off[k][i] = static_cast<float>(p[k] - (T.lo[k] + c[k] * T.cs));
    }
  }
  if (outside) {
    bool finite = true;
#pragma unroll
    for (int k = 0; k < D; ++k) finite = finite && isfinite(p[k]);
    atomicOr(err, finite ? static_cast<uint32_t>(TG_DEV_OUTSIDE_GRID)
                         : static_cast<uint32_t>(TG_DEV_NONFINITE_STATE));
  }
}

// Record of a wall whose sums are empty (rho(0)), or that keeps its
// carried density rho (a split pass without a prepare): zero velocity and
// the equation of state of the density, as k_walls writes them.
template<int D>
__device__ __forceinline__ Dat64 wall_record(const PhysDev& P, const TankDev& T,
                                             double rho, bool keep) {
  const double rho_e = keep ? rho : density_from_potential_f64(P, T, 0.0);
  double pr, cc;
  tait_f64(P, T, rho_e, pr, cc);
  const double inv = 1.0 / rho_e;
  return Dat64{0.0, 0.0, 0.0, rho_e, pr * inv * inv, cc, inv, 0.0};
}
template<int D>
__device__ __forceinline__ Dat32 wall_record(const PhysDev& P, const TankDev& T,
                                             float rho, bool keep) {
  const float rho_e = keep ? rho : deviation_from_potential_f32(P, T, 0.f);
  float pr, cc;
  tait_f32(P, T, rho_e, pr, cc);
  const float inv = 1.f / (T.rho0_f + rho_e);
  return Dat32{0.f, 0.f, 0.f, rho_e, pr * inv * inv, cc, inv, 0.f};
}

// Home state of the wall at cell-order slot e, written by the pass over all
// particles that follows the wall pass (force pass, prepare commit or
// shift): its gathered position and id, zero velocity, acceleration and
// density rate, the density of its record, its sorted key and, in the
// compensated form, its cell offset.
template<int D, int F>
__device__ __forceinline__ void commit_wall(const StageArgs<D, F>& A, int64_t e,
                                            uint32_t id) {
  using R = typename StageArgs<D, F>::R;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    A.X.pos[k][e] = A.Y.pos[k][e];
    A.X.vel[k][e] = R(0);
    A.X.dv[k][e] = R(0);
  }
  if constexpr (F == TG_FP64) {
    A.X.rho[e] = A.datrec[e].rho;
  } else {
    A.X.rho[e] = A.datrec[e].drho;
    float o[3] = {0.f, 0.f, 0.f};
    load_pos(A.posrec, static_cast<uint32_t>(e), o);
#pragma unroll
    for (int k = 0; k < D; ++k) A.X.off[k][e] = o[k];
  }
  A.X.drho[e] = R(0);
  A.X.id[e] = id;
  A.X.key[e] = A.skey[e];
  A.X.pkey[e] = A.skey[e];
}

// ---------------------------------------------------------------------------
template<int D, int F>
__global__ void __launch_bounds__(256) k_reorder(StageArgs<D, F> A) {
  using R = typename StageArgs<D, F>::R;
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const bool valid = j < A.n;
  double dt_a = __longlong_as_double(0x7ff0000000000000ll);
  uint32_t tk = 0xffffffffu;
  float box_xl[3] = {0.f, 0.f, 0.f};  // fluid position for the bounding box
  bool box_fluid = false;
  if (valid) {
    const uint32_t src = A.perm[j];
    const uint32_t key = A.skey[j];
    tk = tank_of_key(key, A.tank_off, A.ntanks);
    const TankDev& T = A.tanks[tk];
    double p[3];
    R v[3];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      p[k] = A.X.pos[k][src];
      v[k] = A.X.vel[k][src];
    }
    const R rho = A.X.rho[src];
    const uint32_t id = A.X.id[src];
    box_fluid = !(id & kWallBit);
    if (A.fbox != nullptr && box_fluid) {
      if constexpr (F == TG_FP64) {
        local_coords<D>(T, p, box_xl);
      } else {
        int cc[3] = {0, 0, 0};
        float oo[3] = {0.f, 0.f, 0.f};
        cell_from_key<D>(T, key, cc);
#pragma unroll
        for (int k = 0; k < D; ++k) oo[k] = A.X.off[k][src];
        local_coords<D>(T, cc, oo, box_xl);
      }
    }
#pragma unroll
    for (int k = 0; k < D; ++k) A.Y.pos[k][j] = p[k];
    A.Y.id[j] = id;
    if (A.carry) {
#pragma unroll
      for (int k = 0; k < D; ++k) {
        A.Y.vel[k][j] = v[k];
        A.Y.dv[k][j] = A.X.dv[k][src];
      }
      A.Y.rho[j] = rho;
      A.Y.drho[j] = A.X.drho[src];
    }
    if (A.copy_start) {
#pragma unroll
      for (int k = 0; k < D; ++k) {
        A.Udst.pos[k][j] = p[k];
        A.Udst.vel[k][j] = v[k];
      }
      A.Udst.rho[j] = rho;
    } else {
#pragma unroll
      for (int k = 0; k < D; ++k) {
        A.Udst.pos[k][j] = A.Usrc.pos[k][src];
        A.Udst.vel[k][j] = A.Usrc.vel[k][src];
      }
      A.Udst.rho[j] = A.Usrc.rho[src];
    }
    // Neighbour position record.
    if constexpr (F == TG_FP64) {
      if constexpr (D == 2) {
        A.posrec[j] = Pos64_2{p[0], p[1]};
      } else {
        A.posrec[j] = Pos64_3{p[0], p[1], p[2], 0.0};
      }
    } else {
      float o[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < D; ++k) o[k] = A.X.off[k][src];
      if constexpr (D == 2) {
        A.posrec[j] = Pos32_2{o[0], o[1]};
      } else {
        // w: the cell's x index as a float, its sign bit (kWallBit) set for
        // a wall, so that a whole row of cells can be read as one range
        // (k_forces and k_walls, 3D compensated form): |w| - (target's cell
        // x) is the candidate's cell offset, exactly.
        int cc[3] = {0, 0, 0};
        cell_from_key<D>(T, key, cc);
        const unsigned wbits = __float_as_uint(static_cast<float>(cc[0])) |
                               (id & kWallBit ? kWallBit : 0u);
        A.posrec[j] = Pos32_3{o[0], o[1], o[2], __uint_as_float(wbits)};
      }
    }
    if (id & kWallBit) {
      const uint32_t slot = atomicAdd(A.wall_count, 1u);
      A.wall_list[slot] = static_cast<uint32_t>(j);
      // rho(0), or the carried density: k_walls overwrites the records of
      // the walls near fluid.
      A.datrec[j] = wall_record<D>(A.phys, T, rho, A.walls_keep != 0);
    } else {
      // Tait state of the fluid particle.
      if constexpr (F == TG_FP64) {
        double pr, c;
        tait_f64(A.phys, T, rho, pr, c);
        const double inv = 1.0 / rho;
        A.datrec[j] = Dat64{v[0], v[1], D == 3 ? v[2] : 0.0, rho,
                            pr * inv * inv, c, inv, 0.0};
        if (A.compute_dt) {
          double dvv[3];
#pragma unroll
          for (int k = 0; k < D; ++k) dvv[k] = A.X.dv[k][src];
          double v2 = v[0] * v[0] + v[1] * v[1];
          double a2 = dvv[0] * dvv[0] + dvv[1] * dvv[1];
          if constexpr (D == 3) {
            v2 += v[2] * v[2];
            a2 += dvv[2] * dvv[2];
          }
          const double h = T.h;
          const double dt_ac = A.phys.cfl * h / (c + sqrt(v2));
          const double dt_vi = A.phys.c_visc * h * h * rho / A.phys.mu;
          const double dt_fo =
              A.phys.c_force * sqrt(h / fmax(sqrt(a2), A.phys.g));
          dt_a = fmin(dt_ac, fmin(dt_vi, dt_fo));
        }
      } else {
        float pr, c;
        tait_f32(A.phys, T, rho, pr, c);
        const float inv = __frcp_rn(T.rho0_f + rho);
        A.datrec[j] = Dat32{v[0], v[1], D == 3 ? v[2] : 0.f, rho,
                            pr * inv * inv, c, inv, 0.f};
        if (A.compute_dt) {
          float dvv[3];
#pragma unroll
          for (int k = 0; k < D; ++k) dvv[k] = A.X.dv[k][src];
          float v2 = v[0] * v[0] + v[1] * v[1];
          float a2 = dvv[0] * dvv[0] + dvv[1] * dvv[1];
          if constexpr (D == 3) {
            v2 += v[2] * v[2];
            a2 += dvv[2] * dvv[2];
          }
          const float h = T.h_f;
          const float rhof = T.rho0_f + rho;
          const float dt_ac = A.phys.cfl_f * h / (c + sqrtf(v2));
          const float dt_vi = A.phys.c_visc_f * h * h * rhof / A.phys.mu_f;
          const float dt_fo =
              A.phys.c_force_f * sqrtf(h / fmaxf(sqrtf(a2), A.phys.g_f));
          dt_a = static_cast<double>(fminf(dt_ac, fminf(dt_vi, dt_fo)));
        }
      }
    }
  }
  if (A.fbox != nullptr) fold_fluid_box<D>(A.fbox, A.ntanks, tk, box_fluid, box_xl);
  if (A.compute_dt) {
    // Warp-level min when the whole warp is in one tank, else per lane.
    const uint32_t t0 = __shfl_sync(0xffffffffu, tk, 0);
    if (__all_sync(0xffffffffu, tk == t0 || tk == 0xffffffffu)) {
      double m = dt_a;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
      }
      if ((threadIdx.x & 31) == 0 && t0 != 0xffffffffu &&
          m < __longlong_as_double(0x7ff0000000000000ll)) {
        atomic_min_pos(A.dt + t0, m);
      }
    } else if (valid && dt_a < __longlong_as_double(0x7ff0000000000000ll)) {
      atomic_min_pos(A.dt + tk, dt_a);
    }
  }
}

// ---------------------------------------------------------------------------
// Wall extrapolation (fluid_equations.hpp:122-164) with a zero wall normal:
//   rho_e = rho(H),  H = sum_b V_b H(rho_b) W_be / sum_b V_b W_be over fluid
//   neighbours b (H = 0 when the Shepard sum is tiny); v_e = 0.
// k_reorder writes every wall's record with rho(0) (or, in a split pass
// with no prepare before it, the carried density); this pass overwrites
// the records of the walls within the support radius of their tank's fluid
// bounding box (for the others the sums are empty, so rho(0) is their
// value).  k_wall_select lists those walls (all of them when the pass has
// no fluid box); k_walls then runs a grid of teams of wall_team lanes over
// the list, each team taking walls in turn, so no team idles while others
// hold long runs of listed walls.  A team splits the wall's cells (2D) or
// rows of cells (3D, fluid records only) and reduces by shuffles.  The
// walls' home state is written by the next pass over all particles
// (commit_wall).  Team widths measured per step in the compensated form:
// 3D 4 lanes 0.7% (one tank) to 1.8% (64 tanks) faster than 8, and 16
// slower; 2D 8 lanes 0.5% faster than 4.  The FP64 form keeps 8.
template<int D, int F>
constexpr int wall_team() {
  return D == 3 && F == TG_FP32C ? 4 : 8;
}

template<int D, int F>
__global__ void __launch_bounds__(256)
    k_wall_select(StageArgs<D, F> A, int64_t n_walls) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  bool act = false;
  uint32_t e = 0;
  if (t < n_walls) {
    e = A.wall_list[t];
    const uint32_t key = A.skey[e];
    const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
    const TankDev& T = A.tanks[tk];
    float xl[3] = {0.f, 0.f, 0.f};
    if constexpr (F == TG_FP64) {
      double pe[3] = {0.0, 0.0, 0.0};
      load_pos(A.posrec, e, pe);
      local_coords<D>(T, pe, xl);
    } else {
      int c[3] = {0, 0, 0};
      float oe[3] = {0.f, 0.f, 0.f};
      cell_from_key<D>(T, key, c);
      load_pos(A.posrec, e, oe);
      local_coords<D>(T, c, oe, xl);
    }
    act = !beyond_fluid<D>(A.fbox, A.ntanks, tk, T, xl);
  }
  // One atomic per warp.
  const unsigned mask = __ballot_sync(0xffffffffu, act);
  const int lane = static_cast<int>(threadIdx.x & 31u);
  uint32_t base = 0;
  if (lane == 0 && mask != 0u) base = atomicAdd(A.wall_count + 1, static_cast<uint32_t>(__popc(mask)));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (act) A.wall_active[base + __popc(mask & ((1u << lane) - 1u))] = e;
}

template<int D, int F, int K>
__global__ void __launch_bounds__(128)
    k_walls(StageArgs<D, F> A) {
  // A split pass without a prepare: the walls keep the carried densities
  // k_reorder put in their records.
  if (A.walls_keep) return;
  const bool all = A.fbox == nullptr;
  const uint32_t* list = all ? A.wall_list : A.wall_active;
  const int64_t count = all ? A.wall_count[0] : A.wall_count[1];
  constexpr int kWallTeam = wall_team<D, F>();
  const int tl = static_cast<int>(threadIdx.x % kWallTeam);
  const int team_in_warp = static_cast<int>((threadIdx.x & 31u) / kWallTeam);
  const unsigned tmask = ((1u << kWallTeam) - 1u) << (team_in_warp * kWallTeam);
  const int64_t teams = static_cast<int64_t>(gridDim.x) * blockDim.x / kWallTeam;
  for (int64_t w = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / kWallTeam;
       w < count; w += teams) {
    const uint32_t ew = list[w];
    const uint32_t key = A.skey[ew];
    const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
    const TankDev& T = A.tanks[tk];
    int c[3] = {0, 0, 0};
    cell_from_key<D>(T, key, c);
    if constexpr (F == TG_FP64) {
      double pe[3] = {0.0, 0.0, 0.0};
      load_pos(A.posrec, ew, pe);
      const double R2 = T.radius2, hinv = T.hinv, w = T.w, m = T.m;
      double S = 0.0, H = 0.0;
      // Face boundaries: the wall normal n_e = normalize(grad gamma) and the
      // hydrostatic term g (r_be . n_e) n_e[1] (fluid_equations.hpp:146-160);
      // zero with particle walls.
      double ne[3] = {0.0, 0.0, 0.0};
      if (A.fc.on) normalize_d<D>(A.fc.ggam + D * static_cast<size_t>(ew), ne);
      auto visit = [&](uint32_t s, uint32_t en, int, int, int) {
        for (uint32_t j = s; j < en; ++j) {
          double pb[3], d[3];
          load_pos(A.posrec, j, pb);
          const double s2 = dist2_exact<D>(pb, pe, d);
          if (s2 > R2) continue;
          const Dat64 b = load_dat(A.datrec, j);
          const double W = w * KernelPoly<K>::value(sqrt(s2) * hinv);
          const double Vb = m * b.invrho;
          double Hb = potential_f64(A.phys, T, b.rho);
          if (A.fc.on) Hb += A.phys.g * dot_d<D>(d, ne) * ne[1];
          S += Vb * W;
          H += Vb * Hb * W;
        }
      };
      float oc[3] = {0.f, 0.f, 0.f};
      cell_offset<D>(T, c, pe, oc);
      for_cells_team<D, true>(T, c, A.k, A.cell_start, tl, kWallTeam, visit, oc);
#pragma unroll
      for (int o = kWallTeam / 2; o > 0; o >>= 1) {
        S += __shfl_xor_sync(tmask, S, o, kWallTeam);
        H += __shfl_xor_sync(tmask, H, o, kWallTeam);
      }
      if (tl == 0) {
        const double Hs = fabs(S) <= 6.0554544523933395e-06 ? 0.0 : H / S;
        const double rho_e = density_from_potential_f64(A.phys, T, Hs);
        double pr, cc;
        tait_f64(A.phys, T, rho_e, pr, cc);
        const double inv = 1.0 / rho_e;
        A.datrec[ew] = Dat64{0.0, 0.0, 0.0, rho_e, pr * inv * inv, cc, inv, 0.0};
      }
    } else {
      const float hinv = T.hinv_f;
      const float w = T.w_f, m = T.m_f;
      const float csz = T.cs_f;
      float oe[3] = {0.f, 0.f, 0.f};
      load_pos(A.posrec, ew, oe);
      Kahan S, H;
      // Face boundaries: wall normal and hydrostatic term (see the FP64
      // path); here r_be = -d.
      float nef[3] = {0.f, 0.f, 0.f};
      if (A.fc.on) {
        double ne[3];
        normalize_d<D>(A.fc.ggam + D * static_cast<size_t>(ew), ne);
#pragma unroll
        for (int k = 0; k < D; ++k) nef[k] = static_cast<float>(ne[k]);
      }
      const Band bd = target_band<D>(T, c, A.k);
      if constexpr (D == 3) {
        // One range per row of cells (records carry the cell's x index and
        // the wall bit), fluid records only.
        auto visit_row = [&](uint32_t s, uint32_t en, int, int dy, int dz) {
          const float oey = oe[1] - dy * csz;
          const float oez = oe[2] - dz * csz;
          for (uint32_t j = s; j < en; ++j) {
            const Pos32_3 b = A.posrec[j];
            if (__float_as_uint(b.w) & kWallBit) continue;
            const float dxc = b.w - static_cast<float>(c[0]);
            float d[3];
            d[0] = (oe[0] - dxc * csz) - b.x;
            d[1] = oey - b.y;
            d[2] = oez - b.z;
            const float s2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (s2 > bd.hi) continue;
            if (s2 >= bd.lo && !within_fp64<D>(A.Y.pos, ew, j, T.radius2)) continue;
            const Dat32 bdat = load_dat(A.datrec, j);
            const float W = w * KernelPoly<K>::value(sqrtf(s2) * hinv);
            const float Vb = m * bdat.invrho;
            float Hb = potential_f32(A.phys, T, bdat.drho);
            if (A.fc.on) {
              Hb -= A.phys.g_f * (d[0] * nef[0] + d[1] * nef[1] + d[2] * nef[2]) * nef[1];
            }
            S.add(Vb * W);
            H.add(Vb * Hb * W);
          }
        };
        for_rows_team<D>(T, c, A.k, A.cell_start, tl, kWallTeam, visit_row, oe);
      } else {
        auto visit = [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
          float oes[3];
          oes[0] = oe[0] - dx * csz;
          oes[1] = oe[1] - dy * csz;
          oes[2] = D == 3 ? oe[2] - dz * csz : 0.f;
          for (uint32_t j = s; j < en; ++j) {
            float ob[3], d[3];
            load_pos(A.posrec, j, ob);
            const float s2 = dist2_exact<D>(oes, ob, d);
            if (s2 > bd.hi) continue;
            if (s2 >= bd.lo && !within_fp64<D>(A.Y.pos, ew, j, T.radius2)) continue;
            const Dat32 b = load_dat(A.datrec, j);
            const float W = w * KernelPoly<K>::value(sqrtf(s2) * hinv);
            const float Vb = m * b.invrho;
            float Hb = potential_f32(A.phys, T, b.drho);
            if (A.fc.on) {
              float dn = d[0] * nef[0] + d[1] * nef[1];
              if constexpr (D == 3) dn += d[2] * nef[2];
              Hb -= A.phys.g_f * dn * nef[1];
            }
            S.add(Vb * W);
            H.add(Vb * Hb * W);
          }
        };
        for_cells_team<D, true>(T, c, A.k, A.cell_start, tl, kWallTeam, visit, oe);
      }
      float Ss = S.value(), Hv = H.value();
#pragma unroll
      for (int o = kWallTeam / 2; o > 0; o >>= 1) {
        Ss += __shfl_xor_sync(tmask, Ss, o, kWallTeam);
        Hv += __shfl_xor_sync(tmask, Hv, o, kWallTeam);
      }
      if (tl == 0) {
        const float Hs = fabsf(Ss) <= 6.0554544523933395e-06f ? 0.f : Hv / Ss;
        const float rho_e = deviation_from_potential_f32(A.phys, T, Hs);
        float pr, cc;
        tait_f32(A.phys, T, rho_e, pr, cc);
        const float inv = 1.f / (T.rho0_f + rho_e);
        A.datrec[ew] = Dat32{0.f, 0.f, 0.f, rho_e, pr * inv * inv, cc, inv, 0.f};
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Fused continuity + momentum + update, gather form.  For a fluid target a
// and every neighbour b != a (walls included):
//   drho_a += m F [ v_ab . r_ab + D_ab ],            grad W_ab = F r_ab
//   dv_a   += m (Pi_ab - P_ab) F r_ab,               dv_a starts at -g e_1
// with P_ab = p_a/rho_a^2 + p_b/rho_b^2 and
//   Ferrari  D_ab = max(c_a, c_b)(rho_a - rho_b) |r_ab| / rho_b
//   Molteni  D_ab = 2 delta h c0 (rho_a - rho_b) / rho_b
//   Morris   Pi_ab = 2 mu (v_ab . r_ab) / (rho_a rho_b |r_ab|^2)
//   Monaghan Pi_ab = alpha h (c_a+c_b) (v_ab.r_ab) / ((|r|^2 + 0.01h^2)
//                    (rho_a+rho_b)) for v_ab . r_ab < 0, else 0
// then r' = r + dt v, v' = v + dt dv, rho' = rho + dt drho and, in the later
// SSPRK stages, u = (1 - w) u_n + w u'.  Last, the key (and FP32 offset)
// of the new position for the next sort.

// Band-list entries per thread of the compensated force pass (shared
// memory: a count and kBandCap slots of two words each), and the band's upper
// end over its lower end: (1 + 2^-14) / (1 - 2^-14) rounded up to
// 1 + 2^-13 + 2^-26 (any band containing R^2 (1 -+ 2^-15) is exact).
constexpr int kBandCap = 4;
constexpr float kBandRatio = 1.0f + 1.0f / 8192.0f + 1.0f / 67108864.0f;

// Resident 128-thread blocks per SM requested for k_forces: 8 for the
// compensated form (64 registers; in 2D measured 2% faster than 10 blocks
// at 48 registers once the band handling joined the pass), 4 for FP64 (its
// FP64 pipe is the limit).
template<int D, int F>
constexpr int forces_min_blocks() {
  return F == TG_FP32C ? 8 : 4;
}

// Physics presets the compensated force kernel is specialised for (the
// per-pair term choices become compile-time): generic reads them at run
// time.
enum { kPhysGeneric = 0, kPhysTextbook = 1, kPhysReference = 2 };

// Pair sums of the compensated form for one target.
template<int D, int K, int Phys = kPhysGeneric>
struct PairF32 {
  float va[3];
  Dat32 a;
  float hinv, wg, m, mu2, ah, eps2, dk, rho0x2;
  int visc, diff;
  bool kahan;
  Kahan drho, dv[3];
  // Plain partial sums of the current cell or row range; the compensated
  // accumulators take one add per range (close) instead of one per pair.
  float pd, pv[3];

  __device__ __forceinline__ void open() {
    pd = 0.f;
    pv[0] = pv[1] = pv[2] = 0.f;
  }
  __device__ __forceinline__ void close() {
    if (Phys != kPhysGeneric || kahan) {
      drho.add(pd);
#pragma unroll
      for (int k = 0; k < D; ++k) dv[k].add(pv[k]);
    } else {
      drho.s += pd;
#pragma unroll
      for (int k = 0; k < D; ++k) dv[k].s += pv[k];
    }
  }

  __device__ __forceinline__ void init(const PhysDev& P, const TankDev& T,
                                       const Dat32& own, int kahan_on) {
    a = own;
    va[0] = own.vx;
    va[1] = own.vy;
    va[2] = own.vz;
    hinv = T.hinv_f;
    wg = T.wg_f;
    m = T.m_f;
    mu2 = 2.f * P.mu_f;
    ah = P.alpha_f * T.h_f;
    eps2 = T.visc_eps2_f;
    dk = T.diff_k_f;
    rho0x2 = 2.f * T.rho0_f;
    visc = P.viscosity;
    diff = P.diffusion;
    kahan = kahan_on != 0;
    dv[1].s = -P.g_f;
  }

  // One neighbour at r_ab = d (|d|^2 = s2, within the support, b != a).
  __device__ __forceinline__ void add(const float* d, float s2, const Dat32& b) {
    const float rinv = rsqrtf(s2);
    const float r = s2 * rinv;
    const float q = r * hinv;
    const float Fk = grad_factor<K>(q, rinv, wg, hinv);
    const float vb[3] = {b.vx, b.vy, b.vz};
    float vd = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) vd += (va[k] - vb[k]) * d[k];
    const float drab = a.drho - b.drho;
    const int df = Phys == kPhysTextbook    ? TG_DIFF_MOLTENI
                   : Phys == kPhysReference ? TG_DIFF_FERRARI
                                            : diff;
    const int vs = Phys == kPhysTextbook    ? TG_VISC_MONAGHAN
                   : Phys == kPhysReference ? TG_VISC_MORRIS
                                            : visc;
    float cont = vd;
    if (df == TG_DIFF_FERRARI) {
      cont += fmaxf(a.c, b.c) * drab * r * b.invrho;
    } else if (df == TG_DIFF_MOLTENI) {
      cont += dk * drab * b.invrho;
    }
    const float dr = m * Fk * cont;
    float Pi;
    if (vs == TG_VISC_MORRIS) {
      Pi = mu2 * vd * a.invrho * b.invrho * (rinv * rinv);
    } else {
      Pi = vd < 0.f ? __fdividef(ah * vd * (a.c + b.c),
                                 (s2 + eps2) * (rho0x2 + a.drho + b.drho))
                    : 0.f;
    }
    const float coef = m * (Pi - (a.P + b.P)) * Fk;
    pd += dr;
#pragma unroll
    for (int k = 0; k < D; ++k) pv[k] += coef * d[k];
  }
};

// Euler update (time_integrator.hpp:203-207), SSPRK lincomb (:212-223) and
// the cell key (and FP32 offset) of the new position; positions in FP64,
// the rest in the form's type.
template<int D, int F>
__device__ __forceinline__ void forces_epilogue(
    const StageArgs<D, F>& A, int64_t i, uint32_t id, uint32_t tk,
    const TankDev& T, const int* c, const typename StageArgs<D, F>::R* va,
    typename StageArgs<D, F>::R rho_self,
    const typename StageArgs<D, F>::R* dv_out,
    typename StageArgs<D, F>::R drho_out) {
  using R = typename StageArgs<D, F>::R;
  const double dt = A.dt[tk];
  const int mode = A.mode;
  const bool half = mode == kPassHalfKickDrift || mode == kPassHalfKick;
  const double dt_v = half ? 0.5 * dt : dt;  // velocity kick
  R dtr, dtr_v;
  if constexpr (F == TG_FP64) {
    dtr = dt;
    dtr_v = dt_v;
  } else {
    dtr = __double2float_rn(dt);
    dtr_v = __double2float_rn(dt_v);
  }
  double pn[3] = {0.0, 0.0, 0.0};
  R vn[3];
  R dv_keep[3];
  R rn = rho_self;
  R drho_keep = drho_out;
  if (mode == kPassRK) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      pn[k] = fma(dt, static_cast<double>(va[k]), A.Y.pos[k][i]);
      vn[k] = va[k] + dtr * dv_out[k];
      dv_keep[k] = dv_out[k];
    }
    rn = rho_self + dtr * drho_out;
  } else if (mode == kPassContinuity) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      pn[k] = A.Y.pos[k][i];
      vn[k] = va[k];
      dv_keep[k] = A.Y.dv[k][i];
    }
    rn = rho_self + dtr * drho_out;
  } else {
    const bool drift = mode != kPassHalfKick;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      vn[k] = va[k] + dtr_v * dv_out[k];
      pn[k] = drift ? fma(dt, static_cast<double>(vn[k]), A.Y.pos[k][i])
                    : A.Y.pos[k][i];
      dv_keep[k] = dv_out[k];
    }
    drho_keep = A.Y.drho[i];
  }
  if (A.lincomb) {
    const double w = A.w_new, w0 = 1.0 - A.w_new;
    R wr, w0r;
    if constexpr (F == TG_FP64) {
      wr = w;
      w0r = w0;
    } else {
      wr = __double2float_rn(w);
      w0r = __double2float_rn(w0);
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
      pn[k] = fma(w0, A.Udst.pos[k][i], w * pn[k]);
      vn[k] = w0r * A.Udst.vel[k][i] + wr * vn[k];
    }
    rn = w0r * A.Udst.rho[i] + wr * rn;
  }
  int cn[3] = {0, 0, 0};
  if constexpr (F == TG_FP64) {
    bool outside = false;
    cell_of<D>(T, pn, cn, outside);
    if (outside) atomicOr(A.err, static_cast<uint32_t>(TG_DEV_OUTSIDE_GRID));
  } else {
    // Offset from the old cell corner (exact FP64 difference, rounded once),
    // then a shift by whole cells in FP32, clamped at the grid border.
    bool outside = false;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const float o = __double2float_rn(
          pn[k] - fma(static_cast<double>(c[k]), T.cs, T.lo[k]));
      const float f = floorf(__fdividef(o, T.cs_f));
      int ck = c[k] + (isfinite(f) ? static_cast<int>(f) : 0);
      if (ck < 0 || ck >= T.nc[k]) {
        outside = true;
        ck = min(max(ck, 0), T.nc[k] - 1);
      }
      cn[k] = ck;
      A.X.off[k][i] = o - static_cast<float>(ck - c[k]) * T.cs_f;
    }
    if (outside) atomicOr(A.err, static_cast<uint32_t>(TG_DEV_OUTSIDE_GRID));
  }
  A.X.pkey[i] = A.skey[i];  // read before the key write: the buffers may alias
  A.X.key[i] = key_of(flat_cell<D>(T, cn), false);
  bool finite = true;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    A.X.pos[k][i] = pn[k];
    A.X.vel[k][i] = vn[k];
    A.X.dv[k][i] = dv_keep[k];
    finite = finite && finite_bits(pn[k]) && isfinite(vn[k]);
  }
  A.X.rho[i] = rn;
  A.X.drho[i] = drho_keep;
  A.X.id[i] = id;
  if (!(finite && isfinite(rn))) {
    atomicOr(A.err, static_cast<uint32_t>(TG_DEV_NONFINITE_STATE));
  }
}

// Face boundaries (fluid_equations.hpp:241-247, 276-292): per adjacent face
// s (a vertex pair, whose fields are averages; vertices have zero velocity)
//   drho_a -= rho_s (v_as . grad gamma_as) / gamma_a
//   dv_a   += (P_as grad gamma_as - Pi_as |grad gamma_as|) / gamma_a,
//   P_as = rho_s (p_a / rho_a^2 + p_s / rho_s^2),
//   Pi_as = 2 mu / (rho_a dr_as) (v_as . t_as) t_as,
//   dr_as = max(h / 2, (r_a - r_s) . n_s), n_s = normalize(grad gamma_as),
//   t_as = normalize(v_as - (v_as . n_s) n_s).
// k_face_terms stores these per particle (FP64, both forms) before the
// force pass, which divides its pair sums by gamma_a, adds them and adds
// gravity; the face integrals stay out of the force loop's registers.

// Density of a face vertex from its data record (either form).
__device__ __forceinline__ double vertex_rho(const Dat64* dat, uint32_t j,
                                             const TankDev&) {
  return load_dat(dat, j).rho;
}
__device__ __forceinline__ double vertex_rho(const Dat32* dat, uint32_t j,
                                             const TankDev& T) {
  return T.rho0 + static_cast<double>(load_dat(dat, j).drho);
}

// Target fields from a data record: velocity, density, P = p / rho^2.
__device__ __forceinline__ void target_fields(const Dat64& a, const TankDev&,
                                              double* v, double& rho, double& P) {
  v[0] = a.vx;
  v[1] = a.vy;
  v[2] = a.vz;
  rho = a.rho;
  P = a.P;
}
__device__ __forceinline__ void target_fields(const Dat32& a, const TankDev& T,
                                              double* v, double& rho, double& P) {
  v[0] = a.vx;
  v[1] = a.vy;
  v[2] = a.vz;
  rho = T.rho0 + static_cast<double>(a.drho);
  P = a.P;
}

// Global cell of a particle's key.
template<int D>
__device__ __forceinline__ uint32_t global_cell(const TankDev& T, const int* c) {
  uint32_t g = static_cast<uint32_t>(c[1]) * T.nc[0] + c[0];
  if constexpr (D == 3) g += static_cast<uint32_t>(c[2]) * T.nc[1] * T.nc[0];
  return T.cell_off + g;
}

// Face vertex average of a scalar: (a + b)/2 or (a + b + c)/3
// (field.hpp:59-64, core/math.hpp:130).
template<int D>
__device__ __forceinline__ double face_avg(const double* x) {
  if constexpr (D == 2) return (x[0] + x[1]) / 2.0;
  else return (x[0] + x[1] + x[2]) / 3.0;
}

// Face terms of continuity and momentum (fluid_equations.hpp:241-247,
// 278-291) of the face particles, one warp per particle with the lanes
// splitting its faces; k_gamma_init zeroed the other particles' terms.
template<int D, int K, int F, class FT>
__global__ void __launch_bounds__(128) k_face_terms(StageArgs<D, F> A) {
  const FaceArgs& fc = A.fc;
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  const uint32_t count = *fc.face_count;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += nwarps) {
    const uint32_t i = fc.face_list[w];
    if (A.Y.id[i] & kWallBit) continue;
    const uint32_t key = A.skey[i];
    const TankDev& T = A.tanks[tank_of_key(key, A.tank_off, A.ntanks)];
    int c[3] = {0, 0, 0};
    cell_from_key<D>(T, key, c);
    const uint32_t gcell = global_cell<D>(T, c);
    double pa[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; ++k) pa[k] = A.Y.pos[k][i];
    const double radius = KernelPoly<K>::unit_radius * T.h;
    const double gam = fc.gamma[i];
    double va[3], rho_a, P_a;
    target_fields(load_dat(A.datrec, i), T, va, rho_a, P_a);
    double drho = 0.0, dv[3] = {0.0, 0.0, 0.0};
    for_adjacent_faces<D>(fc, gcell, pa, radius, lane,
                          [&](bool active, uint32_t f, const double* g) {
      // Each face's flux is weighted by its own vertex densities and
      // pressures, so no edges cancel here.
      double gg[3];
      face_flux_d<K, D, FT>(active, g, face_axes<D>(fc, f), pa, T.h, fc.weight, gg);
      if (!active) return;
      double rv[3], pv[3];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        double cj;
        rv[j] = vertex_rho(A.datrec, fc.slot_of[fc.vert[D * f + j]], T);
        tait_f64(A.phys, T, rv[j], pv[j], cj);
      }
      const double rho_s = face_avg<D>(rv);
      const double p_s = face_avg<D>(pv);
      // The face vertices' velocities are zero (no-slip walls), so
      // v_as = v_a.
      drho -= rho_s * dot_d<D>(va, gg) / gam;
      const double P_as = rho_s * (P_a + p_s / (rho_s * rho_s));
      double n_s[3], t_as[3], vt[3], r_as[3];
      normalize_d<D>(gg, n_s);
      const double vn = dot_d<D>(va, n_s);
#pragma unroll
      for (int k = 0; k < D; ++k) vt[k] = va[k] - vn * n_s[k];
      normalize_d<D>(vt, t_as);
#pragma unroll
      for (int k = 0; k < D; ++k) {
        double xk[3];
#pragma unroll
        for (int j = 0; j < D; ++j) xk[j] = g[D * j + k];
        r_as[k] = pa[k] - face_avg<D>(xk);
      }
      const double dr_as = fmax(T.h / 2.0, dot_d<D>(r_as, n_s));
      const double Pi_s = 2.0 * A.phys.mu / (rho_a * dr_as) * dot_d<D>(va, t_as);
      const double ng = sqrt(dot_d<D>(gg, gg));
#pragma unroll
      for (int k = 0; k < D; ++k) dv[k] += (P_as * gg[k] - Pi_s * t_as[k] * ng) / gam;
    });
    drho = warp_sum(drho);
#pragma unroll
    for (int k = 0; k < D; ++k) dv[k] = warp_sum(dv[k]);
    if (lane == 0) {
      fc.face_drho[i] = drho;
#pragma unroll
      for (int k = 0; k < D; ++k) fc.face_dv[D * i + k] = dv[k];
    }
  }
}

// The force pass's share: pair sums over gamma, plus the stored face terms
// and gravity.
template<int D, int F>
__device__ __forceinline__ void apply_face_terms(const StageArgs<D, F>& A,
                                                 int64_t i, double& drho,
                                                 double* dv) {
  const double gam = A.fc.gamma[i];
  drho = drho / gam + A.fc.face_drho[i];
#pragma unroll
  for (int k = 0; k < D; ++k) dv[k] = dv[k] / gam + A.fc.face_dv[D * i + k];
  dv[1] -= A.phys.g;
}

// The compensated form's band handling for one target (see target_band):
// candidates in the band around R^2 are deferred during the walk to this
// thread's column of a short shared-memory list (slot and the offset code
// of their cell, 2D, or row, 3D), then decided by the FP64 predicate; a full
// list leaves them to a second walk over the band.  The sorted keys cannot
// give a deferred candidate's cell: the force pass rewrites the home keys,
// which may share their buffer.  `exact` is the walk that decides in FP64:
// every candidate (a target whose block reaches a border cell) or the
// band's only (after an overflow).
template<int D, int K, int Phys>
struct BandWalk {
  const StageArgs<D, TG_FP32C>& A;
  const TankDev& T;
  PairF32<D, K, Phys>& acc;
  const float* oa;
  const int* c;
  float csz, lo;
  uint32_t ia;
  uint32_t *n, *slot, *code;

  __device__ __forceinline__ void init(uint32_t* smem) {
    n = smem + threadIdx.x;
    slot = smem + blockDim.x + threadIdx.x;
    code = smem + (1 + kBandCap) * blockDim.x + threadIdx.x;
    *n = 0u;
  }
  __device__ __forceinline__ void defer(uint32_t j, uint32_t cd) {
    const uint32_t e = *n;
    if (e < static_cast<uint32_t>(kBandCap)) {
      slot[e * blockDim.x] = j;
      code[e * blockDim.x] = cd;
    }
    *n = e + 1u;
  }
  // r_ab of candidate j seen from offset (u, v) cells: 2D (dx, dy); 3D
  // (dy, dz), the x offset from the record's cell index.
  __device__ __forceinline__ void rab(uint32_t j, int u, int v, float* d) const {
    if constexpr (D == 2) {
      float ob[2];
      load_pos(A.posrec, j, ob);
      d[0] = (oa[0] - u * csz) - ob[0];
      d[1] = (oa[1] - v * csz) - ob[1];
    } else {
      const Pos32_3 b = A.posrec[j];
      const float dxc = fabsf(b.w) - static_cast<float>(c[0]);
      d[0] = (oa[0] - dxc * csz) - b.x;
      d[1] = (oa[1] - u * csz) - b.y;
      d[2] = (oa[2] - v * csz) - b.z;
    }
  }
  __device__ __forceinline__ void exact(uint32_t s, uint32_t en, int dx, int dy, int dz,
                                        bool band_only) {
    float oas[3];
    oas[0] = oa[0] - dx * csz;
    oas[1] = oa[1] - dy * csz;
    oas[2] = D == 3 ? oa[2] - dz * csz : 0.f;
    acc.open();
    for (uint32_t j = s; j < en; ++j) {
      if (j == ia) continue;
      float ob[3], d[3];
      load_pos(A.posrec, j, ob);
#pragma unroll
      for (int k = 0; k < D; ++k) d[k] = oas[k] - ob[k];
      float s2 = d[0] * d[0] + d[1] * d[1];
      if constexpr (D == 3) s2 += d[2] * d[2];
      if (band_only && (s2 < lo || s2 > lo * kBandRatio)) continue;
      if (!within_fp64<D>(A.Y.pos, ia, j, T.radius2)) continue;
      acc.add(d, s2, load_dat(A.datrec, j));
    }
    acc.close();
  }
  // The deferred candidates: the FP64 decision, then r_ab as the walk
  // computed it.  False when the list overflowed.
  __device__ __forceinline__ bool decide() {
    const uint32_t nb = *n;
    if (nb == 0u) return true;
    if (nb > static_cast<uint32_t>(kBandCap)) return false;
    acc.open();
    for (uint32_t e = 0; e < nb; ++e) {
      const uint32_t j = slot[e * blockDim.x];
      if (!within_fp64<D>(A.Y.pos, ia, j, T.radius2)) continue;
      const uint32_t cd = code[e * blockDim.x];
      float d[3];
      rab(j, static_cast<int>(cd >> 3) - 3, static_cast<int>(cd & 7u) - 3, d);
      float s2 = d[0] * d[0] + d[1] * d[1];
      if constexpr (D == 3) s2 += d[2] * d[2];
      acc.add(d, s2, load_dat(A.datrec, j));
    }
    acc.close();
    return true;
  }
};

// Team lanes share one target: each takes every Team-th cell of the block
// and the team merges its partial sums by shuffles (compensated merges in
// the FP32 form), so a warp advances 32 / Team targets.  The block size is
// a run-time choice (a multiple of 32, at most 256) at the register budget
// of forces_min_blocks 128-thread blocks per SM.
template<int D, int F, int K, int Phys = kPhysGeneric, int Team = 1>
__global__ void __launch_bounds__(256, forces_min_blocks<D, F>() / 2)
    k_forces(StageArgs<D, F> A) {
  using R = typename StageArgs<D, F>::R;
  const int64_t gt = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t i = gt / Team;
  const int lane = Team == 1 ? 0 : static_cast<int>(threadIdx.x % Team);
  // Every exit below is uniform over a team (its lanes share i).
  if (i >= A.n) return;
  const uint32_t id = A.Y.id[i];
  if (id & kWallBit) {
    if (lane == 0) commit_wall(A, i, id);
    return;
  }
  const uint32_t key = A.skey[i];
  const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
  const TankDev& T = A.tanks[tk];
  int c[3] = {0, 0, 0};
  cell_from_key<D>(T, key, c);
  R dv_out[3] = {R(0), R(0), R(0)};
  R drho_out;
  R va[3];
  R rho_self;
  if constexpr (F == TG_FP64) {
    const int visc = A.phys.viscosity, diff = A.phys.diffusion;
    double pa[3] = {0.0, 0.0, 0.0};
    load_pos(A.posrec, static_cast<uint32_t>(i), pa);
    const Dat64 a = load_dat(A.datrec, static_cast<uint32_t>(i));
    va[0] = a.vx;
    va[1] = a.vy;
    va[2] = a.vz;
    rho_self = a.rho;
    const double R2 = T.radius2, hinv = T.hinv, wg = T.wg, m = T.m;
    const double mu2 = 2.0 * A.phys.mu, ah = A.phys.alpha * T.h;
    const double eps2 = T.visc_eps2, dk = T.diff_k;
    double drho = 0.0;
    // Face boundaries: gravity is added after the gamma division.
    const bool faces = A.fc.on;
    double dv[3] = {0.0, (lane == 0 && !faces) ? -A.phys.g : 0.0, 0.0};
    auto visit = [&](uint32_t s, uint32_t en, int, int, int) {
      for (uint32_t j = s; j < en; ++j) {
        if (j == static_cast<uint32_t>(i)) continue;
        double pb[3], d[3];
        load_pos(A.posrec, j, pb);
        const double s2 = dist2_exact<D>(pa, pb, d);
        if (s2 > R2) continue;
        const Dat64 b = load_dat(A.datrec, j);
        const double rinv = rsqrt(s2);
        const double r = s2 * rinv;
        const double q = r * hinv;
        const double Fk = grad_factor<K>(q, rinv, wg, hinv);
        const double vb[3] = {b.vx, b.vy, b.vz};
        double vd = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) vd += (va[k] - vb[k]) * d[k];
        const double drab = a.rho - b.rho;
        double cont = vd;
        if (diff == TG_DIFF_FERRARI) {
          cont += fmax(a.c, b.c) * drab * r * b.invrho;
        } else if (diff == TG_DIFF_MOLTENI) {
          cont += dk * drab * b.invrho;
        }
        drho += m * Fk * cont;
        double Pi;
        if (visc == TG_VISC_MORRIS) {
          Pi = mu2 * vd * a.invrho * b.invrho * (rinv * rinv);
        } else {
          Pi = vd < 0.0 ? ah * vd * (a.c + b.c) /
                              ((s2 + eps2) * (a.rho + b.rho))
                        : 0.0;
        }
        const double coef = m * (Pi - (a.P + b.P)) * Fk;
#pragma unroll
        for (int k = 0; k < D; ++k) dv[k] += coef * d[k];
      }
    };
    float oc[3] = {0.f, 0.f, 0.f};
    cell_offset<D>(T, c, pa, oc);
    if constexpr (Team == 1) {
      for_cells<D, false>(T, c, A.k, A.cell_start, visit, oc);
    } else {
      for_cells_team<D, false>(T, c, A.k, A.cell_start, lane, Team, visit, oc);
      const unsigned mask = team_mask<Team>();
#pragma unroll
      for (int o = Team / 2; o > 0; o >>= 1) {
        drho += __shfl_xor_sync(mask, drho, o, Team);
#pragma unroll
        for (int k = 0; k < D; ++k) dv[k] += __shfl_xor_sync(mask, dv[k], o, Team);
      }
      if (lane != 0) return;
    }
    if (faces) apply_face_terms(A, i, drho, dv);
#pragma unroll
    for (int k = 0; k < D; ++k) dv_out[k] = dv[k];
    drho_out = drho;
  } else {
    PairF32<D, K, Phys> acc;
    acc.init(A.phys, T, load_dat(A.datrec, static_cast<uint32_t>(i)), A.kahan);
    // Gravity once per target; with face boundaries after the gamma division.
    const bool faces = A.fc.on;
    if (lane != 0 || faces) acc.dv[1].s = 0.f;
    float oa[3] = {0.f, 0.f, 0.f};
    load_pos(A.posrec, static_cast<uint32_t>(i), oa);
    const float csz = T.cs_f;
    const uint32_t ia = static_cast<uint32_t>(i);
    // The band around the support radius (see target_band and BandWalk):
    // the walk keeps one FP32 threshold on its common path; below band_lo a
    // candidate is a neighbour, at or above it it is dropped unless it lies
    // in the band, where it is deferred.
    const Band bd = target_band<D>(T, c, A.k);
    const float lo = bd.lo;
    extern __shared__ uint32_t s_band[];
    BandWalk<D, K, Phys> bw{A, T, acc, oa, c, csz, lo, ia};
    bw.init(s_band);
    auto visit = [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
      float oas[3];
      oas[0] = oa[0] - dx * csz;
      oas[1] = oa[1] - dy * csz;
      oas[2] = D == 3 ? oa[2] - dz * csz : 0.f;
      const uint32_t code = D == 2 ? static_cast<uint32_t>(((dx + 3) << 3) | (dy + 3))
                                   : static_cast<uint32_t>(((dy + 3) << 3) | (dz + 3));
      acc.open();
      for (uint32_t j = s; j < en; ++j) {
        if (j == ia) continue;
        float ob[3], d[3];
        load_pos(A.posrec, j, ob);
#pragma unroll
        for (int k = 0; k < D; ++k) d[k] = oas[k] - ob[k];
        float s2 = d[0] * d[0] + d[1] * d[1];
        if constexpr (D == 3) s2 += d[2] * d[2];
        if (s2 >= lo) {
          if (s2 <= lo * kBandRatio) bw.defer(j, code);
          continue;
        }
        acc.add(d, s2, load_dat(A.datrec, j));
      }
      acc.close();
    };
    // 3D: one range per row of cells; each candidate's x offset is moved
    // to the target's cell by its cell's x index (record word w).  Same
    // candidates in the same order as the per-cell walk.
    auto visit_row = [&](uint32_t s, uint32_t en, int, int dy, int dz) {
      if constexpr (D == 3) {
        const float oay = oa[1] - dy * csz;
        const float oaz = oa[2] - dz * csz;
        const uint32_t code = static_cast<uint32_t>(((dy + 3) << 3) | (dz + 3));
        acc.open();
        // The next record is loaded while this one is tested (3D: measured
        // 2.6% faster per step; slower in 2D).  Loading it unconditionally
        // (past the range's end too) measured 2.3% slower per step.
        const float c0 = static_cast<float>(c[0]);
        Pos32_3 bn{};
        if (s < en) bn = A.posrec[s];
        for (uint32_t j = s; j < en; ++j) {
          const Pos32_3 b = bn;
          if (j + 1 < en) bn = A.posrec[j + 1];
          if (j == ia) continue;
          const float dxc = fabsf(b.w) - c0;
          float d[3];
          d[0] = (oa[0] - dxc * csz) - b.x;
          d[1] = oay - b.y;
          d[2] = oaz - b.z;
          const float s2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
          if (s2 >= lo) {
            if (s2 <= lo * kBandRatio) bw.defer(j, code);
            continue;
          }
          acc.add(d, s2, load_dat(A.datrec, j));
        }
        acc.close();
      }
    };
    auto exact_all = [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
      bw.exact(s, en, dx, dy, dz, false);
    };
    auto exact_band = [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
      bw.exact(s, en, dx, dy, dz, true);
    };
    auto decide_band = [&]() {
      if (bw.decide()) return;
      if constexpr (Team == 1) {
        for_cells<D, true>(T, c, A.k, A.cell_start, exact_band, oa);
      } else {
        for_cells_team<D, false>(T, c, A.k, A.cell_start, lane, Team, exact_band, oa);
      }
    };
    if (lo < 0.f) {
      // Near the grid border: every candidate in FP64.
      if constexpr (Team == 1) {
        for_cells<D, true>(T, c, A.k, A.cell_start, exact_all, oa);
      } else {
        for_cells_team<D, false>(T, c, A.k, A.cell_start, lane, Team, exact_all, oa);
      }
    } else if constexpr (Team == 1 && D == 3) {
      for_cells<D, false>(T, c, A.k, A.cell_start, visit_row, oa);
      decide_band();
    } else if constexpr (Team == 1) {
      // 2D: per cell (8-byte records; measured faster than row ranges over
      // 16-byte records).
      for_cells<D, true>(T, c, A.k, A.cell_start, visit, oa);
      decide_band();
    } else {
      for_cells_team<D, false>(T, c, A.k, A.cell_start, lane, Team, visit, oa);
      decide_band();
    }
    if constexpr (Team > 1) {
      const unsigned mask = team_mask<Team>();
#pragma unroll
      for (int o = Team / 2; o > 0; o >>= 1) {
        acc.drho.merge(__shfl_xor_sync(mask, acc.drho.s, o, Team),
                       __shfl_xor_sync(mask, acc.drho.c, o, Team));
#pragma unroll
        for (int k = 0; k < D; ++k) {
          acc.dv[k].merge(__shfl_xor_sync(mask, acc.dv[k].s, o, Team),
                          __shfl_xor_sync(mask, acc.dv[k].c, o, Team));
        }
      }
      if (lane != 0) return;
    }
#pragma unroll
    for (int k = 0; k < D; ++k) {
      va[k] = acc.va[k];
      dv_out[k] = acc.dv[k].value();
    }
    rho_self = acc.a.drho;
    drho_out = acc.drho.value();
    if (faces) {
      double drho = drho_out;
      double dv[3] = {dv_out[0], dv_out[1], dv_out[2]};
      apply_face_terms(A, i, drho, dv);
      drho_out = static_cast<float>(drho);
#pragma unroll
      for (int k = 0; k < D; ++k) dv_out[k] = static_cast<float>(dv[k]);
    }
  }
  forces_epilogue<D, F>(A, i, id, tk, T, c, va, rho_self, dv_out, drho_out);
}

// Bulk copies (cp.async.bulk, global to this CTA's shared memory) behind
// an mbarrier.  Addresses and sizes are multiples of 16 bytes.
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Waits for phase `parity` of the barrier, at most `spins` polls; false
// when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int spins) {
  for (int it = 0; it < spins; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}
constexpr int kCopySpins = 1 << 20;

// 2D compensated form with the block's neighbour window staged in shared
// memory.  A block of 128 consecutive (cell-ordered) targets whose first
// and last target share a tank and a row of cells needs, for every target,
// only the 2k+1 rows around that row over x in [x_first - k, x_last + k];
// each of those row segments is contiguous in cell order, so one thread
// copies them (position and data records, rounded out to 16-byte
// boundaries) into shared memory with bulk copies that complete on an
// mbarrier, and every target then reads its candidates from there.  Blocks
// that straddle rows or tanks, or whose window exceeds the staging
// capacity, read from global memory as k_forces does; so does a block
// whose copies do not complete within the wait limit (flagged in the
// device error word).
constexpr int kStageCap = 800;  // records: 800 x (8 + 32) B = 32 KB
constexpr int kStageRows = 7;   // 2k + 1 for k <= 3

template<int K>
__global__ void __launch_bounds__(128, 7)
    k_forces_staged2(StageArgs<2, TG_FP32C> A) {
  __shared__ __align__(16) float2 s_pos[kStageCap];
  __shared__ __align__(16) float4 s_dat[2 * kStageCap];
  __shared__ uint32_t s_gbeg[kStageRows], s_goff[kStageRows + 1];
  __shared__ int s_ok, s_rows, s_ylo;
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ uint32_t s_band[(1 + 2 * kBandCap) * 128];
  const int64_t i0 = static_cast<int64_t>(blockIdx.x) * blockDim.x;
  const int64_t i = i0 + threadIdx.x;
  if (threadIdx.x == 0) {
    s_ok = 0;
    mbar_init(&s_bar, 1);
    const int64_t ilast = min(i0 + static_cast<int64_t>(blockDim.x), A.n) - 1;
    const uint32_t k0 = A.skey[i0], k1 = A.skey[ilast];
    const uint32_t t0 = tank_of_key(k0, A.tank_off, A.ntanks);
    const uint32_t t1 = tank_of_key(k1, A.tank_off, A.ntanks);
    if (t0 == t1) {
      const TankDev& T = A.tanks[t0];
      int c0[3], c1[3];
      cell_from_key<2>(T, k0, c0);
      cell_from_key<2>(T, k1, c1);
      if (c0[1] == c1[1] && 2 * A.k + 1 <= kStageRows) {
        const int ylo = max(c0[1] - A.k, 0), yhi = min(c0[1] + A.k, T.nc[1] - 1);
        const int xlo = max(c0[0] - A.k, 0), xhi = min(c1[0] + A.k, T.nc[0] - 1);
        uint32_t off = 0;
        for (int y = ylo; y <= yhi; ++y) {
          const uint32_t row = T.cell_off + static_cast<uint32_t>(y) * T.nc[0];
          // Even record bounds: 8-byte position records start on 16 bytes.
          const uint32_t gb = __ldg(A.cell_start + 2 * (row + xlo)) & ~1u;
          const uint32_t ge = (__ldg(A.cell_start + 2 * (row + xhi + 1)) + 1u) & ~1u;
          s_gbeg[y - ylo] = gb;
          s_goff[y - ylo] = off;
          off += ge - gb;
        }
        s_goff[yhi - ylo + 1] = off;
        s_rows = yhi - ylo + 1;
        s_ylo = ylo;
        if (off > 0 && off <= static_cast<uint32_t>(kStageCap)) {
          s_ok = 1;
          mbar_arrive_expect(&s_bar, off * static_cast<uint32_t>(sizeof(float2) + 2 * sizeof(float4)));
          for (int r = 0; r < s_rows; ++r) {
            const uint32_t gb = s_gbeg[r], o = s_goff[r], len = s_goff[r + 1] - o;
            if (len == 0) continue;
            bulk_copy_g2s(s_pos + o, reinterpret_cast<const float2*>(A.posrec) + gb,
                          len * static_cast<uint32_t>(sizeof(float2)), &s_bar);
            bulk_copy_g2s(s_dat + 2 * o, reinterpret_cast<const float4*>(A.datrec) + 2 * gb,
                          len * static_cast<uint32_t>(2 * sizeof(float4)), &s_bar);
          }
        }
      }
    }
  }
  __syncthreads();
  bool staged = s_ok != 0;
  if (staged && !mbar_wait(&s_bar, 0, kCopySpins)) {
    staged = false;
    atomicOr(A.err, static_cast<uint32_t>(TG_DEV_COPY_TIMEOUT));
  }
  // Every thread keeps its answer: a late copy must not leave part of the
  // block on the staged path.
  staged = __syncthreads_and(staged) != 0;
  // Copies still in flight after a timed-out wait: a second bounded wait
  // before any thread leaves (the block's shared memory outlives them).
  if (s_ok != 0 && !staged) mbar_wait(&s_bar, 0, kCopySpins);
  if (i >= A.n) return;
  const uint32_t id = A.Y.id[i];
  if (id & kWallBit) {
    commit_wall(A, i, id);
    return;
  }
  const uint32_t key = A.skey[i];
  const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
  const TankDev& T = A.tanks[tk];
  int c[3] = {0, 0, 0};
  cell_from_key<2>(T, key, c);
  PairF32<2, K> acc;
  acc.init(A.phys, T, load_dat(A.datrec, static_cast<uint32_t>(i)), A.kahan);
  float oa[3] = {0.f, 0.f, 0.f};
  load_pos(A.posrec, static_cast<uint32_t>(i), oa);
  const float csz = T.cs_f;
  const uint32_t ia = static_cast<uint32_t>(i);
  // The band handling of k_forces (BandWalk), so that both passes visit
  // the same candidates and sum them in the same order.
  const float lo = target_band<2>(T, c, A.k).lo;
  BandWalk<2, K, kPhysGeneric> bw{A, T, acc, oa, c, csz, lo, ia};
  bw.init(s_band);
  auto exact_all = [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
    bw.exact(s, en, dx, dy, dz, false);
  };
  auto exact_band = [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
    bw.exact(s, en, dx, dy, dz, true);
  };
  if (lo < 0.f) {
    for_cells<2, true>(T, c, A.k, A.cell_start, exact_all, oa);
  } else {
    if (staged) {
      const int xlo = max(c[0] - A.k, 0), xhi = min(c[0] + A.k, T.nc[0] - 1);
      for (int r = 0; r < s_rows; ++r) {
        const int y = s_ylo + r;
        const uint32_t row = T.cell_off + static_cast<uint32_t>(y) * T.nc[0];
        const int32_t shift = static_cast<int32_t>(s_goff[r]) - static_cast<int32_t>(s_gbeg[r]);
        float oas[3];
        oas[1] = oa[1] - (y - c[1]) * csz;
        uint32_t gs = __ldg(A.cell_start + 2 * (row + xlo));
        for (int x = xlo; x <= xhi; ++x) {
          const uint32_t ge = __ldg(A.cell_start + 2 * (row + x + 1));
          oas[0] = oa[0] - (x - c[0]) * csz;
          const uint32_t code = static_cast<uint32_t>(((x - c[0] + 3) << 3) | (y - c[1] + 3));
          acc.open();
          for (uint32_t j = gs; j < ge; ++j) {
            if (j == ia) continue;
            const int sj = static_cast<int>(j) + shift;
            const float2 ob = s_pos[sj];
            float d[3] = {oas[0] - ob.x, oas[1] - ob.y, 0.f};
            const float s2 = d[0] * d[0] + d[1] * d[1];
            if (s2 >= lo) {
              if (s2 <= lo * kBandRatio) bw.defer(j, code);
              continue;
            }
            const float4 b0 = s_dat[2 * sj], b1 = s_dat[2 * sj + 1];
            acc.add(d, s2, Dat32{b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w});
          }
          acc.close();
          gs = ge;
        }
      }
    } else {
      for_cells<2, true>(T, c, A.k, A.cell_start,
                         [&](uint32_t s, uint32_t en, int dx, int dy, int) {
        float oas[3];
        oas[0] = oa[0] - dx * csz;
        oas[1] = oa[1] - dy * csz;
        const uint32_t code = static_cast<uint32_t>(((dx + 3) << 3) | (dy + 3));
        acc.open();
        for (uint32_t j = s; j < en; ++j) {
          if (j == ia) continue;
          float ob[3], d[3];
          load_pos(A.posrec, j, ob);
          d[0] = oas[0] - ob[0];
          d[1] = oas[1] - ob[1];
          d[2] = 0.f;
          const float s2 = d[0] * d[0] + d[1] * d[1];
          if (s2 >= lo) {
            if (s2 <= lo * kBandRatio) bw.defer(j, code);
            continue;
          }
          acc.add(d, s2, load_dat(A.datrec, j));
        }
        acc.close();
      });
    }
    if (!bw.decide()) for_cells<2, true>(T, c, A.k, A.cell_start, exact_band, oa);
  }
  float va[3], dv_out[3];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    va[k] = acc.va[k];
    dv_out[k] = acc.dv[k].value();
  }
  va[2] = 0.f;
  dv_out[2] = 0.f;
  forces_epilogue<2, TG_FP32C>(A, i, id, tk, T, c, va, acc.a.drho, dv_out,
                               acc.drho.value());
}

// ---------------------------------------------------------------------------
// Neighbour export: counts and order-independent hashes of the neighbour
// set (tank-local upload ids), with the same predicate as k_forces.
template<int D, int F>
__global__ void __launch_bounds__(128)
    k_neigh_count(StageArgs<D, F> A, const uint32_t* __restrict__ id_base,
                  int32_t* __restrict__ counts, uint64_t* __restrict__ hashes,
                  const int64_t* __restrict__ offsets,
                  int32_t* __restrict__ indices) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const uint32_t id = A.Y.id[i] & kIdMask;
  const uint32_t key = A.skey[i];
  const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
  const TankDev& T = A.tanks[tk];
  const uint32_t base = id_base[tk];
  int c[3] = {0, 0, 0};
  cell_from_key<D>(T, key, c);
  int32_t cnt = 0;
  uint64_t hs = 0;
  int64_t out = offsets != nullptr ? offsets[id] : 0;
  if constexpr (F == TG_FP64) {
    double pa[3] = {0.0, 0.0, 0.0};
    load_pos(A.posrec, static_cast<uint32_t>(i), pa);
    for_cells<D, false>(T, c, A.k, A.cell_start,
                        [&](uint32_t s, uint32_t en, int, int, int) {
      for (uint32_t j = s; j < en; ++j) {
        double pb[3], d[3];
        load_pos(A.posrec, j, pb);
        if (dist2_exact<D>(pb, pa, d) > T.radius2) continue;
        const uint32_t lid = (A.Y.id[j] & kIdMask) - base;
        ++cnt;
        hs += splitmix64(static_cast<uint64_t>(lid) + 1u);
        if (indices != nullptr) indices[out++] = static_cast<int32_t>(lid);
      }
    });
  } else {
    float oa[3] = {0.f, 0.f, 0.f};
    load_pos(A.posrec, static_cast<uint32_t>(i), oa);
    const float csz = T.cs_f;
    const Band bd = target_band<D>(T, c, A.k);
    const uint32_t ia = static_cast<uint32_t>(i);
    for_cells<D, true>(T, c, A.k, A.cell_start,
                       [&](uint32_t s, uint32_t en, int dx, int dy, int dz) {
      float oas[3];
      oas[0] = oa[0] - dx * csz;
      oas[1] = oa[1] - dy * csz;
      oas[2] = D == 3 ? oa[2] - dz * csz : 0.f;
      for (uint32_t j = s; j < en; ++j) {
        float ob[3], d[3];
        load_pos(A.posrec, j, ob);
#pragma unroll
        for (int k = 0; k < D; ++k) d[k] = oas[k] - ob[k];
        float s2 = d[0] * d[0] + d[1] * d[1];
        if constexpr (D == 3) s2 += d[2] * d[2];
        if (s2 > bd.hi) continue;
        if (s2 >= bd.lo && !within_fp64<D>(A.Y.pos, ia, j, T.radius2)) continue;
        const uint32_t lid = (A.Y.id[j] & kIdMask) - base;
        ++cnt;
        hs += splitmix64(static_cast<uint64_t>(lid) + 1u);
        if (indices != nullptr) indices[out++] = static_cast<int32_t>(lid);
      }
    });
  }
  if (counts != nullptr) counts[id] = cnt;
  if (hashes != nullptr) hashes[id] = hs;
}

// ---------------------------------------------------------------------------
// Summation density over a point cloud (fluid_equations.hpp:498-502 form,
// self included): rho_a = sum_b m W_ab, with neighbour counts and hashes.
// FP64 positions: FP64 predicate and sum.  FP32 positions: the positions are
// rounded to float once; predicate and kernel in FP32, compensated sum.
template<int D>
struct CloudArgs {
  const void* pos;  // Pos64_* or Pos32_* absolute positions, cell order
  const uint32_t* id;
  const uint32_t* skey;  // sorted keys
  const uint32_t* cell_start;
  const TankDev* tanks;
  const uint32_t* tank_off;
  int ntanks;
  int64_t n;
  int k;
  double* rho;       // by upload id
  int32_t* counts;   // by upload id
  uint64_t* hashes;  // by upload id
  const uint32_t* id_base;
};

template<int D, int K, bool F32>
__global__ void __launch_bounds__(128) k_sumdens(CloudArgs<D> A) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const uint32_t id = A.id[i] & kIdMask;
  const uint32_t key = A.skey[i];
  const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
  const TankDev& T = A.tanks[tk];
  const uint32_t base = A.id_base[tk];
  int c[3] = {0, 0, 0};
  cell_from_key<D>(T, key, c);
  int32_t cnt = 0;
  uint64_t hs = 0;
  double rho;
  if constexpr (!F32) {
    using P = std::conditional_t<D == 2, Pos64_2, Pos64_3>;
    const P* pr = static_cast<const P*>(A.pos);
    double pa[3] = {0.0, 0.0, 0.0};
    load_pos(pr, static_cast<uint32_t>(i), pa);
    const double R2 = T.radius2, hinv = T.hinv, wm = T.w * T.m;
    double acc = 0.0;
    // Cell clipping where the grid carries its FP32 geometry (not in the
    // allocation-free pass, whose grid leaves it unset).
    float oc[3] = {0.f, 0.f, 0.f};
    cell_offset<D>(T, c, pa, oc);
    const float* clip = T.cull_r2_f > 0.f ? oc : nullptr;
    for_cells<D, false>(T, c, A.k, A.cell_start,
                        [&](uint32_t s, uint32_t en, int, int, int) {
      for (uint32_t j = s; j < en; ++j) {
        double pb[3], d[3];
        load_pos(pr, j, pb);
        const double s2 = dist2_exact<D>(pa, pb, d);
        if (s2 > R2) continue;
        acc += wm * KernelPoly<K>::value(sqrt(s2) * hinv);
        ++cnt;
        hs += splitmix64(static_cast<uint64_t>((A.id[j] & kIdMask) - base) + 1u);
      }
    }, clip);
    rho = acc;
  } else {
    using P = std::conditional_t<D == 2, Pos32_2, Pos32_3>;
    const P* pr = static_cast<const P*>(A.pos);
    float pa[3] = {0.f, 0.f, 0.f};
    load_pos(pr, static_cast<uint32_t>(i), pa);
    const float R2 = T.radius2_f, hinv = T.hinv_f;
    const float wm = T.w_f * T.m_f;
    Kahan acc;
    double pd[3] = {pa[0], pa[1], pa[2]};
    float oc[3] = {0.f, 0.f, 0.f};
    cell_offset<D>(T, c, pd, oc);
    const float* clip = T.cull_r2_f > 0.f ? oc : nullptr;
    for_cells<D, false>(T, c, A.k, A.cell_start,
                        [&](uint32_t s, uint32_t en, int, int, int) {
      for (uint32_t j = s; j < en; ++j) {
        float pb[3], d[3];
        load_pos(pr, j, pb);
        const float s2 = dist2_exact<D>(pa, pb, d);
        if (s2 > R2) continue;
        acc.add(wm * KernelPoly<K>::value(sqrtf(s2) * hinv));
        ++cnt;
        hs += splitmix64(static_cast<uint64_t>((A.id[j] & kIdMask) - base) + 1u);
      }
    }, clip);
    rho = static_cast<double>(acc.value());
  }
  if (A.rho != nullptr) A.rho[id] = rho;
  if (A.counts != nullptr) A.counts[id] = cnt;
  if (A.hashes != nullptr) A.hashes[id] = hs;
}

// ---------------------------------------------------------------------------
// gamma and grad gamma of every particle (FluidEquations::compute_gamma,
// fluid_equations.hpp:166-193) in two passes.  k_gamma_init, per particle:
// records the cell-order slot of each fixed particle (for the face terms'
// vertex lookups) and lists the face particles, those whose cell lists
// faces; the others have grad gamma = 0, gamma = the containment answer,
// and zero face terms.  k_gamma_faces, one warp per face particle with the
// lanes splitting its faces: grad gamma = the sum of kernel fluxes, then
// gamma = contains - the sum of antigradient fluxes at r + (2 contains - 1)
// n h^2.  A fixed particle's gamma is never read (its grad gamma gives the
// wall normal), so it is set to 1 without the containment and antigradient
// sums.
template<int D, int F>
__global__ void __launch_bounds__(128) k_gamma_init(StageArgs<D, F> A) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  const FaceArgs& fc = A.fc;
  const uint32_t id = A.Y.id[i];
  const bool wall = (id & kWallBit) != 0;
  if (wall) fc.slot_of[id & kIdMask] = static_cast<uint32_t>(i);
  const uint32_t key = A.skey[i];
  const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
  const TankDev& T = A.tanks[tk];
  int c[3] = {0, 0, 0};
  cell_from_key<D>(T, key, c);
  const uint32_t gcell = global_cell<D>(T, c);
  if (fc.cell_start[gcell + 1] > fc.cell_start[gcell]) {
    fc.face_list[atomicAdd(fc.face_count, 1u)] = static_cast<uint32_t>(i);
    return;
  }
  bool inside = true;
  if (!wall) {
    double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; ++k) x[k] = A.Y.pos[k][i];
    if constexpr (D == 2) inside = face_contains(fc, tk, fc.row_off[tk] + c[1], x);
    else inside = fc.tank_edges[tk] == 0 || face_contains3(fc, tk, gcell, x, 0, 1);
  }
  fc.gamma[i] = inside ? 1.0 : 0.0;
  fc.face_drho[i] = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    fc.ggam[D * i + k] = 0.0;
    fc.face_dv[D * i + k] = 0.0;
  }
}

template<int D, int K, int F, class FT>
__global__ void __launch_bounds__(128) k_gamma_faces(StageArgs<D, F> A) {
  __shared__ uint32_t flist_all[kFaceBlock / 32][kFaceListCap];
  const FaceArgs& fc = A.fc;
  const int lane = threadIdx.x & 31;
  uint32_t* flist = flist_all[threadIdx.x >> 5];
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  const uint32_t count = *fc.face_count;
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < count; w += nwarps) {
    const uint32_t i = fc.face_list[w];
    const bool wall = (A.Y.id[i] & kWallBit) != 0;
    const uint32_t key = A.skey[i];
    const uint32_t tk = tank_of_key(key, A.tank_off, A.ntanks);
    const TankDev& T = A.tanks[tk];
    int c[3] = {0, 0, 0};
    cell_from_key<D>(T, key, c);
    const uint32_t gcell = global_cell<D>(T, c);
    double x[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < D; ++k) x[k] = A.Y.pos[k][i];
    const double radius = KernelPoly<K>::unit_radius * T.h;
    const double wd = fc.weight;
    // The in-range faces of x, found once for both sweeps (the antigradient
    // sweep at xs keeps the adjacency of x); the skip masks come from the
    // same list.  Past the list's capacity both sweeps test the cell list
    // again, as for_adjacent_faces does.
    const int nf = collect_adjacent_faces<D>(fc, gcell, x, radius, lane, flist, kFaceListCap);
    auto sweep = [&](auto&& fn) {
      if (nf <= kFaceListCap) {
        for (int base = 0; base < nf; base += 32) {
          const bool active = base + lane < nf;
          const uint32_t fi = flist[active ? base + lane : base];
          const unsigned skip = active ? face_skip_edges_listed<D>(fc, fi, flist, nf) : 0u;
          fn(active, fi, fc.coords + D * D * static_cast<size_t>(fi), skip);
        }
      } else {
        for_adjacent_faces<D>(fc, gcell, x, radius, lane,
                              [&](bool active, uint32_t fi, const double* f) {
          const unsigned skip = active ? face_skip_edges<D>(fc, fi, x, radius) : 0u;
          fn(active, fi, f, skip);
        });
      }
    };
    double g[3] = {0.0, 0.0, 0.0};
    sweep([&](bool active, uint32_t fi, const double* f, unsigned skip) {
      double fl[3];
      face_flux_d<K, D, FT>(active, f, face_axes<D>(fc, fi), x, T.h, wd, fl, skip);
      if (!active) return;
#pragma unroll
      for (int k = 0; k < D; ++k) g[k] += fl[k];
    });
#pragma unroll
    for (int k = 0; k < D; ++k) g[k] = warp_sum(g[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < D; ++k) fc.ggam[D * i + k] = g[k];
    }
    if (wall) {
      if (lane == 0) fc.gamma[i] = 1.0;
      continue;
    }
    bool inside;
    if constexpr (D == 2) inside = face_contains(fc, tk, fc.row_off[tk] + c[1], x);
    else inside = fc.tank_edges[tk] == 0 || face_contains3(fc, tk, gcell, x, lane, 32);
    double ga = inside ? 1.0 : 0.0;
    const double ng = sqrt(dot_d<D>(g, g));
    if (!(ng <= kTiny)) {
      const double s = 2.0 * ga - 1.0;
      const double h2 = T.h * T.h;
      double xs[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int k = 0; k < D; ++k) xs[k] = x[k] + s * (g[k] / ng) * h2;
      double ag = 0.0;
      sweep([&](bool active, uint32_t fi, const double* f, unsigned skip) {
        const double a =
            face_antigrad_flux_d<K, D, FT>(active, f, face_axes<D>(fc, fi), xs, T.h, wd, skip);
        if (active) ag += a;
      });
      ga -= warp_sum(ag);
    }
    if (lane == 0) fc.gamma[i] = ga;
  }
}

// ---------------------------------------------------------------------------
// Prepare-only commit: the fluid home state takes the gathered cell-order
// copy, the walls theirs from commit_wall.
template<int D, int F>
__global__ void __launch_bounds__(256) k_commit(StageArgs<D, F> A) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= A.n) return;
  const uint32_t id = A.Y.id[j];
  if (id & kWallBit) {
    commit_wall(A, j, id);
    return;
  }
#pragma unroll
  for (int k = 0; k < D; ++k) {
    A.X.pos[k][j] = A.Y.pos[k][j];
    A.X.vel[k][j] = A.Y.vel[k][j];
    A.X.dv[k][j] = A.Y.dv[k][j];
  }
  A.X.rho[j] = A.Y.rho[j];
  A.X.drho[j] = A.Y.drho[j];
  A.X.id[j] = id;
  A.X.key[j] = A.skey[j];
  A.X.pkey[j] = A.skey[j];
  if constexpr (F == TG_FP32C) {
    float o[3] = {0.f, 0.f, 0.f};
    load_pos(A.posrec, static_cast<uint32_t>(j), o);
#pragma unroll
    for (int k = 0; k < D; ++k) A.X.off[k][j] = o[k];
  }
}

// Upload: AoS doubles in upload order into the SoA home state (keys follow
// from k_keys).
template<int D, class R>
__global__ void __launch_bounds__(256)
    k_unpack(StateBuf<R> X, const double* __restrict__ r,
             const double* __restrict__ v, const double* __restrict__ rho,
             const double* __restrict__ dv, const uint32_t* __restrict__ tank_of,
             const TankDev* tanks, const uint32_t* __restrict__ wall_from,
             int64_t n) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t tk = tank_of[i];
  const bool wall = static_cast<uint32_t>(i) >= wall_from[tk];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    X.pos[k][i] = r[i * D + k];
    X.vel[k][i] = static_cast<R>(v[i * D + k]);
    X.dv[k][i] = dv != nullptr ? static_cast<R>(dv[i * D + k]) : R(0);
  }
  if constexpr (sizeof(R) == 8) {
    X.rho[i] = static_cast<R>(rho[i]);
  } else {
    X.rho[i] = static_cast<R>(rho[i] - tanks[tk].rho0);
  }
  X.drho[i] = R(0);
  X.id[i] = static_cast<uint32_t>(i) | (wall ? kWallBit : 0u);
}

// Download: one field of the home state into upload order (AoS for vectors).
template<int D, class R>
__global__ void __launch_bounds__(256)
    k_pack(StateBuf<R> X, const uint32_t* __restrict__ tank_of,
           const TankDev* tanks, PhysDev phys, int field,
           double* __restrict__ out, int64_t n) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t id = X.id[i] & kIdMask;
  const TankDev& T = tanks[tank_of[id]];
  switch (field) {
    case TG_FIELD_R:
#pragma unroll
      for (int k = 0; k < D; ++k) out[int64_t(id) * D + k] = X.pos[k][i];
      break;
    case TG_FIELD_V:
#pragma unroll
      for (int k = 0; k < D; ++k) out[int64_t(id) * D + k] = X.vel[k][i];
      break;
    case TG_FIELD_DV_DT:
#pragma unroll
      for (int k = 0; k < D; ++k) out[int64_t(id) * D + k] = X.dv[k][i];
      break;
    case TG_FIELD_DRHO_DT: out[id] = X.drho[i]; break;
    default: {
      double rho;
      if constexpr (sizeof(R) == 8) {
        rho = X.rho[i];
      } else {
        rho = T.rho0 + static_cast<double>(X.rho[i]);
      }
      if (field == TG_FIELD_RHO) {
        out[id] = rho;
      } else {
        double p, c;
        tait_f64(phys, T, rho, p, c);
        out[id] = field == TG_FIELD_P ? p : c;
      }
    }
  }
}

// Download of the whole state in one pass: r, v, dv/dt (AoS), rho and
// drho/dt into upload order; a null output is skipped.
template<int D, class R>
__global__ void __launch_bounds__(256)
    k_pack_state(StateBuf<R> X, const uint32_t* __restrict__ tank_of,
                 const TankDev* tanks, double* __restrict__ r,
                 double* __restrict__ v, double* __restrict__ rho,
                 double* __restrict__ drho, double* __restrict__ dv, int64_t n) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t id = X.id[i] & kIdMask;
  const int64_t o = static_cast<int64_t>(id) * D;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    if (r != nullptr) r[o + k] = X.pos[k][i];
    if (v != nullptr) v[o + k] = X.vel[k][i];
    if (dv != nullptr) dv[o + k] = X.dv[k][i];
  }
  if (rho != nullptr) {
    if constexpr (sizeof(R) == 8) {
      rho[id] = X.rho[i];
    } else {
      rho[id] = tanks[tank_of[id]].rho0 + static_cast<double>(X.rho[i]);
    }
  }
  if (drho != nullptr) drho[id] = X.drho[i];
}

// End of step: advance per-tank time, keep dt, reset the dt reduction.
static __global__ void k_step_end(double* dt, double* dt_last, double* time,
                                  uint32_t* err, int ntanks) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntanks) return;
  const double d = dt[t];
  if (isfinite(d)) {
    if (!(d > 0.0)) atomicOr(err, static_cast<uint32_t>(TG_DEV_BAD_DT));
    time[t] += d;
    dt_last[t] = d;
  }
  dt[t] = __longlong_as_double(0x7ff0000000000000ll);
}

// Cloud records for the summation density: absolute positions in cell order
// (FP64, or rounded once to FP32) and ids.
template<int D, bool F32>
__global__ void __launch_bounds__(256)
    k_cloud_records(const double* __restrict__ px,
                    const double* __restrict__ py,
                    const double* __restrict__ pz,
                    const uint32_t* __restrict__ id_in,
                    const uint32_t* __restrict__ perm, void* rec,
                    uint32_t* __restrict__ id_out, int64_t n) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t s = perm[j];
  const double x = px[s], y = py[s], z = D == 3 ? pz[s] : 0.0;
  if constexpr (F32) {
    if constexpr (D == 2) {
      static_cast<Pos32_2*>(rec)[j] = Pos32_2{float(x), float(y)};
    } else {
      static_cast<Pos32_3*>(rec)[j] = Pos32_3{float(x), float(y), float(z), 0.f};
    }
  } else {
    if constexpr (D == 2) {
      static_cast<Pos64_2*>(rec)[j] = Pos64_2{x, y};
    } else {
      static_cast<Pos64_3*>(rec)[j] = Pos64_3{x, y, z, 0.0};
    }
  }
  id_out[j] = id_in[s];
}

}  // namespace tg
