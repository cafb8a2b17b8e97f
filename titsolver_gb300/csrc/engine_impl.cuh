// engine_impl.cuh - the typed engine: buffer layout and kernel sequencing of
// one step for a (dimension, arithmetic form, smoothing kernel) triple.
#pragma once

#include <memory>

#include "engine.cuh"
#include "fluid.cuh"
#include "post.cuh"
#include "sort.cuh"

namespace tg {

inline unsigned grid_for(int64_t n, int block) {
  return static_cast<unsigned>((n + block - 1) / block);
}

// Compile-time physics preset of the compensated force kernel for params.
inline int physics_preset(const tg_params& P) {
  if (!P.kahan) return kPhysGeneric;
  if (P.viscosity == TG_VISC_MONAGHAN && P.diffusion == TG_DIFF_MOLTENI) {
    return kPhysTextbook;
  }
  if (P.viscosity == TG_VISC_MORRIS && P.diffusion == TG_DIFF_FERRARI) {
    return kPhysReference;
  }
  return kPhysGeneric;
}

// Kernels with multi-lane force variants: the two the shipped parameter
// sets use (Wendland C2 and C4); the others run one lane per target.
constexpr bool team_kernel(int K) {
  return K == TG_KERNEL_WENDLAND_C2 || K == TG_KERNEL_WENDLAND_C4;
}

template<int D, int F, int K>
class Engine final : public EngineBase {
 public:
  using L = Layout<D, F>;
  using R = typename L::R;
  using PosRec = typename L::PosRec;
  using DatRec = typename L::DatRec;

  cudaError_t allocate(Context& C) override {
    const int64_t n = C.n > 0 ? C.n : 1;
    cudaError_t e = cudaSuccess;
    auto A = [&](auto*& p, int64_t count) {
      if (e == cudaSuccess) {
        e = C.alloc(reinterpret_cast<void**>(&p),
                    static_cast<size_t>(count) * sizeof(*p));
      }
    };
    for (StateBuf<R>* S : {&X_, &Y_}) {
      *S = StateBuf<R>{};
      for (int k = 0; k < D; ++k) {
        A(S->pos[k], n);
        A(S->vel[k], n);
        A(S->dv[k], n);
      }
      A(S->rho, n);
      A(S->drho, n);
      A(S->id, n);
    }
    // The home keys live in the sort's first key buffer.
    X_.key = C.keys_a;
    A(X_.pkey, n);
    if constexpr (F == TG_FP32C) {
      for (int k = 0; k < D; ++k) A(X_.off[k], n);
    }
    for (StartBuf<R>& U : U_) {
      U = StartBuf<R>{};
      for (int k = 0; k < D; ++k) {
        A(U.pos[k], n);
        A(U.vel[k], n);
      }
      A(U.rho, n);
    }
    // Two spare records: the staged force pass copies row segments rounded
    // out to 16-byte boundaries, which may reach one record past the end.
    A(posrec_, n + 2);
    A(datrec_, n + 2);
    post_ = PostArgs<D, F>{};
    if (C.P.post_integrate == TG_POST_SHIFTING) {
      A(post_.N, n * D);
      A(post_.dr, n * D);
      A(post_.gv, n * D * D);
      A(post_.grho, n * D);
      A(post_.count, n);
      A(post_.phi, n);
      A(post_.phi2, n);
      A(post_.rho_raw, n);
    }
    return e;
  }

  cudaError_t upload_state(Context& C, const double* r, const double* v,
                           const double* rho, const double* dv) override {
    if (C.n == 0) return cudaSuccess;
    k_unpack<D, R><<<grid_for(C.n, 256), 256, 0, C.stream>>>(
        X_, r, v, rho, dv, C.d_tank_of, C.d_tanks, C.d_wall_from, C.n);
    C.launches += 1;
    C.keys_valid = false;
    C.order_valid = false;  // the home order is the upload order
    return ensure_keys(C);
  }

  cudaError_t ensure_keys(Context& C) override {
    if (C.keys_valid || C.n == 0) return cudaSuccess;
    k_keys<D, F><<<grid_for(C.n, 256), 256, 0, C.stream>>>(
        X_, C.d_tank_of, C.d_tanks, C.n, C.d_err);
    C.launches += 1;
    C.keys_valid = true;
    return cudaGetLastError();
  }

  cudaError_t enqueue_step(Context& C) override {
    if (C.n == 0) return cudaSuccess;
    static const double w3[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0};
    static const double w2[2] = {1.0, 1.0 / 2.0};
    const int integ = C.P.integrator;
    if (integ == TG_SSPRK2 || integ == TG_SSPRK3) {
      // SSPRKIntegrator::step (time_integrator.hpp:161-185): every stage a
      // prepare (search + walls) and both sums, then the lincomb.
      const bool rk2 = integ == TG_SSPRK2;
      const double* w = rk2 ? w2 : w3;
      for (int s = 0; s < (rk2 ? 2 : 3); ++s) {
        Pass p;
        p.stage = s;
        p.w = w[s];
        cudaError_t e = enqueue_stage(C, p);
        if (e != cudaSuccess) return e;
      }
    } else if (integ == TG_EULER) {
      // SymplecticEulerIntegrator::step (:50-69): prepare, dt, continuity
      // and rho update, then momentum on the new rho (walls as prepared)
      // with v += dt dv, r += dt v.
      Pass a;
      a.mode = kPassContinuity;
      a.carry = 1;
      Pass b = a;
      b.stage = 1;
      b.mode = kPassKickDrift;
      b.walls_keep = 1;
      b.lincomb = 0;
      cudaError_t e = enqueue_stage(C, a);
      if (e == cudaSuccess) e = enqueue_stage(C, b);
      if (e != cudaSuccess) return e;
    } else {
      // VelocityVerletIntegrator::step (:99-123): prepare, dt, momentum with
      // v += dt/2 dv, r += dt v; prepare, continuity and rho update;
      // momentum on the new rho with v += dt/2 dv.
      Pass a;
      a.mode = kPassHalfKickDrift;
      a.carry = 1;
      Pass b = a;
      b.stage = 1;
      b.mode = kPassContinuity;
      b.lincomb = 0;
      Pass c = b;
      c.mode = kPassHalfKick;
      c.walls_keep = 1;
      cudaError_t e = enqueue_stage(C, a);
      if (e == cudaSuccess) e = enqueue_stage(C, b);
      if (e == cudaSuccess) e = enqueue_stage(C, c);
      if (e != cudaSuccess) return e;
    }
    if (C.P.post_integrate == TG_POST_SHIFTING) {
      cudaError_t e = enqueue_post(C);
      if (e != cudaSuccess) return e;
    }
    const int tok = C.group_begin(kGroupForces);
    k_step_end<<<grid_for(C.ntanks, 128), 128, 0, C.stream>>>(
        C.d_dt, C.d_dt_last, C.d_time, C.d_err, C.ntanks);
    C.launches += 1;
    C.group_end(tok);
    return cudaGetLastError();
  }

  cudaError_t enqueue_prepare(Context& C) override {
    if (C.n == 0) return cudaSuccess;
    cudaError_t e = enqueue_sort(C);
    if (e != cudaSuccess) return e;
    StageArgs<D, F> a = args(C, 0);
    a.compute_dt = 0;
    a.carry = 1;
    int tok = C.group_begin(kGroupReorder);
    e = reorder(C, a);
    C.group_end(tok);
    if (e != cudaSuccess) return e;
    tok = C.group_begin(kGroupWalls);
    if (C.n_wall > 0) {
      enqueue_gamma(C, a);
      launch_walls(C, a);
    }
    k_commit<D, F><<<grid_for(C.n, 256), 256, 0, C.stream>>>(a);
    C.launches += 1;
    C.group_end(tok);
    C.keys_valid = true;
    C.order_valid = true;
    return cudaGetLastError();
  }

  cudaError_t enqueue_pack(Context& C, int field) override {
    if (C.n == 0) return cudaSuccess;
    k_pack<D, R><<<grid_for(C.n, 256), 256, 0, C.stream>>>(
        X_, C.d_tank_of, C.d_tanks, C.phys, field, C.d_stage, C.n);
    C.launches += 1;
    return cudaGetLastError();
  }

  cudaError_t enqueue_pack_state(Context& C, double* r, double* v, double* rho,
                                 double* drho, double* dv) override {
    if (C.n == 0) return cudaSuccess;
    k_pack_state<D, R><<<grid_for(C.n, 256), 256, 0, C.stream>>>(
        X_, C.d_tank_of, C.d_tanks, r, v, rho, drho, dv, C.n);
    C.launches += 1;
    return cudaGetLastError();
  }

  cudaError_t enqueue_neighbours(Context& C, int32_t* counts,
                                 uint64_t* hashes, const int64_t* offsets,
                                 int32_t* indices) override {
    if (C.n == 0) return cudaSuccess;
    cudaError_t e = enqueue_sort(C);
    if (e != cudaSuccess) return e;
    StageArgs<D, F> a = args(C, 0);
    a.compute_dt = 0;
    e = reorder(C, a);
    if (e != cudaSuccess) return e;
    k_neigh_count<D, F><<<grid_for(C.n, 128), 128, 0, C.stream>>>(
        a, C.d_id_base, counts, hashes, offsets, indices);
    C.launches += 1;
    // The sort used the home keys as scratch and nothing rewrote them.
    C.keys_valid = false;
    return cudaGetLastError();
  }

  cudaError_t enqueue_sumdens(Context& C, int pos_precision, double* rho,
                              int32_t* counts, uint64_t* hashes) override {
    if (C.n == 0) return cudaSuccess;
    cudaError_t e = enqueue_sort(C);
    if (e != cudaSuccess) return e;
    const bool f32 = pos_precision == TG_POS_FP32;
    int tok = C.group_begin(kGroupReorder);
    if (f32) {
      k_cloud_records<D, true><<<grid_for(C.n, 256), 256, 0, C.stream>>>(
          X_.pos[0], X_.pos[1], X_.pos[2], X_.id, C.perm, C.d_cloud_rec,
          Y_.id, C.n);
    } else {
      k_cloud_records<D, false><<<grid_for(C.n, 256), 256, 0, C.stream>>>(
          X_.pos[0], X_.pos[1], X_.pos[2], X_.id, C.perm, C.d_cloud_rec,
          Y_.id, C.n);
    }
    C.launches += 1;
    C.group_end(tok);
    CloudArgs<D> ca{C.d_cloud_rec, Y_.id, C.sorted_keys, C.cell_start,
                    C.d_tanks,     C.d_tank_off, C.ntanks, C.n,
                    C.k,           rho,   counts, hashes,  C.d_id_base};
    tok = C.group_begin(kGroupForces);
    if (f32) {
      k_sumdens<D, K, true><<<grid_for(C.n, 128), 128, 0, C.stream>>>(ca);
    } else {
      k_sumdens<D, K, false><<<grid_for(C.n, 128), 128, 0, C.stream>>>(ca);
    }
    C.launches += 1;
    C.group_end(tok);
    C.keys_valid = false;
    return cudaGetLastError();
  }

  bool supports_team(int team) const override {
    return team == 1 || (team_kernel(K) && (team == 2 || team == 4));
  }

 private:
  StageArgs<D, F> args(Context& C, int stage) {
    StageArgs<D, F> a{};
    a.X = X_;
    a.Y = Y_;
    a.Usrc = U_[(stage + 1) % 2];
    a.Udst = U_[stage % 2];
    a.perm = C.perm;
    a.skey = C.sorted_keys;
    a.posrec = posrec_;
    a.datrec = datrec_;
    a.cell_start = C.cell_start;
    a.tanks = C.d_tanks;
    a.tank_off = C.d_tank_off;
    a.ntanks = C.ntanks;
    a.phys = C.phys;
    a.dt = C.d_dt;
    a.wall_list = C.wall_list;
    a.wall_count = C.d_wall_count;
    a.wall_active = C.wall_active;
    // The wall pass's fluid-box early-out pays when walls are a sizeable
    // share of the particles (it costs a fold in every reorder).
    a.fbox = C.n_wall > 0 && 4 * C.n_wall >= C.n_fluid ? C.d_fbox : nullptr;
    a.fc = C.faces;
    a.err = C.d_err;
    a.n = C.n;
    a.k = C.k;
    a.copy_start = stage == 0 ? 1 : 0;
    a.compute_dt = stage == 0 ? 1 : 0;
    a.lincomb = stage == 0 ? 0 : 1;
    a.w_new = 1.0;
    a.kahan = C.P.kahan;
    a.carry = 0;
    a.mode = kPassRK;
    a.walls_keep = 0;
    return a;
  }

  cudaError_t reorder(Context& C, const StageArgs<D, F>& a) {
    cudaError_t e = cudaMemsetAsync(C.d_wall_count, 0, 2 * sizeof(uint32_t), C.stream);
    if (e != cudaSuccess) return e;
    if (a.fbox != nullptr) {
      // Empty fluid boxes: mins at the top encoding, maxes at the bottom.
      const size_t half = sizeof(unsigned) * 3 * C.ntanks;
      e = cudaMemsetAsync(C.d_fbox, 0xff, half, C.stream);
      if (e == cudaSuccess) {
        e = cudaMemsetAsync(C.d_fbox + 3 * C.ntanks, 0, half, C.stream);
      }
      if (e != cudaSuccess) return e;
    }
    k_reorder<D, F><<<grid_for(C.n, 256), 256, 0, C.stream>>>(a);
    C.launches += 1;
    return cudaGetLastError();
  }

  // Sort the home keys (valid on entry) into cell order and build the cell
  // table.  When the home state is in the order of an earlier sort (every
  // pass over all particles writes it so, with that sort's keys in pkey),
  // the re-sort moves only the particles whose key changed; otherwise the
  // full radix sort runs, with the home key buffer as scratch.  Both give
  // the same order.
  cudaError_t enqueue_sort(Context& C) {
    cudaError_t e = ensure_keys(C);
    if (e != cudaSuccess) return e;
    const int tok = C.group_begin(kGroupSort);
    if (C.order_valid && C.P.resort != 0) {
      e = near_sort(C.keys_a, X_.pkey, C.n, C.key_bits, C.keys_b, C.vals_b,
                    C.near_scratch, C.stream, &C.launches);
      if (e != cudaSuccess) return e;
      C.sorted_keys = C.keys_b;
      C.perm = C.vals_b;
    } else {
      bool in_b = false;
      e = radix_sort(C.keys_a, C.vals_a, C.keys_b, C.vals_b, C.n, C.key_bits,
                     true, C.sort_scratch, &in_b, C.stream, &C.launches);
      if (e != cudaSuccess) return e;
      C.sorted_keys = in_b ? C.keys_b : C.keys_a;
      C.perm = in_b ? C.vals_b : C.vals_a;
    }
    e = build_cell_table_fill(C.sorted_keys, C.n, C.total_keys, C.cell_start,
                              C.cell_scratch, C.sm_count, C.stream, &C.launches);
    C.group_end(tok);
    return e;
  }

  // FluidEquations::post_integrate with shifting (fluid_equations.hpp:
  // 315-512): a prepare (sort, reorder carrying every field, wall
  // extrapolation), then the five post kernels, which leave the shifted and
  // corrected state and its keys in the home buffers.
  cudaError_t enqueue_post(Context& C) {
    cudaError_t e = enqueue_sort(C);
    if (e != cudaSuccess) return e;
    StageArgs<D, F> a = args(C, 0);
    a.compute_dt = 0;
    a.copy_start = 0;
    a.carry = 1;
    int tok = C.group_begin(kGroupPost);
    e = reorder(C, a);
    if (e != cudaSuccess) return e;
    if (C.n_wall > 0) {
      enqueue_gamma(C, a);
      launch_walls(C, a);
    }
    PostArgs<D, F> p = post_;
    p.S = a;
    p.cos2_fov = C.post_cos2_fov;
    p.k_fs = C.post_k_fs;
    p.shift = -C.P.cfl * 0.2;
    const unsigned grid = grid_for(C.n, 128);
    if (C.faces.on) {
      with_face_real(C, [&](auto real) {
        k_post_faces<D, F, K, decltype(real)><<<face_grid(C), 128, 0, C.stream>>>(p);
      });
      C.launches += 1;
    }
    k_post_sums<D, F, K><<<grid, 128, 0, C.stream>>>(p);
    k_post_phi<D, F><<<grid, 128, 0, C.stream>>>(p);
    k_post_near<D, F, K><<<grid, 128, 0, C.stream>>>(p);
    k_post_shift<D, F><<<grid, 128, 0, C.stream>>>(p);
    k_post_fs<D, F, K><<<grid, 128, 0, C.stream>>>(p);
    C.launches += 5;
    C.group_end(tok);
    C.keys_valid = true;
    C.order_valid = true;
    return cudaGetLastError();
  }

  // Face boundaries: gamma and grad gamma of every particle at the positions
  // of this prepare (before the wall pass, which reads grad gamma).
  void enqueue_gamma(Context& C, const StageArgs<D, F>& a) {
    if (a.fc.on) {
      cudaMemsetAsync(a.fc.face_count, 0, sizeof(uint32_t), C.stream);
      k_gamma_init<D, F><<<grid_for(C.n, 128), 128, 0, C.stream>>>(a);
      with_face_real(C, [&](auto real) {
        k_gamma_faces<D, K, F, decltype(real)><<<face_grid(C), 128, 0, C.stream>>>(a);
      });
      C.launches += 2;
    }
  }

  // Calls fn(float{}) when the face passes evaluate their closed-form
  // integrals in FP32 (tg_params.face_fp32, compensated form only), else
  // fn(double{}); the plain form never instantiates the FP32 passes.
  template<class Fn>
  static void with_face_real(const Context& C, Fn&& fn) {
    if constexpr (F == TG_FP32C) {
      if (C.P.face_fp32 != 0) {
        fn(0.0f);
        return;
      }
    }
    fn(0.0);
  }

  // Grid of the warp-per-face-particle passes: they loop over the face
  // list (its length is known on the device only), four warps per block.
  static unsigned face_grid(const Context& C) {
    const int64_t cap = 32 * static_cast<int64_t>(C.sm_count > 0 ? C.sm_count : 152);
    return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((C.n + 3) / 4, cap)));
  }

  // One force pass of a step: its index (stage 0 copies the start state
  // and reduces dt), lincomb weight, update rule, whether Y carries every
  // field, and whether the walls keep their carried densities.
  struct Pass {
    int stage = 0;
    double w = 1.0;
    int mode = kPassRK;
    int carry = 0;
    int walls_keep = 0;
    int lincomb = -1;  // -1: the SSPRK rule (stages after the first)
  };

  cudaError_t enqueue_stage(Context& C, const Pass& p) {
    cudaError_t e = enqueue_sort(C);
    if (e != cudaSuccess) return e;
    StageArgs<D, F> a = args(C, p.stage);
    a.w_new = p.w;
    a.mode = p.mode;
    a.carry = p.carry;
    a.walls_keep = p.walls_keep;
    if (p.lincomb >= 0) a.lincomb = p.lincomb;
    int tok = C.group_begin(kGroupReorder);
    e = reorder(C, a);
    C.group_end(tok);
    if (e != cudaSuccess) return e;
    if (C.n_wall > 0) {
      tok = C.group_begin(kGroupWalls);
      enqueue_gamma(C, a);
      launch_walls(C, a);
      C.group_end(tok);
    }
    if (a.fc.on) {
      with_face_real(C, [&](auto real) {
        k_face_terms<D, K, F, decltype(real)><<<face_grid(C), 128, 0, C.stream>>>(a);
      });
      C.launches += 1;
    }
    tok = C.group_begin(kGroupForces);
    if constexpr (F == TG_FP32C) {
      const int phys = physics_preset(C.P);
      bool staged = false;
      if constexpr (D == 2) {
        // The staged kernel has no face terms.
        if (C.P.staging && !a.fc.on) {
          k_forces_staged2<K><<<grid_for(C.n, 128), 128, 0, C.stream>>>(a);
          staged = true;
        }
      }
      if (staged) {
      } else if (phys == kPhysTextbook) {
        launch_forces<kPhysTextbook>(C, a);
      } else if (phys == kPhysReference) {
        launch_forces<kPhysReference>(C, a);
      } else {
        launch_forces<kPhysGeneric>(C, a);
      }
    } else {
      launch_forces<kPhysGeneric>(C, a);
    }
    C.launches += 1;
    C.group_end(tok);
    // k_forces wrote the keys of the new positions, in this sort's order.
    C.keys_valid = true;
    C.order_valid = true;
    return cudaGetLastError();
  }

  // The force pass at the context's launch shape: C.force_team lanes per
  // target (team variants exist for the Wendland C2 and C4 kernels) in
  // blocks of C.force_block threads.
  template<int Phys>
  void launch_forces(Context& C, const StageArgs<D, F>& a) {
    const int block = C.force_block;
    // The compensated form's band lists (1 + 2 kBandCap words per thread).
    const size_t smem =
        F == TG_FP32C ? sizeof(uint32_t) * (1 + 2 * kBandCap) * static_cast<size_t>(block) : 0;
    if constexpr (team_kernel(K)) {
      if (C.force_team == 4) {
        k_forces<D, F, K, Phys, 4><<<grid_for(C.n * 4, block), block, smem, C.stream>>>(a);
        return;
      }
      if (C.force_team == 2) {
        k_forces<D, F, K, Phys, 2><<<grid_for(C.n * 2, block), block, smem, C.stream>>>(a);
        return;
      }
    }
    k_forces<D, F, K, Phys, 1><<<grid_for(C.n, block), block, smem, C.stream>>>(a);
  }

  // The wall pass: the walls near fluid listed first (when the pass has a
  // fluid box), then teams of wall_team lanes over the list, at most 16
  // blocks per multiprocessor taking walls in turn.
  void launch_walls(Context& C, const StageArgs<D, F>& a) {
    if (a.fbox != nullptr) {
      k_wall_select<D, F><<<grid_for(C.n_wall, 256), 256, 0, C.stream>>>(a, C.n_wall);
      C.launches += 1;
    }
    const int64_t cap = 16 * static_cast<int64_t>(C.sm_count > 0 ? C.sm_count : 152);
    const unsigned grid = static_cast<unsigned>(
        std::max<int64_t>(1, std::min<int64_t>(grid_for(C.n_wall * wall_team<D, F>(), 128), cap)));
    k_walls<D, F, K><<<grid, 128, 0, C.stream>>>(a);
    C.launches += 1;
  }

  StateBuf<R> X_{}, Y_{};
  StartBuf<R> U_[2]{};
  PostArgs<D, F> post_{};
  PosRec* posrec_ = nullptr;
  DatRec* datrec_ = nullptr;
};

template <int D, int F, int K>
std::unique_ptr<EngineBase> make_engine_instance() {
  return std::make_unique<Engine<D, F, K>>();
}

}  // namespace tg
