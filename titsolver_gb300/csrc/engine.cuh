// engine.cuh - host-side context of the C ABI and the engine interface that
// the per-(dimension, form, kernel) templates implement.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "faces.cuh"

namespace tg {

struct Context;

// Force passes per step of an integrator.
inline int force_passes(int integrator) {
  switch (integrator) {
    case TG_SSPRK2: return 2;
    case TG_EULER: return 2;
    default: return 3;  // SSPRK3, velocity Verlet
  }
}

// Kernel groups timed by the profiler.
enum Group { kGroupSort = 0, kGroupReorder, kGroupWalls, kGroupForces,
             kGroupPost, kGroupCount };

struct EngineBase {
  virtual ~EngineBase() = default;
  // Allocate the typed state for C.n particles.
  virtual cudaError_t allocate(Context& C) = 0;
  // Copy host AoS arrays (upload order) into the home state.
  // Unpack the staged host arrays (upload order: r, v, rho in d_stage,
  // d_stage2, d_stage3; dv/dt in d_stage4 when with_dv) into the home state,
  // then compute the cell keys.
  virtual cudaError_t upload_state(Context& C, const double* r, const double* v,
                                   const double* rho, const double* dv) = 0;
  // Recompute the home cell keys from the positions if they are stale.
  virtual cudaError_t ensure_keys(Context& C) = 0;
  // Enqueue one full integrator step on C.stream.
  virtual cudaError_t enqueue_step(Context& C) = 0;
  // Enqueue FluidEquations::prepare: search + wall extrapolation, leaving
  // the home state in the new cell order.
  virtual cudaError_t enqueue_prepare(Context& C) = 0;
  // Enqueue a pack of one field into the device staging buffer (upload
  // order).
  virtual cudaError_t enqueue_pack(Context& C, int field) = 0;
  // The state fields into device buffers in upload order (nulls skipped).
  virtual cudaError_t enqueue_pack_state(Context& C, double* r, double* v,
                                         double* rho, double* drho,
                                         double* dv) = 0;
  // Enqueue the neighbour export (counts/hashes by id; indices at offsets).
  virtual cudaError_t enqueue_neighbours(Context& C, int32_t* counts,
                                         uint64_t* hashes,
                                         const int64_t* offsets,
                                         int32_t* indices) = 0;
  // Enqueue search + summation density; outputs by id on the device.
  virtual cudaError_t enqueue_sumdens(Context& C, int pos_precision,
                                      double* rho, int32_t* counts,
                                      uint64_t* hashes) = 0;
  // Whether the force pass has a variant with `team` lanes per target.
  virtual bool supports_team(int team) const = 0;
};

// One engine template instance (dimension D, form F, smoothing kernel K).
// Defined in engine_impl.cuh and explicitly instantiated once per instance by
// engine_inst.cu, which the build compiles as separate objects in parallel.
template <int D, int F, int K>
std::unique_ptr<EngineBase> make_engine_instance();

// The engine of a dimension, precision form and smoothing kernel; null for an
// unknown combination.
std::unique_ptr<EngineBase> make_engine(int dim, int form, int kernel);

struct PendingEvent {
  int group;
  cudaEvent_t start, stop;
};

struct Context {
  tg_params P{};
  PhysDev phys{};
  int device = 0;
  int sm_count = 0;  // multiprocessors of the device
  cudaStream_t stream = nullptr;
  // Device-to-host copies that overlap kernels of `stream` (state download
  // with a closing prepare); created on first use.
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ready = nullptr;

  // Particles and tanks.
  int64_t n = 0, n_fluid = 0, n_wall = 0;
  int32_t ntanks = 0;
  std::vector<tg_tank> tanks;
  std::vector<TankDev> tankdev;
  std::vector<uint32_t> id_base;    // first upload index of each tank
  std::vector<uint32_t> wall_from;  // first wall upload index of each tank
  uint32_t total_cells = 0;
  uint32_t total_keys = 0;  // 2 per cell: fluid, then walls
  int key_bits = 0;
  int k = 1;
  bool uploaded = false;
  // Launch shape of the force pass (tg_set_tuning / tg_autotune).
  int force_block = 128;
  int force_team = 1;
  // Boundary faces (tg_tank_faces): host copies per tank and the device
  // view; faces.on = 0 with particle walls.
  struct TankFaces {
    std::vector<int32_t> face_verts;  // dim per face, tank-local fixed index
    std::vector<double> poly;         // 2D: 2 per containment vertex;
                                      // 3D: 9 per containment triangle
  };
  std::vector<TankFaces> face_host;
  FaceArgs faces{};
  std::vector<void*> face_allocations;

  double post_cos2_fov = 0.0;  // cos(pi/4)^2 of the visibility cone
  double post_k_fs = 0.0;      // -log(0.05) / 0.01^2
  double tuned_ms = 0.0;  // device time per step of the tuned shape
  int tuned_candidates = 0;

  // Common device buffers.
  TankDev* d_tanks = nullptr;
  uint32_t* d_tank_off = nullptr;  // first key of each tank
  uint32_t* d_id_base = nullptr;
  uint32_t* d_wall_from = nullptr;
  uint32_t* d_tank_of = nullptr;  // tank of each upload index
  double* d_dt = nullptr;
  double* d_dt_last = nullptr;
  double* d_time = nullptr;
  uint32_t* d_err = nullptr;
  uint32_t* d_wall_count = nullptr;  // [0] walls listed, [1] walls near fluid
  // Per tank: order-preserving encodings of the fluid bounding box of the
  // current stage (FP32, rounded outwards), mins [ntanks x 3] then maxes.
  unsigned* d_fbox = nullptr;
  uint32_t* keys_a = nullptr;
  uint32_t* keys_b = nullptr;
  uint32_t* vals_a = nullptr;
  uint32_t* vals_b = nullptr;
  void* sort_scratch = nullptr;
  uint32_t* cell_start = nullptr;
  void* cell_scratch = nullptr;
  uint32_t* wall_list = nullptr;
  void* near_scratch = nullptr;  // the re-sort's buffers (near_sort)
  uint32_t* wall_active = nullptr;  // walls near fluid this stage (k_wall_select)
  double* d_stage = nullptr;  // n * dim doubles: upload / download staging
  double* d_stage2 = nullptr;
  double* d_stage3 = nullptr;
  double* d_stage4 = nullptr;
  cudaEvent_t timer_ev[2] = {nullptr, nullptr};
  // Summation-density outputs (by id) and records.
  double* d_sd_rho = nullptr;
  int32_t* d_sd_count = nullptr;
  uint64_t* d_sd_hash = nullptr;
  void* d_cloud_rec = nullptr;

  std::vector<void*> allocations;  // everything above and the engine's
  std::unique_ptr<EngineBase> engine;

  // Results of the last sort (set by the engine while enqueueing).
  const uint32_t* sorted_keys = nullptr;
  const uint32_t* perm = nullptr;

  // CUDA graph of one step.
  bool use_graph = true;
  cudaGraphExec_t graph_exec = nullptr;
  int64_t graph_kernels = 0;

  bool walls_fresh = false;
  bool keys_valid = false;  // home keys match the home positions
  bool order_valid = false; // home state in the order of its last sort (pkey)
  bool graph_order = false; // order_valid when the step graph was captured

  // Profiling.
  bool profile = false;
  tg_profile prof{};
  std::vector<PendingEvent> pending;
  std::vector<cudaEvent_t> event_pool;

  int64_t launches = 0;
  std::string last_error;

  cudaError_t alloc(void** p, size_t bytes);
  void release_all();
  void invalidate_graph();

  // Profiling helpers (no-ops unless profile is on and not capturing).
  int group_begin(int group);
  void group_end(int token);
  void drain_profile();
};

}  // namespace tg
