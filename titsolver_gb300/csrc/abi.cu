// abi.cu - the C ABI of include/titgpu.h over the typed engines.
//
// Host responsibilities: argument validation (the reference asserts in Debug
// builds and throws tit::Exception from TIT_ENSURE; here every failure is a
// status code with a message in tg_last_error), the per-tank cell grids,
// device allocation, CUDA-graph capture of one step, and profiling.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <map>
#include <string>
#include <vector>

#include "engine.cuh"
#include "sort.cuh"

// The layout the Python and C++ bindings mirror: 13 int32 fields, padding,
// then the doubles.
static_assert(offsetof(tg_params, xi) == 56 && sizeof(tg_params) == 120,
              "tg_params layout changed: update the bindings");

struct tg_context {
  tg::Context c;
};

namespace tg {

cudaError_t Context::alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) allocations.push_back(*p);
  return e;
}

void Context::release_all() {
  invalidate_graph();
  for (void* p : allocations) cudaFree(p);
  allocations.clear();
  d_tanks = nullptr;
  d_tank_off = nullptr;
  d_id_base = d_wall_from = d_tank_of = nullptr;
  d_dt = d_dt_last = d_time = nullptr;
  d_err = d_wall_count = nullptr;
  d_fbox = nullptr;
  faces = FaceArgs{};
  keys_a = keys_b = vals_a = vals_b = nullptr;
  sort_scratch = nullptr;
  cell_start = wall_list = wall_active = nullptr;
  near_scratch = nullptr;
  order_valid = false;
  cell_scratch = nullptr;
  d_stage = d_stage2 = d_stage3 = d_stage4 = nullptr;
  d_sd_rho = nullptr;
  d_sd_count = nullptr;
  d_sd_hash = nullptr;
  d_cloud_rec = nullptr;
  uploaded = false;
  keys_valid = false;
}

void Context::invalidate_graph() {
  if (graph_exec != nullptr) {
    cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
  }
}

int Context::group_begin(int group) {
  if (!profile) return -1;
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(stream, &st);
  if (st != cudaStreamCaptureStatusNone) return -1;
  PendingEvent pe{group, nullptr, nullptr};
  for (cudaEvent_t* ev : {&pe.start, &pe.stop}) {
    if (!event_pool.empty()) {
      *ev = event_pool.back();
      event_pool.pop_back();
    } else {
      cudaEventCreate(ev);
    }
  }
  cudaEventRecord(pe.start, stream);
  pending.push_back(pe);
  return static_cast<int>(pending.size()) - 1;
}

void Context::group_end(int token) {
  if (token < 0) return;
  cudaEventRecord(pending[static_cast<size_t>(token)].stop, stream);
}

void Context::drain_profile() {
  if (pending.empty()) return;
  cudaStreamSynchronize(stream);
  for (const PendingEvent& pe : pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, pe.start, pe.stop);
    switch (pe.group) {
      case kGroupSort: prof.sort_ms += ms; break;
      case kGroupReorder: prof.reorder_ms += ms; break;
      case kGroupWalls: prof.walls_ms += ms; break;
      case kGroupForces: prof.forces_ms += ms; break;
      default: prof.post_ms += ms; break;
    }
    event_pool.push_back(pe.start);
    event_pool.push_back(pe.stop);
  }
  pending.clear();
}

namespace {

template <int D, int F>
std::unique_ptr<EngineBase> engine_for_kernel(int kernel) {
  switch (kernel) {
    case TG_KERNEL_CUBIC_SPLINE:
      return make_engine_instance<D, F, TG_KERNEL_CUBIC_SPLINE>();
    case TG_KERNEL_QUARTIC_SPLINE:
      return make_engine_instance<D, F, TG_KERNEL_QUARTIC_SPLINE>();
    case TG_KERNEL_QUINTIC_SPLINE:
      return make_engine_instance<D, F, TG_KERNEL_QUINTIC_SPLINE>();
    case TG_KERNEL_WENDLAND_C2:
      return make_engine_instance<D, F, TG_KERNEL_WENDLAND_C2>();
    case TG_KERNEL_WENDLAND_C4:
      return make_engine_instance<D, F, TG_KERNEL_WENDLAND_C4>();
    case TG_KERNEL_WENDLAND_C6:
      return make_engine_instance<D, F, TG_KERNEL_WENDLAND_C6>();
    default: return nullptr;
  }
}

}  // namespace

std::unique_ptr<EngineBase> make_engine(int dim, int form, int kernel) {
  if (form != TG_FP64 && form != TG_FP32C) return nullptr;
  const bool f64 = form == TG_FP64;
  if (dim == 2) {
    return f64 ? engine_for_kernel<2, TG_FP64>(kernel)
               : engine_for_kernel<2, TG_FP32C>(kernel);
  }
  if (dim == 3) {
    return f64 ? engine_for_kernel<3, TG_FP64>(kernel)
               : engine_for_kernel<3, TG_FP32C>(kernel);
  }
  return nullptr;
}

}  // namespace tg

namespace {

using tg::Context;

int fail(Context* C, int status, const std::string& msg) {
  if (C != nullptr) C->last_error = msg;
  return status;
}

int cuda_fail(Context* C, cudaError_t e, const char* where) {
  std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) {
    return fail(C, TG_ERR_OUT_OF_MEMORY, msg);
  }
  return fail(C, TG_ERR_CUDA, msg);
}

#define TG_CUDA(C, call)                                   \
  do {                                                     \
    const cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail((C), e_, #call); \
  } while (0)

int upload_particles(tg_context* ctx, int32_t n_tanks, const tg_tank* tanks,
                     const double* r, const double* v, const double* rho);
int build_faces(tg_context* ctx);

bool valid_params(const tg_params* P, std::string* why) {
  if (P->dim != 2 && P->dim != 3) {
    *why = "dim must be 2 or 3";
    return false;
  }
  if (P->precision != TG_FP64 && P->precision != TG_FP32C) {
    *why = "precision must be TG_FP64 or TG_FP32C";
    return false;
  }
  if (P->kernel < 0 || P->kernel > 5) {
    *why = "unknown kernel";
    return false;
  }
  if (P->integrator < TG_SSPRK3 || P->integrator > TG_VERLET) {
    *why = "unknown integrator";
    return false;
  }
  if (P->viscosity != TG_VISC_MORRIS && P->viscosity != TG_VISC_MONAGHAN) {
    *why = "unknown viscosity model";
    return false;
  }
  if (P->diffusion < 0 || P->diffusion > 2) {
    *why = "unknown diffusion model";
    return false;
  }
  if (P->eos != TG_EOS_TAIT && P->eos != TG_EOS_LINEAR_TAIT) {
    *why = "unknown equation of state";
    return false;
  }
  if (P->resort != 0 && P->resort != 1) {
    *why = "resort must be 0 or 1";
    return false;
  }
  if (P->face_fp32 != 0 && !(P->face_fp32 == 1 && P->precision == TG_FP32C)) {
    *why = "face_fp32 must be 0, or 1 with the FP32C form";
    return false;
  }
  if (P->post_integrate != TG_POST_PREPARE &&
      P->post_integrate != TG_POST_SHIFTING) {
    *why = "unknown post_integrate mode";
    return false;
  }
  if (P->cells_per_radius < 1 || P->cells_per_radius > 3) {
    *why = "cells_per_radius must be 1, 2 or 3";
    return false;
  }
  if (!(P->xi > 1.0) || !(P->g >= 0.0) || !(P->mu >= 0.0) ||
      !(P->alpha >= 0.0) || !(P->delta >= 0.0) || !(P->cfl > 0.0) ||
      !(P->c_force > 0.0) || !(P->c_visc > 0.0)) {
    *why = "physical constants out of range";
    return false;
  }
  return true;
}

double kernel_weight(int k, int dim) {
  const double pi = 3.14159265358979323846;
  const double area = 2.0 * std::sqrt(std::pow(pi, dim)) / std::tgamma(dim / 2.0);
  return 1.0 / (tg::kernel_zero_moment(k, dim) * area);
}

// The device view of a page-locked (cudaMallocHost / cudaHostAlloc /
// registered) host array, or nullptr for other memory.
const double* mapped_host(const double* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
  return static_cast<const double*>(a.devicePointer);
}

int key_bits_for(uint32_t total_cells) {
  int bits = 1;
  while (bits < 32 && (static_cast<uint64_t>(1) << bits) < total_cells) ++bits;
  return bits;
}

}  // namespace

extern "C" {

void tg_params_default(tg_params* p) {
  if (p == nullptr) return;
  std::memset(p, 0, sizeof(*p));
  p->dim = 2;
  p->precision = TG_FP64;
  p->kernel = TG_KERNEL_WENDLAND_C4;
  p->integrator = TG_SSPRK3;
  p->viscosity = TG_VISC_MORRIS;
  p->diffusion = TG_DIFF_FERRARI;
  p->post_integrate = TG_POST_SHIFTING;
  p->cells_per_radius = 2;
  p->kahan = 1;
  p->device = -1;
  p->staging = 0;
  p->resort = 1;
  p->xi = 7.0;
  p->g = 9.81;
  p->mu = 0.001;
  p->alpha = 0.02;
  p->delta = 0.1;
  p->cfl = 0.4;
  p->c_force = 0.25;
  p->c_visc = 0.125;
}

const char* tg_status_string(int status) {
  switch (status) {
    case TG_OK: return "ok";
    case TG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TG_ERR_CUDA: return "CUDA error";
    case TG_ERR_OUT_OF_MEMORY: return "out of device memory";
    case TG_ERR_NOT_READY: return "no particles uploaded";
    case TG_ERR_DEVICE_STATE: return "device error word raised";
    case TG_ERR_CAPACITY: return "output capacity too small";
    case TG_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* tg_last_error(tg_context* ctx) {
  return ctx == nullptr ? "null context" : ctx->c.last_error.c_str();
}

int tg_context_create(const tg_params* params, tg_context** out) {
  if (out == nullptr || params == nullptr) return TG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  std::string why;
  if (!valid_params(params, &why)) return TG_ERR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return TG_ERR_NO_DEVICE;
  }
  if (params->device >= ndev) return TG_ERR_INVALID_ARGUMENT;
  if (params->device >= 0 && cudaSetDevice(params->device) != cudaSuccess) {
    cudaGetLastError();
    return TG_ERR_CUDA;
  }
  tg_context* ctx = new (std::nothrow) tg_context();
  if (ctx == nullptr) return TG_ERR_OUT_OF_MEMORY;
  Context& C = ctx->c;
  C.P = *params;
  cudaGetDevice(&C.device);
  cudaDeviceGetAttribute(&C.sm_count, cudaDevAttrMultiProcessorCount, C.device);
  if (cudaStreamCreateWithFlags(&C.stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return TG_ERR_CUDA;
  }
  C.phys.xi = params->xi;
  C.phys.g = params->g;
  C.phys.mu = params->mu;
  C.phys.alpha = params->alpha;
  C.phys.cfl = params->cfl;
  C.phys.c_force = params->c_force;
  C.phys.c_visc = params->c_visc;
  C.phys.xi_is_7 = params->xi == 7.0 ? 1 : 0;
  C.phys.eos = params->eos;
  C.phys.viscosity = params->viscosity;
  C.phys.diffusion = params->diffusion;
  C.phys.kernel = params->kernel;
  C.phys.xi_f = static_cast<float>(params->xi);
  C.phys.g_f = static_cast<float>(params->g);
  C.phys.mu_f = static_cast<float>(params->mu);
  C.phys.alpha_f = static_cast<float>(params->alpha);
  C.phys.cfl_f = static_cast<float>(params->cfl);
  C.phys.c_force_f = static_cast<float>(params->c_force);
  C.phys.c_visc_f = static_cast<float>(params->c_visc);
  C.k = params->cells_per_radius;
  {
    const double cos_fov = std::cos(3.14159265358979323846 / 4.0);
    C.post_cos2_fov = cos_fov * cos_fov;
    C.post_k_fs = -std::log(0.05) / (0.01 * 0.01);
  }
  C.engine = tg::make_engine(params->dim, params->precision, params->kernel);
  if (!C.engine) {
    cudaStreamDestroy(C.stream);
    delete ctx;
    return TG_ERR_INVALID_ARGUMENT;
  }
  *out = ctx;
  return TG_OK;
}

int tg_context_destroy(tg_context* ctx) {
  if (ctx == nullptr) return TG_OK;
  Context& C = ctx->c;
  cudaStreamSynchronize(C.stream);
  C.pending.clear();
  for (cudaEvent_t e : C.event_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : C.timer_ev) {
    if (e != nullptr) cudaEventDestroy(e);
  }
  C.release_all();
  C.engine.reset();
  if (C.copy_stream != nullptr) {
    cudaStreamSynchronize(C.copy_stream);
    cudaStreamDestroy(C.copy_stream);
  }
  if (C.copy_ready != nullptr) cudaEventDestroy(C.copy_ready);
  cudaStreamDestroy(C.stream);
  delete ctx;
  return TG_OK;
}

int tg_particles_upload(tg_context* ctx, int32_t n_tanks, const tg_tank* tanks,
                        const double* r, const double* v, const double* rho) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  ctx->c.face_host.clear();  // faces index the previous particles
  return upload_particles(ctx, n_tanks, tanks, r, v, rho);
}

}  // extern "C"

namespace {

int upload_particles(tg_context* ctx, int32_t n_tanks, const tg_tank* tanks,
                     const double* r, const double* v, const double* rho) {
  Context& C = ctx->c;
  const int dim = C.P.dim;
  if (n_tanks < 1 || tanks == nullptr) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "need at least one tank");
  }
  int64_t n = 0, nf = 0, nw = 0;
  for (int32_t t = 0; t < n_tanks; ++t) {
    const tg_tank& T = tanks[t];
    if (T.n_fluid < 0 || T.n_wall < 0 || !(T.h > 0.0) || !(T.m > 0.0) ||
        !(T.rho0 > 0.0) || !(T.cs0 > 0.0) || !std::isfinite(T.h) ||
        !std::isfinite(T.m) || !std::isfinite(T.rho0) || !std::isfinite(T.cs0)) {
      return fail(&C, TG_ERR_INVALID_ARGUMENT,
                  "tank " + std::to_string(t) + ": invalid counts or constants");
    }
    n += T.n_fluid + T.n_wall;
    nf += T.n_fluid;
    nw += T.n_wall;
  }
  if (n >= (int64_t{1} << 31) - 1) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "more than 2^31 - 2 particles");
  }
  if (n > 0 && (r == nullptr || v == nullptr || rho == nullptr)) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "null particle array");
  }
  for (int64_t i = 0; i < n; ++i) {
    bool ok = std::isfinite(rho[i]) && rho[i] > 0.0;
    for (int k = 0; k < dim; ++k) {
      ok = ok && std::isfinite(r[i * dim + k]) && std::isfinite(v[i * dim + k]);
    }
    if (!ok) {
      return fail(&C, TG_ERR_INVALID_ARGUMENT,
                  "particle " + std::to_string(i) +
                      ": non-finite state or non-positive density");
    }
  }

  // Per-tank grids.
  std::vector<tg::TankDev> td(static_cast<size_t>(n_tanks));
  std::vector<uint32_t> id_base(static_cast<size_t>(n_tanks));
  std::vector<uint32_t> wall_from(static_cast<size_t>(n_tanks));
  uint64_t total_cells = 0;
  int64_t base = 0;
  for (int32_t t = 0; t < n_tanks; ++t) {
    const tg_tank& T = tanks[t];
    const int64_t nt = T.n_fluid + T.n_wall;
    tg::TankDev& D = td[t];
    std::memset(&D, 0, sizeof(D));
    const double R = tg::kernel_unit_radius(C.P.kernel) * T.h;
    const double cs = R / C.k * (1.0 + 1.0 / 65536.0);
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    if (nt > 0) {
      for (int k = 0; k < dim; ++k) lo[k] = hi[k] = r[base * dim + k];
      for (int64_t i = base; i < base + nt; ++i) {
        for (int k = 0; k < dim; ++k) {
          lo[k] = std::min(lo[k], r[i * dim + k]);
          hi[k] = std::max(hi[k], r[i * dim + k]);
        }
      }
    }
    // Headroom above the tank for splashes (particles beyond the grid are
    // clamped into its border cells, which stays exact but slows them).
    // Margins of R + 2 cells keep every particle's block of cells within k
    // of its own off the border cells.
    const double headroom = 0.25 * (hi[1] - lo[1]);
    uint64_t cells = 1;
    for (int k = 0; k < 3; ++k) {
      if (k < dim) {
        D.lo[k] = lo[k] - (R + 2.0 * cs);
        double top = hi[k] + (R + 2.0 * cs) + (k == 1 ? headroom : 0.0);
        const double ncf = std::max(1.0, std::ceil((top - D.lo[k]) / cs));
        if (ncf > 2.0e9) {
          return fail(&C, TG_ERR_INVALID_ARGUMENT, "tank grid too large");
        }
        D.nc[k] = static_cast<int32_t>(ncf);
      } else {
        D.lo[k] = 0.0;
        D.nc[k] = 1;
      }
      cells *= static_cast<uint64_t>(D.nc[k]);
    }
    D.cs = cs;
    D.inv_cs = 1.0 / cs;
    D.cell_off = static_cast<uint32_t>(total_cells);
    total_cells += cells;
    if (total_cells >= (uint64_t{1} << 30)) {
      return fail(&C, TG_ERR_INVALID_ARGUMENT,
                  "more than 2^30 grid cells; lower cells_per_radius");
    }
    D.h = T.h;
    D.hinv = 1.0 / T.h;
    D.radius2 = R * R;
    const float hf = static_cast<float>(T.h);
    const float Rf = static_cast<float>(tg::kernel_unit_radius(C.P.kernel)) * hf;
    D.radius2_f = Rf * Rf;
    D.band_lo_f = static_cast<float>(R * R * (1.0 - 1.0 / 16384.0));
    D.band_hi_f = static_cast<float>(R * R * (1.0 + 1.0 / 16384.0));
    D.cs_f = static_cast<float>(cs);
    D.inv_cs_f = static_cast<float>(1.0 / cs);
    double hinv_d = 1.0;
    for (int k = 0; k < dim; ++k) hinv_d *= D.hinv;
    D.w = kernel_weight(C.P.kernel, dim) * hinv_d;
    D.wg = D.w * D.hinv;
    D.m = T.m;
    D.rho0 = T.rho0;
    D.cs0 = T.cs0;
    D.B = T.rho0 * T.cs0 * T.cs0 / C.P.xi;
    D.diff_k = 2.0 * C.P.delta * T.h * T.cs0;
    D.visc_eps2 = 0.01 * T.h * T.h;
    D.n_fluid = static_cast<uint32_t>(T.n_fluid);
    D.h_f = static_cast<float>(D.h);
    D.hinv_f = static_cast<float>(D.hinv);
    D.w_f = static_cast<float>(D.w);
    D.wg_f = static_cast<float>(D.wg);
    D.m_f = static_cast<float>(D.m);
    D.rho0_f = static_cast<float>(D.rho0);
    D.cs0_f = static_cast<float>(D.cs0);
    D.B_f = static_cast<float>(D.B);
    D.diff_k_f = static_cast<float>(D.diff_k);
    D.visc_eps2_f = static_cast<float>(D.visc_eps2);
    D.c02_f = static_cast<float>(D.cs0 * D.cs0);
    {
      const double rc = R * (1.0 + 1.0 / 4096.0);
      D.cull_r2_f = static_cast<float>(rc * rc);
      double extent = 0.0;
      for (int k = 0; k < dim; ++k) extent = std::max(extent, D.nc[k] * cs);
      const double rs = rc + extent / 524288.0;
      D.wall_skip_r2_f = static_cast<float>(rs * rs);
    }
    id_base[t] = static_cast<uint32_t>(base);
    wall_from[t] = static_cast<uint32_t>(base + T.n_fluid);
    base += nt;
  }

  // (Re)allocate.
  cudaStreamSynchronize(C.stream);
  C.release_all();
  C.n = n;
  C.n_fluid = nf;
  C.n_wall = nw;
  C.ntanks = n_tanks;
  C.tanks.assign(tanks, tanks + n_tanks);
  C.tankdev = td;
  C.id_base = id_base;
  C.wall_from = wall_from;
  C.total_cells = static_cast<uint32_t>(total_cells);
  C.total_keys = static_cast<uint32_t>(2 * total_cells);
  C.key_bits = key_bits_for(C.total_keys);
  const int64_t nn = n > 0 ? n : 1;
  auto A = [&](auto*& p, size_t bytes) -> cudaError_t {
    return C.alloc(reinterpret_cast<void**>(&p), bytes);
  };
  TG_CUDA(&C, A(C.d_tanks, sizeof(tg::TankDev) * n_tanks));
  TG_CUDA(&C, A(C.d_tank_off, sizeof(uint32_t) * n_tanks));
  TG_CUDA(&C, A(C.d_id_base, sizeof(uint32_t) * n_tanks));
  TG_CUDA(&C, A(C.d_wall_from, sizeof(uint32_t) * n_tanks));
  TG_CUDA(&C, A(C.d_tank_of, sizeof(uint32_t) * nn));
  TG_CUDA(&C, A(C.d_dt, sizeof(double) * n_tanks));
  TG_CUDA(&C, A(C.d_dt_last, sizeof(double) * n_tanks));
  TG_CUDA(&C, A(C.d_time, sizeof(double) * n_tanks));
  TG_CUDA(&C, A(C.d_err, sizeof(uint32_t)));
  TG_CUDA(&C, A(C.d_wall_count, 2 * sizeof(uint32_t)));
  TG_CUDA(&C, A(C.d_fbox, sizeof(unsigned) * 6 * n_tanks));
  TG_CUDA(&C, A(C.keys_a, sizeof(uint32_t) * nn));
  TG_CUDA(&C, A(C.keys_b, sizeof(uint32_t) * nn));
  TG_CUDA(&C, A(C.vals_a, sizeof(uint32_t) * nn));
  TG_CUDA(&C, A(C.vals_b, sizeof(uint32_t) * nn));
  TG_CUDA(&C, C.alloc(&C.sort_scratch, tg::radix_sort_scratch_bytes(nn)));
  TG_CUDA(&C, C.alloc(&C.near_scratch, tg::near_sort_scratch_bytes(nn)));
  TG_CUDA(&C, A(C.cell_start, sizeof(uint32_t) * (2 * total_cells + 1)));
  TG_CUDA(&C, C.alloc(&C.cell_scratch, tg::cell_fill_scratch_bytes(C.total_keys)));
  TG_CUDA(&C, A(C.wall_list, sizeof(uint32_t) * (nw > 0 ? nw : 1)));
  TG_CUDA(&C, A(C.wall_active, sizeof(uint32_t) * (nw > 0 ? nw : 1)));
  TG_CUDA(&C, A(C.d_stage, sizeof(double) * nn * dim));
  TG_CUDA(&C, A(C.d_stage2, sizeof(double) * nn * dim));
  TG_CUDA(&C, A(C.d_stage3, sizeof(double) * nn * dim));
  TG_CUDA(&C, A(C.d_stage4, sizeof(double) * nn * dim));
  TG_CUDA(&C, A(C.d_sd_rho, sizeof(double) * nn));
  TG_CUDA(&C, A(C.d_sd_count, sizeof(int32_t) * nn));
  TG_CUDA(&C, A(C.d_sd_hash, sizeof(uint64_t) * nn));
  TG_CUDA(&C, C.alloc(&C.d_cloud_rec, 32 * static_cast<size_t>(nn)));
  TG_CUDA(&C, C.engine->allocate(C));

  std::vector<uint32_t> tank_of(static_cast<size_t>(nn), 0);
  base = 0;
  for (int32_t t = 0; t < n_tanks; ++t) {
    const int64_t nt = tanks[t].n_fluid + tanks[t].n_wall;
    for (int64_t i = 0; i < nt; ++i) tank_of[base + i] = static_cast<uint32_t>(t);
    base += nt;
  }
  std::vector<double> inf(static_cast<size_t>(n_tanks),
                          std::numeric_limits<double>::infinity());
  std::vector<double> zeros(static_cast<size_t>(n_tanks), 0.0);
  cudaStream_t s = C.stream;
  TG_CUDA(&C, tg::near_sort_reset(C.near_scratch, nn, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_tanks, td.data(), sizeof(tg::TankDev) * n_tanks,
                              cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_id_base, id_base.data(), sizeof(uint32_t) * n_tanks,
                              cudaMemcpyHostToDevice, s));
  std::vector<uint32_t> tank_off(static_cast<size_t>(n_tanks));
  for (int32_t t = 0; t < n_tanks; ++t) tank_off[t] = 2 * td[t].cell_off;
  TG_CUDA(&C, cudaMemcpyAsync(C.d_tank_off, tank_off.data(), sizeof(uint32_t) * n_tanks,
                              cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_wall_from, wall_from.data(),
                              sizeof(uint32_t) * n_tanks, cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_tank_of, tank_of.data(), sizeof(uint32_t) * nn,
                              cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_dt, inf.data(), sizeof(double) * n_tanks,
                              cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_dt_last, zeros.data(), sizeof(double) * n_tanks,
                              cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_time, zeros.data(), sizeof(double) * n_tanks,
                              cudaMemcpyHostToDevice, s));
  TG_CUDA(&C, cudaMemsetAsync(C.d_err, 0, sizeof(uint32_t), s));
  if (n > 0) {
    TG_CUDA(&C, cudaMemcpyAsync(C.d_stage, r, sizeof(double) * n * dim,
                                cudaMemcpyHostToDevice, s));
    TG_CUDA(&C, cudaMemcpyAsync(C.d_stage2, v, sizeof(double) * n * dim,
                                cudaMemcpyHostToDevice, s));
    TG_CUDA(&C, cudaMemcpyAsync(C.d_stage3, rho, sizeof(double) * n,
                                cudaMemcpyHostToDevice, s));
    TG_CUDA(&C, C.engine->upload_state(C, C.d_stage, C.d_stage2, C.d_stage3, nullptr));
  }
  TG_CUDA(&C, cudaStreamSynchronize(s));
  C.uploaded = true;
  C.walls_fresh = false;
  return TG_OK;
}

}  // namespace

extern "C" {

int tg_particles_update(tg_context* ctx, const double* r, const double* v,
                        const double* rho, const double* dv_dt) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (C.n == 0) return TG_OK;
  if (r == nullptr || v == nullptr || rho == nullptr) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "null particle array");
  }
  const int dim = C.P.dim;
  cudaStream_t s = C.stream;
  // Page-locked host arrays are read by the unpack kernel itself over the
  // host link; other host memory goes through the staging buffers.
  const double* dr = mapped_host(r);
  const double* dv = mapped_host(v);
  const double* drho = mapped_host(rho);
  const double* ddv = dv_dt != nullptr ? mapped_host(dv_dt) : nullptr;
  if (dr != nullptr && dv != nullptr && drho != nullptr &&
      (dv_dt == nullptr || ddv != nullptr)) {
    TG_CUDA(&C, C.engine->upload_state(C, dr, dv, drho, ddv));
  } else {
    TG_CUDA(&C, cudaMemcpyAsync(C.d_stage, r, sizeof(double) * C.n * dim,
                                cudaMemcpyHostToDevice, s));
    TG_CUDA(&C, cudaMemcpyAsync(C.d_stage2, v, sizeof(double) * C.n * dim,
                                cudaMemcpyHostToDevice, s));
    TG_CUDA(&C, cudaMemcpyAsync(C.d_stage3, rho, sizeof(double) * C.n,
                                cudaMemcpyHostToDevice, s));
    if (dv_dt != nullptr) {
      TG_CUDA(&C, cudaMemcpyAsync(C.d_stage4, dv_dt, sizeof(double) * C.n * dim,
                                  cudaMemcpyHostToDevice, s));
    }
    TG_CUDA(&C, C.engine->upload_state(C, C.d_stage, C.d_stage2, C.d_stage3,
                                       dv_dt != nullptr ? C.d_stage4 : nullptr));
  }
  // The host arrays may be reused as soon as this returns.
  TG_CUDA(&C, cudaStreamSynchronize(s));
  C.walls_fresh = false;
  return TG_OK;
}

int tg_prepare(tg_context* ctx) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  TG_CUDA(&C, C.engine->enqueue_prepare(C));
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  C.walls_fresh = true;
  return TG_OK;
}

int tg_step(tg_context* ctx, int32_t n_steps, double* dt_out) {
  if (ctx == nullptr || n_steps < 0) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (n_steps > 0 && C.n > 0) {
    TG_CUDA(&C, C.engine->ensure_keys(C));
    if (C.use_graph && !C.profile) {
      // The re-sort is taken only in the home order of an earlier sort, a
      // host-side choice baked into the graph: run a step directly when the
      // order is not there yet, and capture again when it changed.
      if (C.graph_exec != nullptr && C.graph_order != C.order_valid) C.invalidate_graph();
      if (!C.order_valid && C.P.resort != 0 && n_steps > 1) {
        TG_CUDA(&C, C.engine->enqueue_step(C));
        --n_steps;
        C.prof.steps += 1;
      }
      if (C.graph_exec == nullptr) {
        C.graph_order = C.order_valid;
        cudaGraph_t graph = nullptr;
        const int64_t before = C.launches;
        TG_CUDA(&C, cudaStreamBeginCapture(C.stream,
                                           cudaStreamCaptureModeThreadLocal));
        const cudaError_t e = C.engine->enqueue_step(C);
        const cudaError_t e2 = cudaStreamEndCapture(C.stream, &graph);
        if (e != cudaSuccess) return cuda_fail(&C, e, "enqueue_step");
        if (e2 != cudaSuccess) return cuda_fail(&C, e2, "cudaStreamEndCapture");
        C.graph_kernels = C.launches - before;
        C.launches = before;
        const cudaError_t e3 = cudaGraphInstantiate(&C.graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e3 != cudaSuccess) {
          C.graph_exec = nullptr;
          return cuda_fail(&C, e3, "cudaGraphInstantiate");
        }
      }
      for (int32_t i = 0; i < n_steps; ++i) {
        TG_CUDA(&C, cudaGraphLaunch(C.graph_exec, C.stream));
        C.launches += C.graph_kernels;
      }
    } else {
      for (int32_t i = 0; i < n_steps; ++i) {
        TG_CUDA(&C, C.engine->enqueue_step(C));
        C.prof.stages += tg::force_passes(C.P.integrator);
        C.prof.forces_launches += tg::force_passes(C.P.integrator);
      }
    }
    C.prof.steps += n_steps;
    // With shifting, the post-integration prepare left the walls as the
    // reference leaves them (extrapolated before the shift); otherwise the
    // reference's closing prepare runs on the next density download.
    C.walls_fresh = C.P.post_integrate == TG_POST_SHIFTING;
  }
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  C.drain_profile();
  uint32_t err = 0;
  TG_CUDA(&C, cudaMemcpy(&err, C.d_err, sizeof(err), cudaMemcpyDeviceToHost));
  if (dt_out != nullptr) {
    TG_CUDA(&C, cudaMemcpy(dt_out, C.d_dt_last, sizeof(double) * C.ntanks,
                           cudaMemcpyDeviceToHost));
  }
  if (err & (TG_DEV_NONFINITE_STATE | TG_DEV_BAD_DT)) {
    return fail(&C, TG_ERR_DEVICE_STATE,
                "device error word " + std::to_string(err) +
                    " (non-finite state or bad time step)");
  }
  return TG_OK;
}

int tg_time(tg_context* ctx, double* time_out) {
  if (ctx == nullptr || time_out == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  TG_CUDA(&C, cudaMemcpy(time_out, C.d_time, sizeof(double) * C.ntanks,
                         cudaMemcpyDeviceToHost));
  return TG_OK;
}

int tg_particles_download(tg_context* ctx, int32_t field, double* out) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (field < TG_FIELD_R || field > TG_FIELD_CS) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "unknown field");
  }
  if (C.n == 0) return TG_OK;
  if (out == nullptr) return fail(&C, TG_ERR_INVALID_ARGUMENT, "null output");
  if ((field == TG_FIELD_RHO || field == TG_FIELD_P || field == TG_FIELD_CS) &&
      !C.walls_fresh && C.n_wall > 0) {
    TG_CUDA(&C, C.engine->enqueue_prepare(C));
    C.walls_fresh = true;
  }
  TG_CUDA(&C, C.engine->enqueue_pack(C, field));
  const int comps = (field == TG_FIELD_R || field == TG_FIELD_V ||
                     field == TG_FIELD_DV_DT)
                        ? C.P.dim
                        : 1;
  TG_CUDA(&C, cudaMemcpyAsync(out, C.d_stage, sizeof(double) * C.n * comps,
                              cudaMemcpyDeviceToHost, C.stream));
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  return TG_OK;
}

int tg_particles_download_state(tg_context* ctx, double* r, double* v,
                                double* rho, double* drho_dt, double* dv_dt) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (C.n == 0) return TG_OK;
  const size_t n = static_cast<size_t>(C.n), dim = static_cast<size_t>(C.P.dim);
  double* d_rho = C.d_stage3;
  double* d_drho = C.d_stage3 + n;
  const auto get = [&](double* dst, const double* src, size_t count,
                       cudaStream_t s) -> cudaError_t {
    if (dst == nullptr) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost, s);
  };
  const bool prepare = rho != nullptr && !C.walls_fresh && C.n_wall > 0;
  if (!prepare) {
    TG_CUDA(&C, C.engine->enqueue_pack_state(C, r ? C.d_stage : nullptr,
                                             v ? C.d_stage2 : nullptr,
                                             rho ? d_rho : nullptr,
                                             drho_dt ? d_drho : nullptr,
                                             dv_dt ? C.d_stage4 : nullptr));
    TG_CUDA(&C, get(r, C.d_stage, n * dim, C.stream));
    TG_CUDA(&C, get(v, C.d_stage2, n * dim, C.stream));
    TG_CUDA(&C, get(rho, d_rho, n, C.stream));
    TG_CUDA(&C, get(drho_dt, d_drho, n, C.stream));
    TG_CUDA(&C, get(dv_dt, C.d_stage4, n * dim, C.stream));
    TG_CUDA(&C, cudaStreamSynchronize(C.stream));
    return TG_OK;
  }
  // The densities need the closing prepare (the wall extrapolation at the
  // current positions); r, v and dv/dt do not change in it (it only puts
  // the home state in the new cell order), so they are packed first and
  // copied on a second stream while the prepare runs.
  if (C.copy_stream == nullptr) {
    TG_CUDA(&C, cudaStreamCreateWithFlags(&C.copy_stream, cudaStreamNonBlocking));
    TG_CUDA(&C, cudaEventCreateWithFlags(&C.copy_ready, cudaEventDisableTiming));
  }
  TG_CUDA(&C, C.engine->enqueue_pack_state(C, r ? C.d_stage : nullptr,
                                           v ? C.d_stage2 : nullptr, nullptr, nullptr,
                                           dv_dt ? C.d_stage4 : nullptr));
  TG_CUDA(&C, cudaEventRecord(C.copy_ready, C.stream));
  TG_CUDA(&C, cudaStreamWaitEvent(C.copy_stream, C.copy_ready, 0));
  TG_CUDA(&C, get(r, C.d_stage, n * dim, C.copy_stream));
  TG_CUDA(&C, get(v, C.d_stage2, n * dim, C.copy_stream));
  TG_CUDA(&C, get(dv_dt, C.d_stage4, n * dim, C.copy_stream));
  TG_CUDA(&C, C.engine->enqueue_prepare(C));
  C.walls_fresh = true;
  TG_CUDA(&C, C.engine->enqueue_pack_state(C, nullptr, nullptr, d_rho,
                                           drho_dt ? d_drho : nullptr, nullptr));
  TG_CUDA(&C, get(rho, d_rho, n, C.stream));
  TG_CUDA(&C, get(drho_dt, d_drho, n, C.stream));
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  TG_CUDA(&C, cudaStreamSynchronize(C.copy_stream));
  return TG_OK;
}

int tg_neighbour_counts(tg_context* ctx, int32_t* counts, uint64_t* hashes) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (C.n == 0) return TG_OK;
  TG_CUDA(&C, C.engine->enqueue_neighbours(C, C.d_sd_count, C.d_sd_hash,
                                           nullptr, nullptr));
  if (counts != nullptr) {
    TG_CUDA(&C, cudaMemcpyAsync(counts, C.d_sd_count, sizeof(int32_t) * C.n,
                                cudaMemcpyDeviceToHost, C.stream));
  }
  if (hashes != nullptr) {
    TG_CUDA(&C, cudaMemcpyAsync(hashes, C.d_sd_hash, sizeof(uint64_t) * C.n,
                                cudaMemcpyDeviceToHost, C.stream));
  }
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  return TG_OK;
}

int tg_neighbour_lists(tg_context* ctx, int64_t* offsets, int32_t* indices,
                       int64_t capacity) {
  if (ctx == nullptr || offsets == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  const int64_t n = C.n;
  offsets[0] = 0;
  if (n == 0) return TG_OK;
  std::vector<int32_t> counts(static_cast<size_t>(n));
  const int st = tg_neighbour_counts(ctx, counts.data(), nullptr);
  if (st != TG_OK) return st;
  for (int64_t i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + counts[i];
  const int64_t total = offsets[n];
  if (indices == nullptr || capacity < total) {
    return fail(&C, TG_ERR_CAPACITY,
                "neighbour lists need " + std::to_string(total) + " entries");
  }
  int64_t* d_off = nullptr;
  int32_t* d_idx = nullptr;
  TG_CUDA(&C, cudaMalloc(&d_off, sizeof(int64_t) * (n + 1)));
  cudaError_t e = cudaMalloc(&d_idx, sizeof(int32_t) * (total > 0 ? total : 1));
  if (e != cudaSuccess) {
    cudaFree(d_off);
    return cuda_fail(&C, e, "cudaMalloc");
  }
  e = cudaMemcpyAsync(d_off, offsets, sizeof(int64_t) * (n + 1),
                      cudaMemcpyHostToDevice, C.stream);
  if (e == cudaSuccess) {
    e = C.engine->enqueue_neighbours(C, nullptr, nullptr, d_off, d_idx);
  }
  if (e == cudaSuccess) {
    e = cudaMemcpyAsync(indices, d_idx, sizeof(int32_t) * total,
                        cudaMemcpyDeviceToHost, C.stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(C.stream);
  cudaFree(d_off);
  cudaFree(d_idx);
  if (e != cudaSuccess) return cuda_fail(&C, e, "tg_neighbour_lists");
  for (int64_t i = 0; i < n; ++i) {
    std::sort(indices + offsets[i], indices + offsets[i + 1]);
  }
  return TG_OK;
}

int tg_summation_density(tg_context* ctx, int32_t pos_precision,
                         double* rho_out, int32_t* counts, uint64_t* hashes) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (pos_precision != TG_POS_FP64 && pos_precision != TG_POS_FP32) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "unknown position precision");
  }
  if (C.n == 0) return TG_OK;
  TG_CUDA(&C, C.engine->enqueue_sumdens(C, pos_precision, C.d_sd_rho,
                                        C.d_sd_count, C.d_sd_hash));
  if (rho_out != nullptr) {
    TG_CUDA(&C, cudaMemcpyAsync(rho_out, C.d_sd_rho, sizeof(double) * C.n,
                                cudaMemcpyDeviceToHost, C.stream));
  }
  if (counts != nullptr) {
    TG_CUDA(&C, cudaMemcpyAsync(counts, C.d_sd_count, sizeof(int32_t) * C.n,
                                cudaMemcpyDeviceToHost, C.stream));
  }
  if (hashes != nullptr) {
    TG_CUDA(&C, cudaMemcpyAsync(hashes, C.d_sd_hash, sizeof(uint64_t) * C.n,
                                cudaMemcpyDeviceToHost, C.stream));
  }
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  C.drain_profile();
  return TG_OK;
}

int tg_summation_density_resident(tg_context* ctx, int32_t pos_precision) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (pos_precision != TG_POS_FP64 && pos_precision != TG_POS_FP32) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "unknown position precision");
  }
  if (C.n == 0) return TG_OK;
  TG_CUDA(&C, C.engine->enqueue_sumdens(C, pos_precision, C.d_sd_rho,
                                        C.d_sd_count, C.d_sd_hash));
  return TG_OK;
}

int tg_device_status(tg_context* ctx, uint32_t* flags) {
  if (ctx == nullptr || flags == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  *flags = 0;
  if (!C.uploaded) return TG_OK;
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  TG_CUDA(&C, cudaMemcpy(flags, C.d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  TG_CUDA(&C, cudaMemset(C.d_err, 0, sizeof(uint32_t)));
  return TG_OK;
}

int tg_profile_enable(tg_context* ctx, int32_t enable) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  C.drain_profile();
  C.profile = enable != 0;
  std::memset(&C.prof, 0, sizeof(C.prof));
  return TG_OK;
}

int tg_profile_read(tg_context* ctx, tg_profile* out) {
  if (ctx == nullptr || out == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  C.drain_profile();
  *out = C.prof;
  return TG_OK;
}

int tg_set_graph(tg_context* ctx, int32_t enable) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  ctx->c.use_graph = enable != 0;
  return TG_OK;
}

int tg_launch_count(tg_context* ctx, int64_t* count) {
  if (ctx == nullptr || count == nullptr) return TG_ERR_INVALID_ARGUMENT;
  *count = ctx->c.launches;
  return TG_OK;
}

int tg_synchronize(tg_context* ctx) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  TG_CUDA(&ctx->c, cudaStreamSynchronize(ctx->c.stream));
  return TG_OK;
}

int tg_timer_start(tg_context* ctx) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  for (cudaEvent_t& ev : C.timer_ev) {
    if (ev == nullptr) TG_CUDA(&C, cudaEventCreate(&ev));
  }
  TG_CUDA(&C, cudaEventRecord(C.timer_ev[0], C.stream));
  return TG_OK;
}

int tg_timer_stop(tg_context* ctx, double* ms) {
  if (ctx == nullptr || ms == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (C.timer_ev[0] == nullptr) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "timer not started");
  }
  TG_CUDA(&C, cudaEventRecord(C.timer_ev[1], C.stream));
  TG_CUDA(&C, cudaEventSynchronize(C.timer_ev[1]));
  float f = 0.f;
  TG_CUDA(&C, cudaEventElapsedTime(&f, C.timer_ev[0], C.timer_ev[1]));
  *ms = f;
  return TG_OK;
}

// ---- boundary faces ------------------------------------------------------
}  // extern "C"

namespace {

// Exact generalized winding number of a closed triangle mesh at x (9
// doubles per triangle; the solid-angle sum of the device's
// face_contains3).
double winding_number3(const std::vector<double>& tris, size_t first, size_t count,
                       const double* x) {
  double w = 0.0;
  for (size_t i = first; i < first + count; ++i) {
    const double* t = tris.data() + 9 * i;
    double ap[3], bp[3], cp[3];
    for (int k = 0; k < 3; ++k) {
      ap[k] = t[k] - x[k];
      bp[k] = t[3 + k] - x[k];
      cp[k] = t[6 + k] - x[k];
    }
    auto dot = [](const double* a, const double* b) {
      return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
    };
    const double na = std::sqrt(dot(ap, ap)), nb = std::sqrt(dot(bp, bp)),
                 nc = std::sqrt(dot(cp, cp));
    const double den = na * nb * nc + dot(ap, bp) * nc + dot(bp, cp) * na + dot(cp, ap) * nb;
    const double bc[3] = {bp[1] * cp[2] - bp[2] * cp[1], bp[2] * cp[0] - bp[0] * cp[2],
                          bp[0] * cp[1] - bp[1] * cp[0]};
    w += std::atan2(dot(ap, bc), den) / (2.0 * 3.141592653589793);
  }
  return w;
}

// Device tables of the boundary faces of every tank (face_host): face
// coordinates and vertex ids, per-cell face lists (each face registered in
// every cell of its bounding box grown by the support radius, so a cell's
// list holds every face within reach of its points, ascending), the
// containment tables (2D: per-row polygon edge lists; 3D: per-cell answers
// and the surface's triangles), and the per-particle gamma buffers.
//
// 3D containment per tank: every cell that a containment triangle's
// bounding box (grown by a hair) reaches is marked for the exact test; the
// remaining cells split into face-connected components that the surface
// does not cross, so the winding number is constant on each, and one exact
// evaluation at a cell centre answers for the whole component.
int build_faces(tg_context* ctx) {
  Context& C = ctx->c;
  C.faces = tg::FaceArgs{};
  bool any = false;
  for (const auto& t : C.face_host) any = any || !t.face_verts.empty();
  if (!any) return TG_OK;
  const int32_t nt = C.ntanks;
  const int D = C.P.dim;
  // Fixed-particle positions (the face vertices).
  std::vector<double> r(static_cast<size_t>(C.n) * D);
  int st = tg_particles_download(ctx, TG_FIELD_R, r.data());
  if (st != TG_OK) return st;
  const double unit_radius = tg::kernel_unit_radius(C.P.kernel);
  std::vector<double> coords, edges, cont_tri;
  std::vector<uint32_t> vert;
  std::vector<uint32_t> cell_count(static_cast<size_t>(C.total_cells) + 1, 0);
  std::vector<std::pair<uint32_t, uint32_t>> cell_pairs;  // (cell, face)
  std::vector<uint32_t> row_off(static_cast<size_t>(nt), 0), tank_edges(static_cast<size_t>(nt), 0);
  std::vector<uint32_t> cont_start(static_cast<size_t>(nt) + 1, 0);
  std::vector<int8_t> cell_state;
  if (D == 3) cell_state.assign(static_cast<size_t>(C.total_cells), 1);
  uint32_t total_rows = 0;
  for (int32_t t = 0; t < nt; ++t) {
    row_off[t] = total_rows;
    if (D == 2) total_rows += static_cast<uint32_t>(C.tankdev[t].nc[1]);
  }
  std::vector<std::vector<uint32_t>> row_lists(total_rows);
  for (int32_t t = 0; t < nt; ++t) {
    cont_start[t] = static_cast<uint32_t>(cont_tri.size() / 9);
    if (static_cast<size_t>(t) >= C.face_host.size()) continue;
    const auto& F = C.face_host[t];
    if (F.face_verts.empty()) continue;
    const tg::TankDev& T = C.tankdev[t];
    const double R = unit_radius * C.tanks[t].h;
    auto cell_index = [&](double x, int k) {
      const double f = std::floor((x - T.lo[k]) * T.inv_cs);
      return static_cast<int>(std::min(std::max(f, 0.0), static_cast<double>(T.nc[k] - 1)));
    };
    auto gcell = [&](int x, int y, int z) {
      return T.cell_off + (static_cast<uint32_t>(z) * T.nc[1] + static_cast<uint32_t>(y)) *
                              static_cast<uint32_t>(T.nc[0]) + static_cast<uint32_t>(x);
    };
    for (size_t f = 0; f < F.face_verts.size() / D; ++f) {
      const uint32_t gf = static_cast<uint32_t>(vert.size() / D);
      double lo[3] = {0.0, 0.0, 0.0}, hi[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < D; ++j) {
        const uint32_t u = C.wall_from[t] + static_cast<uint32_t>(F.face_verts[D * f + j]);
        vert.push_back(u);
        for (int k = 0; k < D; ++k) {
          const double x = r[static_cast<size_t>(D) * u + k];
          coords.push_back(x);
          lo[k] = j == 0 ? x : std::min(lo[k], x);
          hi[k] = j == 0 ? x : std::max(hi[k], x);
        }
      }
      int c0[3] = {0, 0, 0}, c1[3] = {0, 0, 0};
      for (int k = 0; k < D; ++k) {
        c0[k] = cell_index(lo[k] - R, k);
        c1[k] = cell_index(hi[k] + R, k);
      }
      for (int z = c0[2]; z <= c1[2]; ++z) {
        for (int y = c0[1]; y <= c1[1]; ++y) {
          for (int x = c0[0]; x <= c1[0]; ++x) {
            const uint32_t gc = gcell(x, y, z);
            cell_pairs.emplace_back(gc, gf);
            ++cell_count[gc];
          }
        }
      }
    }
    if (D == 2) {
      const size_t np = F.poly.size() / 2;
      for (size_t e = 0; e < np; ++e) {
        const size_t e1 = (e + 1) % np;
        const double x0 = F.poly[2 * e], y0 = F.poly[2 * e + 1];
        const double x1 = F.poly[2 * e1], y1 = F.poly[2 * e1 + 1];
        const uint32_t ge = static_cast<uint32_t>(edges.size() / 4);
        edges.insert(edges.end(), {x0, y0, x1, y1});
        const int r0 = cell_index(std::min(y0, y1), 1), r1 = cell_index(std::max(y0, y1), 1);
        for (int y = r0; y <= r1; ++y) row_lists[row_off[t] + y].push_back(ge);
        ++tank_edges[t];
      }
      continue;
    }
    // 3D containment of this tank.
    const size_t first = cont_tri.size() / 9;
    const size_t ntri = F.poly.size() / 9;
    cont_tri.insert(cont_tri.end(), F.poly.begin(), F.poly.end());
    tank_edges[t] = static_cast<uint32_t>(ntri);
    const double hair = 1e-9 * T.cs;
    for (size_t i = 0; i < ntri; ++i) {
      const double* tri = F.poly.data() + 9 * i;
      int c0[3], c1[3];
      for (int k = 0; k < 3; ++k) {
        const double lo = std::min(std::min(tri[k], tri[3 + k]), tri[6 + k]);
        const double hi = std::max(std::max(tri[k], tri[3 + k]), tri[6 + k]);
        c0[k] = cell_index(lo - hair, k);
        c1[k] = cell_index(hi + hair, k);
      }
      for (int z = c0[2]; z <= c1[2]; ++z) {
        for (int y = c0[1]; y <= c1[1]; ++y) {
          for (int x = c0[0]; x <= c1[0]; ++x) cell_state[gcell(x, y, z)] = -1;
        }
      }
    }
    // Components of the unmarked cells (face neighbours), one exact
    // evaluation each.
    const uint32_t ncell = static_cast<uint32_t>(T.nc[0]) * T.nc[1] * T.nc[2];
    std::vector<uint8_t> seen(ncell, 0);
    std::vector<uint32_t> stack;
    for (uint32_t l = 0; l < ncell; ++l) {
      if (seen[l] || cell_state[T.cell_off + l] < 0) continue;
      const int lx = static_cast<int>(l % T.nc[0]);
      const int ly = static_cast<int>((l / T.nc[0]) % T.nc[1]);
      const int lz = static_cast<int>(l / (static_cast<uint32_t>(T.nc[0]) * T.nc[1]));
      const double centre[3] = {T.lo[0] + (lx + 0.5) * T.cs, T.lo[1] + (ly + 0.5) * T.cs,
                                T.lo[2] + (lz + 0.5) * T.cs};
      const int8_t in = winding_number3(cont_tri, first, ntri, centre) > 0.5 ? 1 : 0;
      stack.assign(1, l);
      seen[l] = 1;
      while (!stack.empty()) {
        const uint32_t m = stack.back();
        stack.pop_back();
        cell_state[T.cell_off + m] = in;
        const int mx = static_cast<int>(m % T.nc[0]);
        const int my = static_cast<int>((m / T.nc[0]) % T.nc[1]);
        const int mz = static_cast<int>(m / (static_cast<uint32_t>(T.nc[0]) * T.nc[1]));
        const int nb[6][3] = {{mx - 1, my, mz}, {mx + 1, my, mz}, {mx, my - 1, mz},
                              {mx, my + 1, mz}, {mx, my, mz - 1}, {mx, my, mz + 1}};
        for (const auto& q : nb) {
          if (q[0] < 0 || q[1] < 0 || q[2] < 0 || q[0] >= T.nc[0] || q[1] >= T.nc[1] ||
              q[2] >= T.nc[2]) {
            continue;
          }
          const uint32_t n2 = gcell(q[0], q[1], q[2]) - T.cell_off;
          if (seen[n2] || cell_state[T.cell_off + n2] < 0) continue;
          seen[n2] = 1;
          stack.push_back(n2);
        }
      }
    }
  }
  cont_start[nt] = static_cast<uint32_t>(cont_tri.size() / 9);
  // Coplanar neighbours across each edge (3D) or collinear neighbours
  // across each end (2D), see face_skip_edges: 3D, the edge shared by
  // exactly two faces that traverse it in opposite directions, with equal
  // unit normals and the same plane; 2D, the only segment ending at a
  // vertex and the only one starting there, on the same line with the same
  // direction.
  const size_t nfaces = vert.size() / static_cast<size_t>(D);
  std::vector<int32_t> edge_nbr(std::max<size_t>(1, static_cast<size_t>(D) * nfaces), -1);
  if (D == 2) {
    std::map<uint32_t, std::pair<std::vector<uint32_t>, std::vector<uint32_t>>> at;  // in, out
    double scale = 0.0;
    for (size_t f = 0; f < nfaces; ++f) {
      at[vert[2 * f + 1]].first.push_back(static_cast<uint32_t>(f));
      at[vert[2 * f]].second.push_back(static_cast<uint32_t>(f));
      for (int k = 0; k < 4; ++k) scale = std::max(scale, std::fabs(coords[4 * f + k]));
    }
    const auto line = [&](size_t f) {
      const double* a = coords.data() + 4 * f;
      double e[2] = {a[2] - a[0], a[3] - a[1]};
      const double len = std::sqrt(e[0] * e[0] + e[1] * e[1]);
      if (len > 0.0) {
        e[0] /= len;
        e[1] /= len;
      }
      return std::array<double, 3>{e[0], e[1], e[1] * a[0] - e[0] * a[1]};
    };
    const double tol_n = 1e-12, tol_d = 1e-12 * std::max(scale, 1.0);
    for (const auto& [u, io] : at) {
      if (io.first.size() != 1 || io.second.size() != 1) continue;
      const uint32_t fi = io.first[0], fo = io.second[0];
      if (fi == fo) continue;
      const auto P = line(fi), Q = line(fo);
      if (std::fabs(P[0] - Q[0]) > tol_n || std::fabs(P[1] - Q[1]) > tol_n ||
          std::fabs(P[2] - Q[2]) > tol_d || P[0] * P[0] + P[1] * P[1] < 0.5) {
        continue;
      }
      edge_nbr[2 * fi + 1] = static_cast<int32_t>(fo);  // across fi's end b
      edge_nbr[2 * fo] = static_cast<int32_t>(fi);      // across fo's end a
    }
  }
  if (D == 3) {
    std::vector<std::array<double, 4>> plane(nfaces);  // unit normal, offset
    double scale = 0.0;
    for (size_t f = 0; f < nfaces; ++f) {
      const double* a = coords.data() + 9 * f;
      const double u[3] = {a[3] - a[0], a[4] - a[1], a[5] - a[2]};
      const double w[3] = {a[6] - a[0], a[7] - a[1], a[8] - a[2]};
      double n[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2],
                     u[0] * w[1] - u[1] * w[0]};
      const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      if (len > 0.0) {
        for (double& c : n) c /= len;
      }
      plane[f] = {n[0], n[1], n[2], n[0] * a[0] + n[1] * a[1] + n[2] * a[2]};
      for (int k = 0; k < 9; ++k) scale = std::max(scale, std::fabs(a[k]));
    }
    std::map<std::pair<uint32_t, uint32_t>, std::vector<std::pair<uint32_t, int>>> edges_of;
    for (size_t f = 0; f < nfaces; ++f) {
      for (int e = 0; e < 3; ++e) {
        const uint32_t p0 = vert[3 * f + e], p1 = vert[3 * f + (e + 1) % 3];
        edges_of[{std::min(p0, p1), std::max(p0, p1)}].emplace_back(
            static_cast<uint32_t>(f), e);
      }
    }
    const double tol_n = 1e-12, tol_d = 1e-12 * std::max(scale, 1.0);
    for (const auto& [key, list] : edges_of) {
      if (list.size() != 2) continue;
      const auto [f0, e0] = list[0];
      const auto [f1, e1] = list[1];
      // Opposite traversal: f0 runs p -> q where f1 runs q -> p.
      if (vert[3 * f0 + e0] != vert[3 * f1 + (e1 + 1) % 3]) continue;
      const auto& P = plane[f0];
      const auto& Q = plane[f1];
      if (std::fabs(P[0] - Q[0]) > tol_n || std::fabs(P[1] - Q[1]) > tol_n ||
          std::fabs(P[2] - Q[2]) > tol_n || std::fabs(P[3] - Q[3]) > tol_d ||
          P[0] * P[0] + P[1] * P[1] + P[2] * P[2] < 0.5) {
        continue;
      }
      edge_nbr[3 * f0 + e0] = static_cast<int32_t>(f1);
      edge_nbr[3 * f1 + e1] = static_cast<int32_t>(f0);
    }
  }
  // CSR of the per-cell face lists (faces ascending within each cell).
  std::vector<uint32_t> cell_start(static_cast<size_t>(C.total_cells) + 1, 0);
  for (uint32_t c = 0; c < C.total_cells; ++c) cell_start[c + 1] = cell_start[c] + cell_count[c];
  std::vector<uint32_t> cell_face(cell_pairs.size() > 0 ? cell_pairs.size() : 1);
  {
    std::vector<uint32_t> fill(cell_start.begin(), cell_start.end() - 1);
    for (const auto& [gc, gf] : cell_pairs) cell_face[fill[gc]++] = gf;
  }
  std::vector<uint32_t> row_start(static_cast<size_t>(total_rows) + 1, 0), row_edge;
  for (uint32_t y = 0; y < total_rows; ++y) {
    row_start[y + 1] = row_start[y] + static_cast<uint32_t>(row_lists[y].size());
    row_edge.insert(row_edge.end(), row_lists[y].begin(), row_lists[y].end());
  }
  if (row_edge.empty()) row_edge.push_back(0);
  if (edges.empty()) edges.assign(4, 0.0);
  if (cont_tri.empty()) cont_tri.assign(9, 0.0);
  if (cell_state.empty()) cell_state.assign(1, 1);
  tg::FaceArgs fa{};
  auto up = [&](auto*& dst, const auto& src) -> cudaError_t {
    using T = std::remove_const_t<std::remove_pointer_t<std::remove_reference_t<decltype(dst)>>>;
    void* p = nullptr;
    cudaError_t e = C.alloc(&p, sizeof(T) * src.size());
    if (e == cudaSuccess) {
      e = cudaMemcpyAsync(p, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, C.stream);
    }
    dst = static_cast<T*>(p);
    return e;
  };
  TG_CUDA(&C, up(fa.coords, coords));
  {
    // The frame of every face, once (the faces are fixed).
    const uint32_t nfaces = static_cast<uint32_t>(coords.size() / (D * D));
    const size_t per = D == 2 ? tg::kFrameDoubles<2> : tg::kFrameDoubles<3>;
    void* fr = nullptr;
    TG_CUDA(&C, C.alloc(&fr, sizeof(double) * per * std::max<uint32_t>(nfaces, 1)));
    fa.frame = static_cast<const double*>(fr);
    if (nfaces > 0) {
      const unsigned grid = (nfaces + 127) / 128;
      if (D == 2) {
        tg::k_face_frames<2><<<grid, 128, 0, C.stream>>>(fa.coords, static_cast<double*>(fr), nfaces);
      } else {
        tg::k_face_frames<3><<<grid, 128, 0, C.stream>>>(fa.coords, static_cast<double*>(fr), nfaces);
      }
      TG_CUDA(&C, cudaGetLastError());
    }
  }
  TG_CUDA(&C, up(fa.edge_nbr, edge_nbr));
  TG_CUDA(&C, up(fa.vert, vert));
  TG_CUDA(&C, up(fa.cell_start, cell_start));
  TG_CUDA(&C, up(fa.cell_face, cell_face));
  TG_CUDA(&C, up(fa.poly_edge, edges));
  TG_CUDA(&C, up(fa.row_start, row_start));
  TG_CUDA(&C, up(fa.row_edge, row_edge));
  TG_CUDA(&C, up(fa.row_off, row_off));
  TG_CUDA(&C, up(fa.tank_edges, tank_edges));
  TG_CUDA(&C, up(fa.cell_state, cell_state));
  TG_CUDA(&C, up(fa.cont_tri, cont_tri));
  TG_CUDA(&C, up(fa.cont_start, cont_start));
  const int64_t nn = C.n > 0 ? C.n : 1;
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.slot_of), sizeof(uint32_t) * nn));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.face_list), sizeof(uint32_t) * nn));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.face_count), sizeof(uint32_t)));
  TG_CUDA(&C, cudaMemsetAsync(fa.face_count, 0, sizeof(uint32_t), C.stream));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.gamma), sizeof(double) * nn));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.ggam), sizeof(double) * D * nn));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.face_drho), sizeof(double) * nn));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.face_dv), sizeof(double) * D * nn));
  TG_CUDA(&C, C.alloc(reinterpret_cast<void**>(&fa.post_face),
                      sizeof(double) * (2 * D + 2 * D * D) * nn));
  fa.weight = kernel_weight(C.P.kernel, D);
  fa.on = 1;
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  C.faces = fa;
  C.invalidate_graph();
  C.walls_fresh = false;
  return TG_OK;
}

}  // namespace

extern "C" {

int tg_tank_faces(tg_context* ctx, int32_t tank, int32_t n_faces,
                  const int32_t* face_verts, int32_t n_poly,
                  const double* poly) {
  if (ctx == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  const int D = C.P.dim;
  if (tank < 0 || tank >= C.ntanks || n_faces < 0) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "bad tank or face count");
  }
  const int32_t min_poly = D == 2 ? 3 : 4;
  if (n_faces > 0 && (face_verts == nullptr || n_poly < min_poly || poly == nullptr)) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT,
                D == 2 ? "faces need vertex pairs and a containment polygon"
                       : "faces need vertex triples and a containment mesh");
  }
  for (int32_t i = 0; i < D * n_faces; ++i) {
    if (face_verts[i] < 0 || face_verts[i] >= C.tanks[tank].n_wall) {
      return fail(&C, TG_ERR_INVALID_ARGUMENT,
                  "face vertex is not a fixed particle of the tank");
    }
  }
  // The containment: 2D a loop of n_poly vertices, 3D n_poly triangles.
  const size_t poly_doubles =
      n_faces > 0 ? (D == 2 ? 2 : 9) * static_cast<size_t>(n_poly) : 0;
  for (size_t i = 0; i < poly_doubles; ++i) {
    if (!std::isfinite(poly[i])) {
      return fail(&C, TG_ERR_INVALID_ARGUMENT, "non-finite containment surface");
    }
  }
  if (C.face_host.size() < static_cast<size_t>(C.ntanks)) C.face_host.resize(C.ntanks);
  auto& F = C.face_host[tank];
  F.face_verts.assign(face_verts, face_verts + D * static_cast<size_t>(n_faces));
  F.poly.assign(poly, poly + poly_doubles);
  return build_faces(ctx);
}

// ---- launch-shape tuning -----------------------------------------------
}  // extern "C"

namespace {

// Host copy of the whole particle state and the per-tank clocks, in upload
// order, so that trial steps can be undone.
struct Snapshot {
  std::vector<double> r, v, rho, dv, time, dt_last;
};

int take_snapshot(tg_context* ctx, Snapshot* S) {
  Context& C = ctx->c;
  const size_t n = static_cast<size_t>(C.n), d = static_cast<size_t>(C.P.dim);
  S->r.resize(n * d);
  S->v.resize(n * d);
  S->dv.resize(n * d);
  S->rho.resize(n);
  S->time.resize(static_cast<size_t>(C.ntanks));
  S->dt_last.resize(static_cast<size_t>(C.ntanks));
  int st = tg_particles_download(ctx, TG_FIELD_R, S->r.data());
  if (st == TG_OK) st = tg_particles_download(ctx, TG_FIELD_V, S->v.data());
  if (st == TG_OK) st = tg_particles_download(ctx, TG_FIELD_RHO, S->rho.data());
  if (st == TG_OK) st = tg_particles_download(ctx, TG_FIELD_DV_DT, S->dv.data());
  if (st != TG_OK) return st;
  TG_CUDA(&C, cudaMemcpy(S->time.data(), C.d_time, sizeof(double) * C.ntanks,
                         cudaMemcpyDeviceToHost));
  TG_CUDA(&C, cudaMemcpy(S->dt_last.data(), C.d_dt_last,
                         sizeof(double) * C.ntanks, cudaMemcpyDeviceToHost));
  return TG_OK;
}

// Put a snapshot back.  A new cells_per_radius re-grids the tanks (from the
// snapshot's positions) before the state goes back.
int restore_snapshot(tg_context* ctx, const Snapshot& S, int k) {
  Context& C = ctx->c;
  if (k != C.k) {
    const int old_k = C.k;
    C.k = k;
    C.P.cells_per_radius = k;
    const std::vector<tg_tank> tanks = C.tanks;
    int st = upload_particles(ctx, C.ntanks, tanks.data(), S.r.data(),
                              S.v.data(), S.rho.data());
    if (st != TG_OK) {
      // Back to the old grid (the same data fitted it before).
      C.k = old_k;
      C.P.cells_per_radius = old_k;
      const std::string why = C.last_error;
      upload_particles(ctx, C.ntanks, tanks.data(), S.r.data(), S.v.data(),
                       S.rho.data());
      build_faces(ctx);
      C.last_error = why;
      return st;
    }
    // The new grid needs new face tables.
    st = build_faces(ctx);
    if (st != TG_OK) return st;
  }
  const int st = tg_particles_update(ctx, S.r.data(), S.v.data(), S.rho.data(),
                                     S.dv.data());
  if (st != TG_OK) return st;
  TG_CUDA(&C, cudaMemcpyAsync(C.d_time, S.time.data(),
                              sizeof(double) * C.ntanks,
                              cudaMemcpyHostToDevice, C.stream));
  TG_CUDA(&C, cudaMemcpyAsync(C.d_dt_last, S.dt_last.data(),
                              sizeof(double) * C.ntanks,
                              cudaMemcpyHostToDevice, C.stream));
  TG_CUDA(&C, cudaStreamSynchronize(C.stream));
  return TG_OK;
}

bool valid_shape(const Context& C, const tg_tuning& t) {
  return t.cells_per_radius >= 1 && t.cells_per_radius <= 3 &&
         (t.block_size == 64 || t.block_size == 128 || t.block_size == 256) &&
         (t.lanes_per_particle == 1 || t.lanes_per_particle == 2 ||
          t.lanes_per_particle == 4) &&
         C.engine->supports_team(t.lanes_per_particle);
}

}  // namespace

extern "C" {

int tg_get_tuning(tg_context* ctx, tg_tuning* out) {
  if (ctx == nullptr || out == nullptr) return TG_ERR_INVALID_ARGUMENT;
  const Context& C = ctx->c;
  std::memset(out, 0, sizeof(*out));
  out->cells_per_radius = C.k;
  out->block_size = C.force_block;
  out->lanes_per_particle = C.force_team;
  out->ms_per_step = C.tuned_ms;
  out->candidates = C.tuned_candidates;
  return TG_OK;
}

int tg_set_tuning(tg_context* ctx, const tg_tuning* tuning) {
  if (ctx == nullptr || tuning == nullptr) return TG_ERR_INVALID_ARGUMENT;
  Context& C = ctx->c;
  if (!valid_shape(C, *tuning)) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT,
                "launch shape: cells_per_radius 1..3, block_size 64/128/256, "
                "lanes_per_particle 1/2/4 (2 and 4 for Wendland C2/C4 only)");
  }
  if (tuning->cells_per_radius != C.k) {
    if (C.uploaded && C.n > 0) {
      Snapshot S;
      int st = take_snapshot(ctx, &S);
      if (st == TG_OK) st = restore_snapshot(ctx, S, tuning->cells_per_radius);
      if (st != TG_OK) return st;
    } else {
      C.k = tuning->cells_per_radius;
      C.P.cells_per_radius = C.k;
    }
  }
  C.force_block = tuning->block_size;
  C.force_team = tuning->lanes_per_particle;
  C.invalidate_graph();
  return TG_OK;
}

int tg_autotune(tg_context* ctx, int32_t trial_steps, tg_tuning* out) {
  if (ctx == nullptr || trial_steps < 1 || trial_steps > 1000) {
    return TG_ERR_INVALID_ARGUMENT;
  }
  Context& C = ctx->c;
  if (!C.uploaded) return fail(&C, TG_ERR_NOT_READY, "no particles uploaded");
  if (C.n_fluid == 0) return fail(&C, TG_ERR_INVALID_ARGUMENT, "no fluid");
  Snapshot S;
  int st = take_snapshot(ctx, &S);
  if (st != TG_OK) return st;
  tg_tuning best{};
  tg_get_tuning(ctx, &best);
  best.ms_per_step = std::numeric_limits<double>::infinity();
  int timed = 0;
  // Time `trial_steps` graph-replayed steps of one shape (one untimed step
  // first captures the graph); the state goes back afterwards.
  auto trial = [&](tg_tuning t, double* ms) -> int {
    *ms = std::numeric_limits<double>::infinity();
    int s = restore_snapshot(ctx, S, t.cells_per_radius);
    if (s == TG_ERR_INVALID_ARGUMENT) return TG_OK;  // grid too large: skip
    if (s != TG_OK) return s;
    C.force_block = t.block_size;
    C.force_team = t.lanes_per_particle;
    C.invalidate_graph();
    s = tg_step(ctx, 1, nullptr);
    if (s == TG_OK) s = tg_timer_start(ctx);
    if (s == TG_OK) s = tg_step(ctx, trial_steps, nullptr);
    double total = 0.0;
    if (s == TG_OK) s = tg_timer_stop(ctx, &total);
    if (s != TG_OK) return s;
    *ms = total / trial_steps;
    ++timed;
    return TG_OK;
  };
  auto consider = [&](tg_tuning t) -> int {
    if (!valid_shape(C, t)) return TG_OK;
    double ms = 0.0;
    const int s = trial(t, &ms);
    if (s != TG_OK) return s;
    if (ms < best.ms_per_step) {
      best = t;
      best.ms_per_step = ms;
    }
    return TG_OK;
  };
  // Coordinate search: cell size, then lanes per target, then block size,
  // each with the others at their best so far.
  tg_tuning base = best;
  base.block_size = 128;
  base.lanes_per_particle = 1;
  for (int k = 1; k <= 3 && st == TG_OK; ++k) {
    tg_tuning t = base;
    t.cells_per_radius = k;
    st = consider(t);
  }
  for (int lanes : {2, 4}) {
    if (st != TG_OK) break;
    tg_tuning t = best;
    t.lanes_per_particle = lanes;
    st = consider(t);
  }
  for (int block : {64, 256}) {
    if (st != TG_OK) break;
    tg_tuning t = best;
    t.block_size = block;
    st = consider(t);
  }
  // Leave the context at the best shape with the state of the call.
  const int st2 = restore_snapshot(
      ctx, S, std::isfinite(best.ms_per_step) ? best.cells_per_radius : C.k);
  if (st != TG_OK) return st;
  if (st2 != TG_OK) return st2;
  if (!std::isfinite(best.ms_per_step)) {
    return fail(&C, TG_ERR_INVALID_ARGUMENT, "no launch shape fits");
  }
  C.force_block = best.block_size;
  C.force_team = best.lanes_per_particle;
  C.invalidate_graph();
  C.tuned_ms = best.ms_per_step;
  C.tuned_candidates = timed;
  best.candidates = timed;
  if (out != nullptr) *out = best;
  return TG_OK;
}

int tg_host_alloc(size_t bytes, void** out) {
  if (out == nullptr) return TG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const cudaError_t e = cudaMallocHost(out, bytes > 0 ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? TG_ERR_OUT_OF_MEMORY : TG_ERR_CUDA;
  }
  return TG_OK;
}

int tg_host_free(void* ptr) {
  if (ptr != nullptr) cudaFreeHost(ptr);
  return TG_OK;
}

}  // extern "C"
