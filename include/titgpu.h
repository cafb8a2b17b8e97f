/*
 * titgpu.h - C ABI of the GB300 WCSPH hot path (neighbour search, fused
 * kernel sums and the SSPRK step) of TitSolver.
 *
 * TitSolver exposes this path only as header-only C++26 templates with closed
 * concepts; there is no plugin or FFI layer to bind.  The entry points below
 * replace, one for one, the calls a titwcsph-style driver makes:
 *
 *   tg_context_create     FluidEquations{g, mu, domain, containment,
 *                         TaitEquationOfState{cs_0, rho_0}, Kernel{}}
 *                         (source/tit/sph/fluid_equations.hpp:61-69) together
 *                         with SSPRKIntegrator{equations, order}
 *                         (source/tit/sph/time_integrator.hpp:153-156) and
 *                         ParticleMesh{GridSearch{h_0}, ...}
 *                         (source/tit/sph/particle_mesh.hpp:53-61)
 *   tg_particles_upload   ParticleArray::append + r[a] = ..., h[particles] =,
 *                         m[a] =, rho[a] = (source/tit/sph/particle_array.hpp
 *                         :188-199; source/titwcsph/wcsph.cpp:104-142) and
 *                         FluidEquations::initialize (fluid_equations.hpp:79-89)
 *   tg_step               dt = SSPRKIntegrator::step(mesh, particles)
 *                         (time_integrator.hpp:161-185), repeated n times
 *   tg_particles_download field[particles] reads used by ParticleArray::write
 *                         (particle_array.hpp:165-172)
 *   tg_neighbour_*        ParticleMesh adjacency (particle_mesh.hpp:123-147):
 *                         sorted lists, self included, inclusive predicate
 *   tg_summation_density  the summation density sum_b m_b W_ab of
 *                         fluid_equations.hpp:498-502 over a point cloud
 *
 * Conventions: every function returns an int status (TG_OK = 0, else a
 * TG_ERR_* code); no C++ exception crosses the boundary.  One context owns one
 * CUDA stream on the device that was current when it was created; calls on a
 * context must come from one host thread at a time.  Particle arrays are in
 * upload order: tank after tank, each tank its fluid particles first and its
 * fixed (wall) particles after them (the fluid-then-fixed ranges of
 * particle_array.hpp:211-228).  Vectors are stored AoS (x, y[, z]) per
 * particle, as std::vector<Vec<Real, Dim>> stores them.
 */
#ifndef TITGPU_H
#define TITGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  TG_OK = 0,
  TG_ERR_INVALID_ARGUMENT = 1, /* bad size, mode or pointer */
  TG_ERR_CUDA = 2,             /* a CUDA runtime call failed */
  TG_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed */
  TG_ERR_NOT_READY = 4,        /* no particles uploaded yet */
  TG_ERR_DEVICE_STATE = 5,     /* a kernel raised the device error word */
  TG_ERR_CAPACITY = 6,         /* output buffer too small */
  TG_ERR_NO_DEVICE = 7         /* no CUDA device visible */
};

/* Device error word bits (tg_device_status). */
enum {
  TG_DEV_NONFINITE_STATE = 1u << 0, /* NaN/Inf position, velocity or density */
  TG_DEV_OUTSIDE_GRID = 1u << 1,    /* particle clamped into the border cells */
  TG_DEV_BAD_DT = 1u << 2,          /* non-positive or non-finite time step */
  TG_DEV_COPY_TIMEOUT = 1u << 3     /* a bulk copy into shared memory did not
                                       complete within its wait limit (the
                                       pass read global memory instead) */
};

/* ---- enumerations ------------------------------------------------------ */
/* Arithmetic form of the pair sums. */
enum { TG_FP64 = 0, TG_FP32C = 1 };
/* Position precision of a point cloud (tg_summation_density). */
enum { TG_POS_FP64 = 0, TG_POS_FP32 = 1 };
/* Smoothing kernels, the closed set of source/tit/sph/kernel.hpp:459-465. */
enum {
  TG_KERNEL_CUBIC_SPLINE = 0,
  TG_KERNEL_QUARTIC_SPLINE = 1,
  TG_KERNEL_QUINTIC_SPLINE = 2,
  TG_KERNEL_WENDLAND_C2 = 3, /* QuarticWendlandKernel */
  TG_KERNEL_WENDLAND_C4 = 4, /* SixthOrderWendlandKernel */
  TG_KERNEL_WENDLAND_C6 = 5  /* EighthOrderWendlandKernel */
};
/* Time integrators (source/tit/sph/time_integrator.hpp). */
enum {
  TG_SSPRK3 = 0,  /* SSPRKIntegrator{eq, SSPRKOrder::three} :140-228 */
  TG_SSPRK2 = 1,  /* SSPRKIntegrator{eq, SSPRKOrder::two} */
  TG_EULER = 2,   /* SymplecticEulerIntegrator :31-75 */
  TG_VERLET = 3   /* VelocityVerletIntegrator :80-129 */
};
/* Viscosity term of the momentum sum. */
enum {
  TG_VISC_MORRIS = 0,  /* laminar mu, fluid_equations.hpp:299-300 */
  TG_VISC_MONAGHAN = 1 /* artificial alpha (Monaghan 1992) */
};
/* Density diffusion term of the continuity sum. */
enum {
  TG_DIFF_FERRARI = 0, /* fluid_equations.hpp:253-258 */
  TG_DIFF_MOLTENI = 1, /* delta-SPH (Molteni & Colagrossi 2009) */
  TG_DIFF_NONE = 2
};
/* Post-integration stage (fluid_equations.hpp:315-321). */
enum {
  TG_POST_PREPARE = 0, /* refresh mesh and wall state only (the next step's
                          prepare does this anyway: no extra pass) */
  TG_POST_SHIFTING = 1 /* + apply_shifts + free-surface density correction
                          (fluid_equations.hpp:331-512): one more search,
                          wall extrapolation and five passes per step */
};
/* Fields for tg_particles_download (names of source/tit/sph/field.hpp). */
enum {
  TG_FIELD_R = 0,       /* Dim doubles per particle */
  TG_FIELD_V = 1,       /* Dim */
  TG_FIELD_RHO = 2,     /* 1 */
  TG_FIELD_DRHO_DT = 3, /* 1 */
  TG_FIELD_DV_DT = 4,   /* Dim */
  TG_FIELD_P = 5,       /* 1, Tait pressure of the downloaded rho */
  TG_FIELD_CS = 6       /* 1, sound speed of the downloaded rho */
};

/* Equation of state (the closed set of equation_of_state.hpp:127-129). */
enum {
  TG_EOS_TAIT = 0,       /* TaitEquationOfState (equation_of_state.hpp:19-72):
                            p = rho0 cs0^2/xi ((rho/rho0)^xi - 1) */
  TG_EOS_LINEAR_TAIT = 1 /* LinearTaitEquationOfState (:78-122):
                            p = cs0^2 (rho - rho0), c = cs0; xi unused */
};

/* ---- parameter blocks -------------------------------------------------- */
/* Global physics and numerics.  tg_params_default() fills the reference's
 * values: SixthOrderWendlandKernel (wcsph.cpp:89), xi = 7
 * (equation_of_state.hpp:29), g = 9.81 and mu = 0.001 (wcsph.cpp:47,52),
 * Morris viscosity, Ferrari diffusion, CFL 0.4, C_force 0.25, C_visc 0.125
 * (fluid_equations.hpp:518-520), SSPRK3, post-integration with shifting and
 * the free-surface correction (FluidEquations::post_integrate always runs
 * them, fluid_equations.hpp:315-321), FP64. */
typedef struct tg_params {
  int32_t dim;              /* 2 or 3 */
  int32_t precision;        /* TG_FP64 | TG_FP32C */
  int32_t kernel;           /* TG_KERNEL_* */
  int32_t integrator;       /* TG_SSPRK3 | TG_SSPRK2 | TG_EULER | TG_VERLET */
  int32_t viscosity;        /* TG_VISC_* */
  int32_t diffusion;        /* TG_DIFF_* */
  int32_t post_integrate;   /* TG_POST_* */
  int32_t cells_per_radius; /* grid cells per support radius, 1..3 */
  int32_t kahan;            /* FP32C: 1 = compensated sums, 0 = plain */
  int32_t device;           /* CUDA device ordinal; -1 = the current one */
  int32_t staging;          /* 2D FP32C: copy each block's neighbour
                               window into shared memory with bulk copies
                               (1) or read it through L1 (0, default;
                               measured faster on GB300) */
  int32_t eos;              /* TG_EOS_TAIT (default) | TG_EOS_LINEAR_TAIT */
  int32_t face_fp32;        /* TG_FP32C with face walls: the closed-form face
                               integrals in FP32 (1) or FP64 (0, default).
                               FP32 runs the face passes ~1.7x faster in 3D
                               at a larger drift from the FP64 form; must be
                               0 with TG_FP64. */
  int32_t resort;           /* 1 (default): between stages, re-sort only the
                               particles whose cell changed and merge them
                               into the previous order; 0: a full radix sort
                               every stage.  Same order either way. */
  double xi;      /* Tait polytropic index */
  double g;       /* gravity, acting along -axis 1 */
  double mu;      /* Morris dynamic viscosity */
  double alpha;   /* Monaghan artificial viscosity */
  double delta;   /* delta-SPH coefficient */
  double cfl;     /* acoustic CFL number */
  double c_force; /* force time step coefficient */
  double c_visc;  /* viscous time step coefficient */
} tg_params;

/* One independent tank (one ParticleArray of the reference). */
typedef struct tg_tank {
  int64_t n_fluid; /* fluid particles, first in the tank's block */
  int64_t n_wall;  /* fixed particles, after the fluid */
  double h;        /* kernel width, uniform in the tank */
  double m;        /* particle mass, uniform in the tank */
  double rho0;     /* Tait reference density */
  double cs0;      /* Tait reference sound speed */
} tg_tank;

/* Accumulated device time per kernel group, in milliseconds. */
typedef struct tg_profile {
  double sort_ms;    /* cell keys, radix sort, cell table */
  double reorder_ms; /* gather into cell order, dt reduction */
  double walls_ms;   /* wall state extrapolation */
  double forces_ms;  /* fused continuity + momentum + RK update */
  double post_ms;    /* post-integration passes */
  int64_t forces_launches;
  int64_t stages;
  int64_t steps;
} tg_profile;

typedef struct tg_context tg_context;

/* ---- entry points ------------------------------------------------------ */
/* Defaults as described at tg_params.  Never fails. */
void tg_params_default(tg_params* params);

/* Create a context on the current CUDA device (see header comment). */
int tg_context_create(const tg_params* params, tg_context** out);
/* Destroy a context and release its device memory.  NULL is a no-op. */
int tg_context_destroy(tg_context* ctx);

/* Upload particles of n_tanks tanks.  r and v hold Dim doubles per particle,
 * rho one.  Replaces any previous particles; sets per-tank time to zero. */
int tg_particles_upload(tg_context* ctx, int32_t n_tanks, const tg_tank* tanks,
                        const double* r, const double* v, const double* rho);

/* Replace the state of the uploaded particles (same tanks and counts) with
 * new host values: r, v (Dim doubles per particle), rho, and optionally
 * dv_dt (NULL resets it to zero; it feeds the force time step).  The cell
 * grids of the tanks are kept.  This is the per-step host->device sync of a
 * driver that keeps its ParticleArray on the host.  Page-locked arrays
 * (tg_host_alloc, cudaHostAlloc, registered) are read by the device
 * directly, others are staged; the arrays may be reused when it returns. */
int tg_particles_update(tg_context* ctx, const double* r, const double* v,
                        const double* rho, const double* dv_dt);

/* FluidEquations::prepare (fluid_equations.hpp:99-105): rebuild the
 * neighbour search and extrapolate the wall state at the current positions.
 * Downloads of rho, p and cs run it on their own when positions changed. */
int tg_prepare(tg_context* ctx);

/* Advance every tank by n_steps integrator steps (each with its own dt).
 * dt_out (n_tanks doubles, may be NULL) receives the last step's dt. */
int tg_step(tg_context* ctx, int32_t n_steps, double* dt_out);

/* Per-tank accumulated time (n_tanks doubles). */
int tg_time(tg_context* ctx, double* time_out);

/* Copy a field into out, in upload order. */
int tg_particles_download(tg_context* ctx, int32_t field, double* out);

/* Copy the state fields r, v (n x dim), rho, drho/dt (n) and dv/dt
 * (n x dim) in upload order, each skipped when NULL: one pass over the
 * device state, the copies issued back to back, one wait.  Replaces the
 * per-field reads of ParticleArray after a step (particle_array.hpp:165-172,
 * field.hpp:172-218) in a host loop that reads the whole state. */
int tg_particles_download_state(tg_context* ctx, double* r, double* v,
                                double* rho, double* drho_dt, double* dv_dt);

/* Neighbour count and order-independent hash (sum of splitmix64(id + 1))
 * of every particle's neighbour set at the current positions: all particles
 * of its tank within 2h, inclusive, self included.  In upload order. */
int tg_neighbour_counts(tg_context* ctx, int32_t* counts, uint64_t* hashes);

/* Full neighbour lists as CSR: offsets (n + 1), indices (capacity), each row
 * sorted ascending, ids in upload order and tank-local (as in the
 * reference's per-ParticleArray adjacency).  Fails with TG_ERR_CAPACITY and
 * writes the needed size to offsets[n] when capacity is short. */
int tg_neighbour_lists(tg_context* ctx, int64_t* offsets, int32_t* indices,
                       int64_t capacity);

/* Summation density rho_a = sum_b m W_ab over the uploaded particles (all
 * treated alike, self included), with neighbour counts and hashes.  The
 * position precision selects FP64 or FP32 predicate and arithmetic.
 * Any output pointer may be NULL. */
int tg_summation_density(tg_context* ctx, int32_t pos_precision,
                         double* rho_out, int32_t* counts, uint64_t* hashes);

/* Device-resident variant for timing: runs the search + summation pass on
 * the context's resident particles and leaves results on the device. */
int tg_summation_density_resident(tg_context* ctx, int32_t pos_precision);

/* Read and clear the device error word (TG_DEV_* bits). */
int tg_device_status(tg_context* ctx, uint32_t* flags);

/* Kernel-group timing with CUDA events on the context stream. */
int tg_profile_enable(tg_context* ctx, int32_t enable);
int tg_profile_read(tg_context* ctx, tg_profile* out);

/* Capture the step in a CUDA graph and replay it (1) or launch kernels
 * directly (0).  Default 1. */
int tg_set_graph(tg_context* ctx, int32_t enable);

/* Number of kernel launches issued since context creation. */
int tg_launch_count(tg_context* ctx, int64_t* count);

/* Synchronise the context stream. */
int tg_synchronize(tg_context* ctx);

/* CUDA-event timer on the context stream: start, then stop returns the
 * elapsed device time in milliseconds (stop synchronises). */
int tg_timer_start(tg_context* ctx);
int tg_timer_stop(tg_context* ctx, double* ms);

/* Page-locked host memory for fast uploads and downloads. */
int tg_host_alloc(size_t bytes, void** out);
int tg_host_free(void* ptr);

/* Summation density of a point cloud that allocates nothing.  No
 * counterpart in the reference: it serves callers that may not allocate
 * device memory (a host framework that owns all device memory and forbids
 * allocation inside its callbacks, or a real-time loop that must not block
 * in the allocator).  Inputs and outputs are caller-owned DEVICE pointers:
 * r (n x dim doubles, AoS), rho (n doubles), counts (n int32), hashes
 * (n uint64); any output may be NULL but not all.  The result equals
 * tg_summation_density with TG_POS_FP64 on the same points (all particles
 * alike, self included, inclusive 2h predicate).
 *
 * Scratch is a fixed file-scope device array of 4,495,616 bytes (about
 * 4.5 MB) that every GPU loading this library holds until exit; n above
 * TG_NOALLOC_MAX_POINTS returns TG_ERR_CAPACITY.  Work is enqueued on
 * `stream` (NULL = legacy
 * default stream) without synchronising; results are ready when the stream
 * reaches that point.  The first call on a device looks up the scratch
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept for
 * the life of the process: resetting a device (cudaDeviceReset, or a reset
 * of its primary context) after the first call on it is not supported, as
 * the reloaded module may place the array elsewhere.  Every call shares the one
 * array, which keeps the last call's contents (each call rewrites all it
 * reads), so calls that overlap on the GPU (different streams or threads
 * without ordering) race and corrupt each other. */
#define TG_NOALLOC_MAX_POINTS 65536
int tg_summation_density_noalloc(int32_t dim, int32_t kernel, int64_t n,
                                 const double* r, double h, double m,
                                 double* rho, int32_t* counts, uint64_t* hashes,
                                 void* stream);

/* ---- boundary faces ------------------------------------------------------ */
/* The reference's semi-analytical wall mode for one tank: FluidEquations
 * with a non-empty domain surface and a containment function
 * (fluid_equations.hpp:122-193 gamma, grad gamma and the wall extrapolation
 * with the wall normal; :241-247 and :276-292 the face terms of continuity
 * and momentum; :335-349, :465-467, :491-511 the face terms of shifting and
 * the free-surface correction; kernel.hpp:194-221 the kernel flux and
 * antigradient flux of a face).  Segments in 2D, triangles in 3D; both
 * arithmetic forms (the face sums run in FP64 either way).
 *
 * face_verts: dim per face, indices into the tank's fixed particles (0 = the
 * tank's first fixed particle), which are the face vertices and stay fixed
 * (titwcsph appends one fixed particle per vertex of the tessellated
 * domain, wcsph.cpp:109-112).  A face's normal, normalize(cross(b - a)) in
 * 2D and normalize(cross(b - a, c - a)) in 3D, points into the fluid.
 * poly: the containment surface; in 2D n_poly (x, y) vertices of a closed
 * loop, in 3D n_poly triangles (9 doubles each: a, b, c) of a closed mesh
 * with outward normals.  A point is inside when the surface's winding number
 * around it exceeds 1/2 (the reference passes a FastWinding of the domain,
 * fast_winding.hpp:80-95).  In 3D every particle near the surface evaluates
 * the exact winding number over all n_poly triangles, so a coarse
 * containment mesh (as titwcsph's separate containment domain) keeps that
 * cheap.  n_faces = 0 returns the tank to particle walls.  Call after
 * tg_particles_upload (a new upload drops the faces); applies to the
 * following steps. */
int tg_tank_faces(tg_context* ctx, int32_t tank, int32_t n_faces,
                  const int32_t* face_verts, int32_t n_poly,
                  const double* poly);

/* ---- launch shape and the autotuner ----------------------------------- */
/* Launch shape of a context: the grid's cell size (cells_per_radius cells
 * across the kernel support radius, as GridSearch{spacing} picks the cell
 * size in source/tit/geom/search/grid_search.hpp:73-113), the force pass's
 * threads per block, and its lanes per fluid particle (1, 2 or 4: the lanes
 * split the particle's neighbour cells, so a warp advances 32, 16 or 8
 * particles; 2 and 4 exist for the Wendland C2 and C4 kernels). */
typedef struct tg_tuning {
  int32_t cells_per_radius;   /* 1..3 */
  int32_t block_size;         /* 64, 128 or 256 */
  int32_t lanes_per_particle; /* 1, 2 or 4 */
  int32_t candidates;         /* shapes timed by the last tg_autotune */
  double ms_per_step;         /* device ms per step of the tuned shape
                                 (0 before any tg_autotune) */
} tg_tuning;

/* Current launch shape. */
int tg_get_tuning(tg_context* ctx, tg_tuning* out);
/* Set the launch shape.  A new cells_per_radius re-grids the tanks from the
 * current positions and keeps the particle state and clocks. */
int tg_set_tuning(tg_context* ctx, const tg_tuning* tuning);
/* Autotuner (no reference counterpart; the reference fixes its grid cell
 * size in the driver): times trial_steps steps of each candidate shape on
 * the uploaded particles, by coordinate search over cells_per_radius, then
 * lanes_per_particle, then block_size, and leaves the context at the
 * fastest shape with the particle state and clocks of the call (the trial
 * steps are undone).  out (may be NULL) receives the choice. */
int tg_autotune(tg_context* ctx, int32_t trial_steps, tg_tuning* out);

/* Human-readable text of a status code, and of the context's last error. */
const char* tg_status_string(int status);
const char* tg_last_error(tg_context* ctx);

#ifdef __cplusplus
}
#endif

#endif /* TITGPU_H */
