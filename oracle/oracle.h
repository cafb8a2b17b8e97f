/*
 * oracle.h - CPU restatement of TitSolver's WCSPH hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU path and
 * the timed CPU baseline; only the tests, the smoke check and the benchmark's
 * CPU-baseline leg may load it.  The product path never calls it.
 *
 * The reference (C++26, GCC 16, vcpkg) cannot be compiled on this toolchain
 * (g++ 13, no network), so this is a C++20 restatement of the reference's
 * files, each function citing the file:line it follows.  It is compiled
 * IEEE-strict (-O3 -ffp-contract=off, no fast-math).  It is pinned against
 * the reference's own unit tests for this path (kernel normalisation and
 * derivative checks of source/tit/sph/kernel.test.cpp, naive-vs-grid search
 * of source/tit/geom/search.test.cpp) re-expressed in tests/; the fluid step
 * itself has no reference test or golden vector (the titwcsph checksum is
 * platform specific), so step parity beyond the restatement is unpinned.
 */
#ifndef TITGPU_ORACLE_H
#define TITGPU_ORACLE_H

#include <stdint.h>

#include "../include/titgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel support radius (units of h) and normalisation weight for Dim. */
void or_kernel_info(int32_t kernel, int32_t dim, double* unit_radius,
                    double* weight);
/* W(x, h) and grad W(x, h) (kernel.hpp:142-163). */
double or_kernel_value(int32_t kernel, int32_t dim, const double* x, double h);
void or_kernel_grad(int32_t kernel, int32_t dim, const double* x, double h,
                    double* out);
/* Unit polynomial value and derivative at q. */
double or_kernel_unit_value(int32_t kernel, double q);
double or_kernel_unit_deriv(int32_t kernel, double q);

/* Tait EOS (equation_of_state.hpp:37-64). */
/* Pressure, sound speed, potential H(rho) and rho(H(rho)) of equation of
 * state eos (TG_EOS_TAIT or TG_EOS_LINEAR_TAIT). */
void or_eos(int32_t eos, double rho, double rho0, double cs0, double xi,
            double* p, double* cs, double* potential, double* rho_back);
void or_tait(double rho, double rho0, double cs0, double xi, double* p,
             double* cs, double* potential);
double or_tait_density_from_potential(double H, double rho0, double cs0,
                                      double xi);

/* splitmix64, used for order-independent neighbour-set hashes. */
uint64_t or_splitmix64(uint64_t x);

/* Grid neighbour search (GridIndex, grid_search.hpp:45-102) with the
 * inclusive sphere predicate; rows sorted ascending, self included.
 * Returns the total number of entries; fills offsets (n + 1) always and
 * indices only if capacity suffices. */
int64_t or_grid_search(int32_t dim, int64_t n, const double* r, double radius,
                       double size_hint, int64_t* offsets, int32_t* indices,
                       int64_t capacity, int32_t nthreads);
/* The same with FP32 positions and FP32 predicate arithmetic. */
int64_t or_grid_search_f32(int32_t dim, int64_t n, const float* r,
                           float radius, float size_hint, int64_t* offsets,
                           int32_t* indices, int64_t capacity,
                           int32_t nthreads);
/* Naive O(N^2) search of search.test.cpp:40-55; inclusive selects <= or <. */
int64_t or_naive_search(int32_t dim, int64_t n, const double* r,
                        double radius, int32_t inclusive, int64_t* offsets,
                        int32_t* indices, int64_t capacity);

/* Uniform points in the unit box from std::mt19937{seed} and
 * std::uniform_real_distribution{0.0, 1.0}, as search.test.cpp:131-155. */
void or_mt19937_uniform_points(uint32_t seed, int64_t count, double* out);

/* Summation density rho_a = sum_b m W_ab (fluid_equations.hpp:498-502),
 * self included, with counts and hashes.  pos_precision selects FP64 or
 * FP32 (predicate, kernel and sum in float). */
int32_t or_summation_density(int32_t dim, int32_t kernel,
                             int32_t pos_precision, int64_t n,
                             const double* r, double h, double m,
                             double* rho, int32_t* counts, uint64_t* hashes,
                             int32_t nthreads);

/* n_steps integrator steps of FluidEquations with particle walls
 * (fluid_equations.hpp:79-321, time_integrator.hpp:31-228), in place.
 * Arrays are in upload order (see titgpu.h).  dt_out gets each tank's last
 * dt; time_io (may be NULL) is advanced by the dts. */
int32_t or_wcsph_step(const tg_params* params, int32_t n_tanks,
                      const tg_tank* tanks, double* r, double* v, double* rho,
                      double* drho_dt, double* dv_dt, int32_t n_steps,
                      double* dt_out, double* time_io, int32_t nthreads);

/* Boundary faces of one tank (semi-analytical walls): n_faces faces as dim
 * indices each into the tank's fixed particles (the face vertices; segments
 * in 2D, triangles in 3D), and the containment surface: in 2D a closed loop
 * of n_poly vertices (x, y), in 3D n_poly triangles (9 doubles each) of a
 * closed mesh with outward normals.  A point is inside when the surface's
 * winding number around it exceeds 1/2.  n_faces = 0: particle walls. */
typedef struct or_tank_faces {
  int32_t n_faces;
  const int32_t* face_verts;
  int32_t n_poly;
  const double* poly;
} or_tank_faces;

/* or_wcsph_step with per-tank boundary faces (faces may be NULL). */
int32_t or_wcsph_step_faces(const tg_params* params, int32_t n_tanks,
                            const tg_tank* tanks, double* r, double* v,
                            double* rho, double* drho_dt, double* dv_dt,
                            int32_t n_steps, double* dt_out, double* time_io,
                            int32_t nthreads, const or_tank_faces* faces);

/* Kernel flux (2 components) and antigradient flux of segment a-b at x with
 * width h (kernel.hpp:194-221), and the polygon winding number at x. */
void or_kernel_flux2(int32_t kernel, const double* a, const double* b,
                     const double* x, double h, double* out);
double or_kernel_antigrad_flux2(int32_t kernel, const double* a,
                                const double* b, const double* x, double h);
double or_winding_number2(int32_t n_poly, const double* poly, const double* x);

/* Kernel flux (3 components) and antigradient flux of triangle a-b-c at x
 * with width h, the triangle mesh winding number at x, and the
 * triangle-sphere overlap test of the face adjacency. */
void or_kernel_flux3(int32_t kernel, const double* a, const double* b,
                     const double* c, const double* x, double h, double* out);
double or_kernel_antigrad_flux3(int32_t kernel, const double* a,
                                const double* b, const double* c,
                                const double* x, double h);
double or_winding_number3(int32_t n_tris, const double* tris, const double* x);
int32_t or_triangle_in_sphere(const double* a, const double* b, const double* c,
                              const double* x, double radius);
/* Triangle::clamp (closest point, 3 doubles) and Triangle::project (the
 * vertices in the plane frame around origin, 6 doubles). */
void or_triangle_clamp(const double* a, const double* b, const double* c,
                       const double* x, double* out);
void or_triangle_project(const double* a, const double* b, const double* c,
                         const double* origin, double* out);

/* Neighbour counts and hashes of every particle in its tank (tank-local ids),
 * via or_grid_search with radius = unit_radius * h. */
int32_t or_tank_neighbour_counts(const tg_params* params, int32_t n_tanks,
                                 const tg_tank* tanks, const double* r,
                                 int32_t* counts, uint64_t* hashes,
                                 int32_t nthreads);

#ifdef __cplusplus
}
#endif

#endif /* TITGPU_ORACLE_H */
