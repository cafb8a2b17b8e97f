/*
 * titgpu.hpp - C++20 host mirror of TitSolver's particle-array,
 * fluid-equation and time-integrator API, driving the GB300 path through the
 * C ABI of titgpu.h.
 *
 * The reference API is header-only C++26 with closed concepts
 * (source/tit/sph/particle_mesh.hpp:263-264, time_integrator.hpp:25-26), so a
 * GPU backend cannot be plugged into it; this header restates the names and
 * call shapes a titwcsph-style driver uses instead:
 *
 *   ParticleArray{Space<Real, Dim>{}, integrator}   particle_array.hpp:160-162
 *   particles.append(ParticleType::fluid|fixed)     particle_array.hpp:188-199
 *   r[a] = ..., m[a] = ..., rho[a] = ..., h[particles] = h_0
 *                                                   field.hpp:172-218
 *   particles.all() / fluid() / fixed()             particle_array.hpp:203-228
 *   TaitEquationOfState{cs_0, rho_0[, xi]}          equation_of_state.hpp:19-72
 *   LinearTaitEquationOfState{cs_0, rho_0}          equation_of_state.hpp:78-122
 *   FluidEquations{g, mu, domain, containment, eos, kernel}
 *                                                   fluid_equations.hpp:61-69
 *   SSPRKIntegrator{equations, SSPRKOrder::three}   time_integrator.hpp:153-156
 *   SymplecticEulerIntegrator{equations}            time_integrator.hpp:31-75
 *   VelocityVerletIntegrator{equations}             time_integrator.hpp:80-129
 *   ParticleMesh{geom::GridSearch{h_0}, ...}        particle_mesh.hpp:53-61
 *   equations.initialize(mesh, particles)           fluid_equations.hpp:79-89
 *   dt = integrator.step(mesh, particles)           time_integrator.hpp:161-185
 *
 * The particle state lives on the GPU once initialize() has run.  Host field
 * access after a step downloads the state first; a host write is uploaded
 * (tg_particles_update) before the next step.  Errors throw tit::Exception,
 * as TIT_ENSURE does (source/tit/core/exception.hpp:81).
 *
 * Walls: either fixed particles with an empty domain surface ("particle
 * walls": gamma = 1 and no face terms, fluid_equations.hpp:122-163), or
 * the reference's semi-analytical face walls: a tessellated domain surface
 * (segments in 2D, triangles in 3D) whose vertices are the fixed particles
 * and a winding-number containment (geom::MakeFastWinding), as titwcsph
 * sets up (wcsph.cpp:55-77, 109-112).  Every fluid particle must lie inside
 * the containment.
 *
 * GPU-only choices (precision form, the textbook term set, CFL constants)
 * come in an optional trailing sph::GpuOptions argument of FluidEquations.
 */
#ifndef TITGPU_HPP
#define TITGPU_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <ranges>
#include <span>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "titgpu.h"

namespace tit {

/// Error thrown for every failed call (the role of tit::Exception).
class Exception : public std::runtime_error {
public:
  using std::runtime_error::runtime_error;
};

namespace gpu_detail {
inline void ensure(int status, tg_context* ctx, const char* what) {
  if (status == TG_OK) return;
  std::string msg = std::string{what} + " failed: " + tg_status_string(status);
  if (ctx != nullptr) {
    const char* why = tg_last_error(ctx);
    if (why != nullptr && *why != '\0') msg += " (" + std::string{why} + ")";
  }
  throw Exception{msg};
}
} // namespace gpu_detail

template<class T>
constexpr auto pow2(T x) noexcept -> T {
  return x * x;
}

/// Small fixed-size vector with the arithmetic a driver writes.
template<class Real, std::size_t Dim>
class Vec {
public:
  constexpr Vec() noexcept = default;
  template<class... Args>
    requires(sizeof...(Args) == Dim && Dim > 1)
  constexpr Vec(Args... args) noexcept : c_{static_cast<Real>(args)...} {}

  constexpr auto operator[](std::size_t i) noexcept -> Real& { return c_[i]; }
  constexpr auto operator[](std::size_t i) const noexcept -> const Real& {
    return c_[i];
  }
  static constexpr auto dim() noexcept -> std::size_t { return Dim; }

  constexpr auto operator+=(const Vec& o) noexcept -> Vec& {
    for (std::size_t i = 0; i < Dim; ++i) c_[i] += o.c_[i];
    return *this;
  }
  constexpr auto operator-=(const Vec& o) noexcept -> Vec& {
    for (std::size_t i = 0; i < Dim; ++i) c_[i] -= o.c_[i];
    return *this;
  }
  constexpr auto operator*=(Real s) noexcept -> Vec& {
    for (auto& x : c_) x *= s;
    return *this;
  }
  friend constexpr auto operator+(Vec a, const Vec& b) noexcept -> Vec {
    return a += b;
  }
  friend constexpr auto operator-(Vec a, const Vec& b) noexcept -> Vec {
    return a -= b;
  }
  friend constexpr auto operator*(Real s, Vec a) noexcept -> Vec {
    return a *= s;
  }
  friend constexpr auto operator*(Vec a, Real s) noexcept -> Vec {
    return a *= s;
  }
  friend constexpr auto operator/(Vec a, Real s) noexcept -> Vec {
    for (auto& x : a.c_) x /= s;
    return a;
  }
  friend constexpr auto operator==(const Vec&, const Vec&) noexcept
      -> bool = default;

private:
  std::array<Real, Dim> c_{};
};

template<class T, class... U>
Vec(T, U...) -> Vec<std::common_type_t<T, U...>, 1 + sizeof...(U)>;

namespace geom {

/// Boundary surface (source/tit/geom/surface.hpp): vertices and faces
/// (segments in 2D, triangles in 3D).  An empty surface means particle
/// walls; a surface with faces selects the semi-analytical wall mode, whose
/// fixed particles are the surface's vertices in order (wcsph.cpp:109-112).
template<class V>
class Surface {
public:
  auto append_vert(const V& v) -> std::size_t {
    verts_.push_back(v);
    return verts_.size() - 1;
  }
  void append_face(std::array<std::size_t, V::dim()> face) {
    faces_.push_back(face);
  }
  auto num_verts() const noexcept -> std::size_t { return verts_.size(); }
  auto num_faces() const noexcept -> std::size_t { return faces_.size(); }
  auto vert(std::size_t i) const -> const V& { return verts_.at(i); }
  auto face_verts(std::size_t i) const -> const std::array<std::size_t, V::dim()>& {
    return faces_.at(i);
  }

private:
  std::vector<V> verts_;
  std::vector<std::array<std::size_t, V::dim()>> faces_;
};

/// Split every face into max(1, ceil(length / d_max)) segments: the
/// original vertices first, then each face's new vertices in order
/// (source/tit/geom/tessellation.hpp:30-60).
template<class V>
  requires (V::dim() == 2)
auto tessellate(const Surface<V>& surf, double d_max) -> Surface<V> {
  if (!(d_max > 0.0)) throw Exception{"tessellate: d_max <= 0"};
  Surface<V> out;
  for (std::size_t i = 0; i < surf.num_verts(); ++i) out.append_vert(surf.vert(i));
  using Num = std::remove_cvref_t<decltype(surf.vert(0)[0])>;
  for (std::size_t fi = 0; fi < surf.num_faces(); ++fi) {
    const auto [ia, ib] = surf.face_verts(fi);
    const V a = surf.vert(ia), b = surf.vert(ib);
    const V ba = b - a;
    const double len = std::sqrt(static_cast<double>(ba[0] * ba[0] + ba[1] * ba[1]));
    const auto n = std::max<std::size_t>(
        1, static_cast<std::size_t>(std::ceil(len / d_max)));
    std::size_t prev = ia;
    for (std::size_t i = 1; i < n; ++i) {
      const Num t = static_cast<Num>(i) / static_cast<Num>(n);
      out.append_vert(a + t * ba);
      const std::size_t vi = out.num_verts() - 1;
      out.append_face({prev, vi});
      prev = vi;
    }
    out.append_face({prev, ib});
  }
  return out;
}

/// 3D: red refinement until no edge is longer than d_max.  Each round
/// bisects every edge longer than d_max (one midpoint per edge, appended in
/// the order the faces' edges ab, bc, ca are met), then splits each
/// triangle into 2, 3 or 4 by its bisected edges, keeping its orientation
/// (source/tit/geom/tessellation.hpp:66-186).
template<class V>
  requires (V::dim() == 3)
auto tessellate(const Surface<V>& surf, double d_max) -> Surface<V> {
  if (!(d_max > 0.0)) throw Exception{"tessellate: d_max <= 0"};
  std::vector<V> verts;
  for (std::size_t i = 0; i < surf.num_verts(); ++i) verts.push_back(surf.vert(i));
  using Tri = std::array<std::size_t, 3>;
  std::vector<Tri> tris, next;
  for (std::size_t fi = 0; fi < surf.num_faces(); ++fi) tris.push_back(surf.face_verts(fi));
  std::map<std::pair<std::size_t, std::size_t>, std::size_t> mid;
  constexpr std::size_t none = static_cast<std::size_t>(-1);
  for (;;) {
    mid.clear();
    const auto split = [&](std::size_t a, std::size_t b) {
      const auto key = std::minmax(a, b);
      if (mid.contains(key)) return;
      const V e = verts[b] - verts[a];
      if (static_cast<double>(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) <= d_max * d_max) {
        return;
      }
      using Num = std::remove_cvref_t<decltype(verts[a][0])>;
      verts.push_back((verts[a] + verts[b]) * Num{0.5});
      mid.emplace(key, verts.size() - 1);
    };
    for (const auto& [a, b, c] : tris) {
      split(a, b);
      split(b, c);
      split(c, a);
    }
    if (mid.empty()) break;
    const auto at = [&](std::size_t a, std::size_t b) {
      const auto it = mid.find(std::minmax(a, b));
      return it == mid.end() ? none : it->second;
    };
    next.clear();
    for (const auto& [a, b, c] : tris) {
      const std::size_t ab = at(a, b), bc = at(b, c), ca = at(c, a);
      const int n = (ab != none) + (bc != none) + (ca != none);
      if (n == 3) {
        next.insert(next.end(), {Tri{a, ab, ca}, Tri{ab, b, bc}, Tri{ca, bc, c}, Tri{ab, bc, ca}});
      } else if (n == 2 && ca == none) {
        next.insert(next.end(), {Tri{a, ab, c}, Tri{ab, bc, c}, Tri{ab, b, bc}});
      } else if (n == 2 && ab == none) {
        next.insert(next.end(), {Tri{b, bc, a}, Tri{bc, ca, a}, Tri{bc, c, ca}});
      } else if (n == 2) {
        next.insert(next.end(), {Tri{c, ca, b}, Tri{ca, ab, b}, Tri{ca, a, ab}});
      } else if (ab != none) {
        next.insert(next.end(), {Tri{a, ab, c}, Tri{ab, b, c}});
      } else if (bc != none) {
        next.insert(next.end(), {Tri{b, bc, a}, Tri{bc, c, a}});
      } else if (ca != none) {
        next.insert(next.end(), {Tri{c, ca, b}, Tri{ca, a, b}});
      } else {
        next.push_back(Tri{a, b, c});
      }
    }
    tris.swap(next);
  }
  Surface<V> out;
  for (const V& v : verts) out.append_vert(v);
  for (const Tri& t : tris) out.append_face(t);
  return out;
}

/// Containment by the winding number of a closed surface (> 1/2 inside),
/// the role of the reference's FastWinding (fast_winding.hpp:80-95): the
/// exact generalized winding number, summed per face (Segment / Triangle
/// ::winding_number), so the faces may come in any order.  The GPU receives
/// the surface itself (surface_data: in 2D the vertices of the closed loop
/// the segments chain into, in 3D 9 doubles per triangle).
template<class V>
class Winding {
public:
  explicit Winding(const Surface<V>& surf) {
    for (std::size_t fi = 0; fi < surf.num_faces(); ++fi) {
      for (const auto v : surf.face_verts(fi)) pts_.push_back(surf.vert(v));
    }
    if constexpr (V::dim() == 2) {
      // Chain the segments into one closed loop for the GPU.
      if (surf.num_faces() == 0) return;
      std::vector<std::size_t> next(surf.num_verts(), static_cast<std::size_t>(-1));
      for (std::size_t fi = 0; fi < surf.num_faces(); ++fi) {
        const auto [a, b] = surf.face_verts(fi);
        if (next[a] != static_cast<std::size_t>(-1)) {
          throw Exception{"Winding: a 2D containment vertex starts two segments"};
        }
        next[a] = b;
      }
      const std::size_t start = surf.face_verts(0)[0];
      std::size_t v = start;
      for (std::size_t k = 0; k < surf.num_faces(); ++k) {
        loop_.push_back(surf.vert(v));
        v = next[v];
        if (v == static_cast<std::size_t>(-1)) {
          throw Exception{"Winding: the 2D containment segments do not close"};
        }
        if (v == start) break;
      }
      if (v != start || loop_.size() != surf.num_faces()) {
        throw Exception{"Winding: the 2D containment must be one closed loop"};
      }
    }
  }
  auto operator()(const V& x) const -> double {
    constexpr double two_pi = 2.0 * 3.14159265358979323846;
    double w = 0.0;
    if constexpr (V::dim() == 2) {
      for (std::size_t i = 0; i < pts_.size(); i += 2) {
        const V a = pts_[i] - x, b = pts_[i + 1] - x;
        w += std::atan2(static_cast<double>(a[0] * b[1] - a[1] * b[0]),
                        static_cast<double>(a[0] * b[0] + a[1] * b[1]));
      }
    } else {
      // Solid angle of each triangle (Van Oosterom and Strackee), as
      // Triangle::winding_number (geom/triangle.hpp).
      const auto dot = [](const V& a, const V& b) {
        return static_cast<double>(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]);
      };
      for (std::size_t i = 0; i < pts_.size(); i += 3) {
        const V a = pts_[i] - x, b = pts_[i + 1] - x, c = pts_[i + 2] - x;
        const double na = std::sqrt(dot(a, a)), nb = std::sqrt(dot(b, b)),
                     nc = std::sqrt(dot(c, c));
        const double det =
            static_cast<double>(a[0] * (b[1] * c[2] - b[2] * c[1]) +
                                a[1] * (b[2] * c[0] - b[0] * c[2]) +
                                a[2] * (b[0] * c[1] - b[1] * c[0]));
        w += std::atan2(det, na * nb * nc + dot(a, b) * nc + dot(b, c) * na +
                                 dot(c, a) * nb);
      }
    }
    return w / two_pi;
  }
  auto contains(const V& x) const -> bool { return (*this)(x) > 0.5; }
  auto surface_data() const -> std::vector<double> {
    std::vector<double> out;
    for (const V& v : V::dim() == 2 ? loop_ : pts_) {
      for (std::size_t k = 0; k < V::dim(); ++k) out.push_back(static_cast<double>(v[k]));
    }
    return out;
  }
  /// The 2D loop's vertices (x, y), as surface_data.
  auto polygon() const -> std::vector<double> { return surface_data(); }

private:
  std::vector<V> pts_;   // the faces' vertices, dim per face
  std::vector<V> loop_;  // 2D: the chained loop
};

/// Maker of winding-number containment functions (the reference's
/// MakeFastWinding, fast_winding.hpp).
template<class Num>
struct MakeFastWinding {
  template<class V>
  auto operator()(const Surface<V>& surf) const -> Winding<V> {
    return Winding<V>{surf};
  }
};

/// Grid neighbour search with the given cell spacing
/// (source/tit/geom/search/grid_search.hpp:73-113).  On the GPU the spacing
/// picks how many grid cells span the kernel support radius (1, 2 or 3).
struct GridSearch {
  double spacing;
  explicit GridSearch(double cell_spacing) : spacing{cell_spacing} {
    if (!(cell_spacing > 0.0)) throw Exception{"GridSearch: spacing <= 0"};
  }
};

/// K-dimensional tree search (source/tit/geom/search/kd_tree_search.hpp
/// :151-165).  The neighbour sets are those of the inclusive sphere
/// predicate whatever the index, so on the GPU it selects the grid search
/// with the library's default cells per support radius.
struct KDTreeSearch {};
inline constexpr KDTreeSearch kd_tree_indexing{};

/// Face search and partitioners of the reference mesh.  The GPU path has no
/// faces and sums in gather form, so these only record the driver's choice.
struct GridFaceSearch {
  double spacing;
  explicit GridFaceSearch(double cell_spacing) : spacing{cell_spacing} {}
};
struct RecursiveInertialBisection {};
struct KMeansClustering {};
struct PixelatedPartition {
  template<class... Args>
  explicit PixelatedPartition(Args&&... /*args*/) noexcept {}
};

/// Containment functor that accepts every point.
struct AllInside {
  template<class V>
  constexpr auto operator()(const V& /*point*/) const noexcept -> bool {
    return true;
  }
};

} // namespace geom

namespace sph {

template<class Real, std::size_t Dim>
struct Space {
  using real_t = Real;
  static constexpr std::size_t dim = Dim;
};

/// Particle types (source/tit/sph/particle_array.hpp).
enum class ParticleType : std::uint8_t { fluid, fixed, count };

// Smoothing kernels: the closed set of source/tit/sph/kernel.hpp:459-465.
// `unit_radius` is the support radius in units of h.
struct CubicSplineKernel {
  static constexpr std::int32_t gpu_id = TG_KERNEL_CUBIC_SPLINE;
  static constexpr double unit_radius = 2.0;
};
struct QuarticSplineKernel {
  static constexpr std::int32_t gpu_id = TG_KERNEL_QUARTIC_SPLINE;
  static constexpr double unit_radius = 2.5;
};
struct QuinticSplineKernel {
  static constexpr std::int32_t gpu_id = TG_KERNEL_QUINTIC_SPLINE;
  static constexpr double unit_radius = 3.0;
};
struct QuarticWendlandKernel {
  static constexpr std::int32_t gpu_id = TG_KERNEL_WENDLAND_C2;
  static constexpr double unit_radius = 2.0;
};
struct SixthOrderWendlandKernel {
  static constexpr std::int32_t gpu_id = TG_KERNEL_WENDLAND_C4;
  static constexpr double unit_radius = 2.0;
};
struct EighthOrderWendlandKernel {
  static constexpr std::int32_t gpu_id = TG_KERNEL_WENDLAND_C6;
  static constexpr double unit_radius = 2.0;
};

/// Tait equation of state (source/tit/sph/equation_of_state.hpp:19-72).
template<class Num>
class TaitEquationOfState {
public:
  constexpr explicit TaitEquationOfState(Num cs_0, Num rho_0, Num xi = Num{7})
      : cs_0_{cs_0}, rho_0_{rho_0}, xi_{xi} {
    if (!(cs_0 > Num{0}) || !(rho_0 > Num{0}) || !(xi > Num{1})) {
      throw Exception{"TaitEquationOfState: need cs_0 > 0, rho_0 > 0, xi > 1"};
    }
  }
  auto pressure_from_density(Num rho) const -> Num {
    return rho_0_ * pow2(cs_0_) / xi_ * (std::pow(rho / rho_0_, xi_) - 1);
  }
  auto sound_speed_from_density(Num rho) const -> Num {
    return cs_0_ * std::pow(rho / rho_0_, (xi_ - 1) / 2);
  }
  constexpr auto cs_0() const noexcept -> Num { return cs_0_; }
  constexpr auto rho_0() const noexcept -> Num { return rho_0_; }
  constexpr auto xi() const noexcept -> Num { return xi_; }

  static constexpr std::int32_t gpu_id = TG_EOS_TAIT;

private:
  Num cs_0_;
  Num rho_0_;
  Num xi_;
};

/// Linear Tait equation of state (source/tit/sph/equation_of_state.hpp
/// :78-122): p = cs_0^2 (rho - rho_0), constant sound speed cs_0.
template<class Num>
class LinearTaitEquationOfState {
public:
  constexpr LinearTaitEquationOfState(Num cs_0, Num rho_0)
      : cs_0_{cs_0}, rho_0_{rho_0} {
    if (!(cs_0 > Num{0}) || !(rho_0 > Num{0})) {
      throw Exception{"LinearTaitEquationOfState: need cs_0 > 0, rho_0 > 0"};
    }
  }
  auto pressure_from_density(Num rho) const -> Num {
    return pow2(cs_0_) * (rho - rho_0_);
  }
  auto density_from_pressure(Num p) const -> Num {
    return rho_0_ + p / pow2(cs_0_);
  }
  auto sound_speed_from_density(Num /*rho*/) const -> Num { return cs_0_; }
  constexpr auto cs_0() const noexcept -> Num { return cs_0_; }
  constexpr auto rho_0() const noexcept -> Num { return rho_0_; }
  static constexpr std::int32_t gpu_id = TG_EOS_LINEAR_TAIT;

private:
  Num cs_0_;
  Num rho_0_;
};

template<class Num>
LinearTaitEquationOfState(Num, Num) -> LinearTaitEquationOfState<Num>;

/// Arithmetic form of the GPU pair sums.
enum class Precision : std::int32_t {
  fp64 = TG_FP64,                  ///< plain FP64
  fp32_compensated = TG_FP32C,     ///< FP32 sums with Kahan compensation
};

/// GPU-side choices with no counterpart in the reference constructor.  The
/// defaults are the reference's own terms: Morris viscosity with the given
/// mu, Ferrari diffusion, CFL 0.4, C_force 0.25, C_visc 0.125
/// (fluid_equations.hpp:518-520), shifting after every step.
struct GpuOptions {
  Precision precision = Precision::fp64;
  std::int32_t viscosity = TG_VISC_MORRIS;
  std::int32_t diffusion = TG_DIFF_FERRARI;
  double alpha = 0.0; ///< Monaghan artificial viscosity (TG_VISC_MONAGHAN)
  double delta = 0.0; ///< delta-SPH coefficient (TG_DIFF_MOLTENI)
  double cfl = 0.4;
  double c_force = 0.25;
  double c_visc = 0.125;
  bool kahan = true;
  /// Face walls in the compensated form: closed-form face integrals in FP32
  /// (faster, larger drift from the FP64 form) instead of FP64.
  bool face_fp32 = false;
  std::int32_t device = -1; ///< CUDA ordinal; -1 = the current device
  bool graph = true;        ///< replay each step as a CUDA graph
  bool autotune = false;    ///< pick launch shapes with tg_autotune
  /// Particle shifting and the free-surface density correction after each
  /// step; FluidEquations::post_integrate always runs them
  /// (fluid_equations.hpp:315-321).
  bool shifting = true;
};

template<class PA>
class ParticleView;
template<class Real, std::size_t Dim>
class ParticleArray;

/// Thin handle of the reference ParticleMesh: it keeps the search spacing
/// (the neighbour structure itself lives on the GPU, inside the particles'
/// context).
class ParticleMesh {
public:
  template<class... Rest>
  explicit ParticleMesh(geom::GridSearch search, Rest&&... /*rest*/) noexcept
      : spacing_{search.spacing} {}
  template<class... Rest>
  explicit ParticleMesh(geom::KDTreeSearch /*search*/, Rest&&... /*rest*/) noexcept
      : spacing_{0.0} {}
  /// Grid search spacing (0: the library's default grid, as for a k-d tree).
  auto spacing() const noexcept -> double { return spacing_; }

private:
  double spacing_;
};

/// Fluid equations (source/tit/sph/fluid_equations.hpp:61-69) with either
/// equation of state of the reference's closed set.
template<class Real, std::size_t Dim, class Containment, class EOS, class Kernel>
class FluidEquations {
  static_assert(std::is_same_v<EOS, TaitEquationOfState<Real>> ||
                    std::is_same_v<EOS, LinearTaitEquationOfState<Real>>,
                "equation_of_state: TaitEquationOfState or LinearTaitEquationOfState");

public:
  FluidEquations(Real g,
                 Real mu,
                 geom::Surface<Vec<Real, Dim>> domain,
                 Containment containment,
                 EOS eos,
                 Kernel /*kernel*/,
                 GpuOptions options = {})
      : g_{g}, mu_{mu}, domain_{std::move(domain)},
        containment_{std::move(containment)}, eos_{eos}, options_{options} {
    if (domain_.num_faces() != 0) {
      if constexpr (!has_surface_) {
        throw Exception{"FluidEquations: boundary faces need a "
                        "winding-number containment (geom::MakeFastWinding)"};
      }
    }
  }

  /// Create the GPU context and upload the particles
  /// (FluidEquations::initialize, fluid_equations.hpp:79-89).
  template<class PA>
  void initialize(ParticleMesh& mesh, PA& particles) const {
    for (const auto a : particles.fluid()) {
      if (!contains_(std::as_const(particles).position(a.index()))) {
        throw Exception{"FluidEquations::initialize: a fluid particle lies "
                        "outside the containment (gamma = 0)"};
      }
    }
    tg_params P;
    tg_params_default(&P);
    P.dim = static_cast<std::int32_t>(Dim);
    P.precision = static_cast<std::int32_t>(options_.precision);
    P.kernel = Kernel::gpu_id;
    P.integrator = particles.integrator_id();
    P.post_integrate = options_.shifting ? TG_POST_SHIFTING : TG_POST_PREPARE;
    P.viscosity = options_.viscosity;
    P.diffusion = options_.diffusion;
    P.kahan = options_.kahan ? 1 : 0;
    P.face_fp32 = options_.face_fp32 ? 1 : 0;
    P.device = options_.device;
    P.eos = EOS::gpu_id;
    if constexpr (requires { eos_.xi(); }) P.xi = static_cast<double>(eos_.xi());
    P.g = static_cast<double>(g_);
    P.mu = static_cast<double>(mu_);
    P.alpha = options_.alpha;
    P.delta = options_.delta;
    P.cfl = options_.cfl;
    P.c_force = options_.c_force;
    P.c_visc = options_.c_visc;
    // Cells of the grid search's spacing across the support radius (the
    // default grid for a k-d tree search).
    if (mesh.spacing() > 0.0) {
      const double radius = Kernel::unit_radius * particles.uniform_h();
      const long k = std::lround(radius / mesh.spacing());
      P.cells_per_radius = static_cast<std::int32_t>(k < 1 ? 1 : (k > 3 ? 3 : k));
    }
    particles.attach_(P,
                      static_cast<double>(eos_.rho_0()),
                      static_cast<double>(eos_.cs_0()),
                      options_.graph,
                      options_.autotune && domain_.num_faces() == 0);
    if constexpr (has_surface_) {
      if (domain_.num_faces() != 0) attach_faces_(particles);
    }
  }

  auto eos() const noexcept -> const EOS& { return eos_; }

private:
  auto contains_(const Vec<Real, Dim>& x) const -> bool {
    if constexpr (requires { containment_.contains(x); }) {
      return containment_.contains(x);
    } else {
      return static_cast<bool>(containment_(x));
    }
  }

  static constexpr bool has_surface_ =
      requires(const Containment& c) { c.surface_data(); };

  // The tank's fixed particles must be the domain's vertices, in order
  // (wcsph.cpp:109-112); the faces index them.
  template<class PA>
  void attach_faces_(PA& particles) const {
    const auto& cp = std::as_const(particles);
    if (cp.size() - cp.num_fluid() < domain_.num_verts()) {
      throw Exception{"initialize: fewer fixed particles than domain vertices"};
    }
    for (std::size_t i = 0; i < domain_.num_verts(); ++i) {
      if (!(cp.position(cp.num_fluid() + i) == domain_.vert(i))) {
        throw Exception{"initialize: fixed particle " + std::to_string(i) +
                        " is not domain vertex " + std::to_string(i)};
      }
    }
    std::vector<std::int32_t> fv;
    for (std::size_t fi = 0; fi < domain_.num_faces(); ++fi) {
      for (const auto v : domain_.face_verts(fi)) {
        fv.push_back(static_cast<std::int32_t>(v));
      }
    }
    const std::vector<double> surf = containment_.surface_data();
    const std::size_t per = Dim == 2 ? 2 : 9;
    gpu_detail::ensure(
        tg_tank_faces(particles.context(), 0,
                      static_cast<std::int32_t>(domain_.num_faces()), fv.data(),
                      static_cast<std::int32_t>(surf.size() / per), surf.data()),
        particles.context(), "tg_tank_faces");
    if (options_.autotune) {
      tg_tuning tuned{};
      gpu_detail::ensure(tg_autotune(particles.context(), 3, &tuned),
                         particles.context(), "tg_autotune");
    }
  }

  Real g_;
  Real mu_;
  geom::Surface<Vec<Real, Dim>> domain_;
  Containment containment_;
  EOS eos_;
  GpuOptions options_;
};

template<class Real, std::size_t Dim, class Containment, class EOS, class Kernel>
FluidEquations(Real,
               Real,
               geom::Surface<Vec<Real, Dim>>,
               Containment,
               EOS,
               Kernel,
               GpuOptions = {})
    -> FluidEquations<Real, Dim, Containment, EOS, Kernel>;

namespace integrator_detail {
// One GPU step of a ParticleArray bound to a context.
template<class Equations, class PA>
auto step(const Equations& equations, ParticleMesh& mesh, PA& particles)
    -> double {
  if (!particles.attached()) equations.initialize(mesh, particles);
  return particles.step_();
}
} // namespace integrator_detail

/// SSPRK order (time_integrator.hpp).
enum class SSPRKOrder : std::uint8_t { two, three };

/// SSPRK integrator (time_integrator.hpp:140-228).
template<class Equations>
class SSPRKIntegrator {
public:
  explicit SSPRKIntegrator(Equations equations,
                           SSPRKOrder order = SSPRKOrder::three)
      : equations_{std::move(equations)}, order_{order} {}
  auto gpu_integrator() const noexcept -> std::int32_t {
    return order_ == SSPRKOrder::three ? TG_SSPRK3 : TG_SSPRK2;
  }
  template<class PA>
  auto step(ParticleMesh& mesh, PA& particles) const {
    return static_cast<typename PA::real_t>(
        integrator_detail::step(equations_, mesh, particles));
  }
  auto equations() const noexcept -> const Equations& { return equations_; }

private:
  Equations equations_;
  SSPRKOrder order_;
};

/// Symplectic Euler integrator (time_integrator.hpp:31-75).
template<class Equations>
class SymplecticEulerIntegrator {
public:
  explicit SymplecticEulerIntegrator(Equations equations)
      : equations_{std::move(equations)} {}
  static constexpr auto gpu_integrator() noexcept -> std::int32_t {
    return TG_EULER;
  }
  template<class PA>
  auto step(ParticleMesh& mesh, PA& particles) const {
    return static_cast<typename PA::real_t>(
        integrator_detail::step(equations_, mesh, particles));
  }

private:
  Equations equations_;
};

/// Velocity Verlet integrator (time_integrator.hpp:80-129).
template<class Equations>
class VelocityVerletIntegrator {
public:
  explicit VelocityVerletIntegrator(Equations equations)
      : equations_{std::move(equations)} {}
  static constexpr auto gpu_integrator() noexcept -> std::int32_t {
    return TG_VERLET;
  }
  template<class PA>
  auto step(ParticleMesh& mesh, PA& particles) const {
    return static_cast<typename PA::real_t>(
        integrator_detail::step(equations_, mesh, particles));
  }

private:
  Equations equations_;
};

/// A particle of a ParticleArray: the array and the particle's index, fluid
/// particles first (particle_array.hpp:188-199).
template<class PA>
class ParticleView {
public:
  constexpr ParticleView(PA& array, std::size_t index) noexcept
      : array_{&array}, index_{index} {}
  constexpr auto array() const noexcept -> PA& { return *array_; }
  constexpr auto index() const noexcept -> std::size_t { return index_; }
  auto has_type(ParticleType type) const noexcept -> bool {
    return array_->type_of(index_) == type;
  }

private:
  PA* array_;
  std::size_t index_;
};

/// Particle array (particle_array.hpp:139-293) whose state is mirrored on
/// one GPU context.  Real is the driver's floating type; the GPU computes in
/// FP64 or the FP32-compensated form whatever Real is.
template<class Real, std::size_t Dim>
class ParticleArray {
public:
  using real_t = Real;
  using vec_t = Vec<Real, Dim>;
  static constexpr std::size_t dim = Dim;

  template<class Integrator>
  ParticleArray(Space<Real, Dim> /*space*/, const Integrator& integrator)
      : integrator_id_{integrator.gpu_integrator()} {}

  ParticleArray(const ParticleArray&) = delete;
  auto operator=(const ParticleArray&) -> ParticleArray& = delete;
  ParticleArray(ParticleArray&&) noexcept = default;
  auto operator=(ParticleArray&&) noexcept -> ParticleArray& = default;
  ~ParticleArray() { detach_(); }

  auto size() const noexcept -> std::size_t { return r_.size(); }
  auto num_fluid() const noexcept -> std::size_t { return n_fluid_; }

  /// Append a particle; fluid particles go before the fixed ones.
  auto append(ParticleType type) -> ParticleView<ParticleArray> {
    if (type != ParticleType::fluid && type != ParticleType::fixed) {
      throw Exception{"ParticleArray::append: invalid particle type"};
    }
    if (ctx_ != nullptr) {
      throw Exception{"ParticleArray::append: particles are on the GPU"};
    }
    const std::size_t at = type == ParticleType::fluid ? n_fluid_++ : size();
    r_.emplace(r_.begin() + static_cast<std::ptrdiff_t>(at));
    v_.emplace(v_.begin() + static_cast<std::ptrdiff_t>(at));
    dv_dt_.emplace(dv_dt_.begin() + static_cast<std::ptrdiff_t>(at));
    rho_.emplace(rho_.begin() + static_cast<std::ptrdiff_t>(at));
    drho_dt_.emplace(drho_dt_.begin() + static_cast<std::ptrdiff_t>(at));
    m_.emplace(m_.begin() + static_cast<std::ptrdiff_t>(at));
    return {*this, at};
  }

  auto all() noexcept { return views_(0, size()); }
  auto fluid() noexcept { return views_(0, n_fluid_); }
  auto fixed() noexcept { return views_(n_fluid_, size()); }
  auto typed(ParticleType type) noexcept {
    return type == ParticleType::fluid ? fluid() : fixed();
  }

  auto type_of(std::size_t i) const noexcept -> ParticleType {
    return i < n_fluid_ ? ParticleType::fluid : ParticleType::fixed;
  }

  // ---- field storage (used by the field objects below) --------------------
  auto position(std::size_t i) -> vec_t& { return pull_mut_(r_)[i]; }
  auto position(std::size_t i) const -> const vec_t& { return pull_(r_)[i]; }
  auto velocity(std::size_t i) -> vec_t& { return pull_mut_(v_)[i]; }
  auto velocity(std::size_t i) const -> const vec_t& { return pull_(v_)[i]; }
  auto accel(std::size_t i) -> vec_t& { return pull_mut_(dv_dt_)[i]; }
  auto accel(std::size_t i) const -> const vec_t& { return pull_(dv_dt_)[i]; }
  auto density(std::size_t i) -> Real& { return pull_mut_(rho_)[i]; }
  auto density(std::size_t i) const -> const Real& { return pull_(rho_)[i]; }
  auto drho(std::size_t i) const -> const Real& { return pull_(drho_dt_)[i]; }
  auto mass(std::size_t i) -> Real& {
    if (ctx_ != nullptr) throw Exception{"m: masses are fixed on the GPU"};
    return m_[i];
  }
  auto mass(std::size_t i) const -> const Real& { return m_[i]; }
  auto uniform_h() -> Real& {
    if (ctx_ != nullptr) throw Exception{"h: widths are fixed on the GPU"};
    return h_;
  }
  auto uniform_h() const -> const Real& { return h_; }

  // ---- GPU binding (FluidEquations::initialize and the integrators) -------
  auto integrator_id() const noexcept -> std::int32_t { return integrator_id_; }
  auto attached() const noexcept -> bool { return ctx_ != nullptr; }
  auto context() const noexcept -> tg_context* { return ctx_; }

  void attach_(tg_params P, double rho_0, double cs_0, bool graph,
               bool autotune) {
    if (n_fluid_ == 0) throw Exception{"initialize: no fluid particles"};
    if (!(h_ > Real{0})) throw Exception{"initialize: set h[particles] first"};
    for (std::size_t i = 1; i < size(); ++i) {
      if (m_[i] != m_[0]) {
        throw Exception{"initialize: the GPU path needs one uniform mass"};
      }
    }
    detach_();
    tg_context* ctx = nullptr;
    gpu_detail::ensure(tg_context_create(&P, &ctx), nullptr,
                       "tg_context_create");
    ctx_ = ctx;
    tg_tank tank{};
    tank.n_fluid = static_cast<std::int64_t>(n_fluid_);
    tank.n_wall = static_cast<std::int64_t>(size() - n_fluid_);
    tank.h = static_cast<double>(h_);
    tank.m = static_cast<double>(m_[0]);
    tank.rho0 = rho_0;
    tank.cs0 = cs_0;
    std::vector<double> r, v, rho;
    pack_(r, v, rho);
    gpu_detail::ensure(tg_particles_upload(ctx_, 1, &tank, r.data(), v.data(),
                                           rho.data()),
                       ctx_, "tg_particles_upload");
    gpu_detail::ensure(tg_set_graph(ctx_, graph ? 1 : 0), ctx_,
                       "tg_set_graph");
    if (autotune) {
      tg_tuning tuned{};
      gpu_detail::ensure(tg_autotune(ctx_, 3, &tuned), ctx_, "tg_autotune");
    }
    state_ = State::synced;
  }

  auto step_() -> double {
    if (state_ == State::host_ahead) push_();
    double dt = 0.0;
    gpu_detail::ensure(tg_step(ctx_, 1, &dt), ctx_, "tg_step");
    state_ = State::device_ahead;
    return dt;
  }

  /// Write the particle fields as a new frame of `series`
  /// (ParticleArray::write, particle_array.hpp:165-172): r, v, dv_dt, rho,
  /// drho_dt, p, cs and m under the reference's field names.  The fields are
  /// copied from the device here; the storage writes them on a background
  /// thread while the caller goes on stepping.  Include titgpu_data.hpp for
  /// the storage.
  template<class Series>
  void write(double time, const Series& series) const {
    sync();
    auto& storage = series.storage();
    using Blob = typename std::remove_reference_t<decltype(storage)>::blob_type;
    std::vector<Blob> arrays;
    arrays.push_back(Blob::of(std::string{"r"}, std::span<const vec_t>{r_}));
    arrays.push_back(Blob::of(std::string{"v"}, std::span<const vec_t>{v_}));
    arrays.push_back(
        Blob::of(std::string{"dv_dt"}, std::span<const vec_t>{dv_dt_}));
    arrays.push_back(Blob::of(std::string{"rho"}, std::span<const Real>{rho_}));
    arrays.push_back(
        Blob::of(std::string{"drho_dt"}, std::span<const Real>{drho_dt_}));
    if (ctx_ != nullptr) {
      std::vector<double> buf(size());
      std::vector<Real> col(size());
      for (const auto& [field, name] :
           {std::pair{TG_FIELD_P, "p"}, std::pair{TG_FIELD_CS, "cs"}}) {
        gpu_detail::ensure(tg_particles_download(ctx_, field, buf.data()),
                           ctx_, "tg_particles_download");
        for (std::size_t i = 0; i < size(); ++i) {
          col[i] = static_cast<Real>(buf[i]);
        }
        arrays.push_back(Blob::of(std::string{name}, std::span<const Real>{col}));
      }
    }
    arrays.push_back(Blob::of(std::string{"m"}, std::span<const Real>{m_}));
    storage.write_frame_async(series.id(), time, std::move(arrays));
  }

  /// Bring the host copy up to date (one state download after GPU steps).
  void sync() const {
    if (state_ != State::device_ahead) return;
    const std::size_t n = size();
    std::vector<double> r(n * Dim), v(n * Dim), dv(n * Dim), rho(n), drho(n);
    gpu_detail::ensure(tg_particles_download_state(ctx_, r.data(), v.data(), rho.data(),
                                                   drho.data(), dv.data()),
                       ctx_, "tg_particles_download_state");
    for (std::size_t i = 0; i < n; ++i) {
      for (std::size_t d = 0; d < Dim; ++d) {
        r_[i][d] = static_cast<Real>(r[i * Dim + d]);
        v_[i][d] = static_cast<Real>(v[i * Dim + d]);
        dv_dt_[i][d] = static_cast<Real>(dv[i * Dim + d]);
      }
      rho_[i] = static_cast<Real>(rho[i]);
      drho_dt_[i] = static_cast<Real>(drho[i]);
    }
    state_ = State::synced;
  }

private:
  enum class State : std::uint8_t { host_only, synced, device_ahead, host_ahead };

  auto views_(std::size_t lo, std::size_t hi) noexcept {
    return std::views::iota(lo, hi) |
           std::views::transform([this](std::size_t i) {
             return ParticleView<ParticleArray>{*this, i};
           });
  }

  template<class T>
  auto pull_(const std::vector<T>& col) const -> const std::vector<T>& {
    sync();
    return col;
  }
  template<class T>
  auto pull_mut_(std::vector<T>& col) -> std::vector<T>& {
    sync();
    if (state_ == State::synced) state_ = State::host_ahead;
    return col;
  }

  void pack_(std::vector<double>& r, std::vector<double>& v,
             std::vector<double>& rho, std::vector<double>* dv = nullptr) const {
    const std::size_t n = size();
    r.resize(n * Dim);
    v.resize(n * Dim);
    rho.resize(n);
    if (dv != nullptr) dv->resize(n * Dim);
    for (std::size_t i = 0; i < n; ++i) {
      for (std::size_t d = 0; d < Dim; ++d) {
        r[i * Dim + d] = static_cast<double>(r_[i][d]);
        v[i * Dim + d] = static_cast<double>(v_[i][d]);
        if (dv != nullptr) (*dv)[i * Dim + d] = static_cast<double>(dv_dt_[i][d]);
      }
      rho[i] = static_cast<double>(rho_[i]);
    }
  }

  void push_() {
    std::vector<double> r, v, rho, dv;
    pack_(r, v, rho, &dv);
    gpu_detail::ensure(tg_particles_update(ctx_, r.data(), v.data(),
                                           rho.data(), dv.data()),
                       ctx_, "tg_particles_update");
    state_ = State::synced;
  }

  void detach_() noexcept {
    if (ctx_ != nullptr) tg_context_destroy(ctx_);
    ctx_ = nullptr;
    state_ = State::host_only;
  }

  std::int32_t integrator_id_;
  std::size_t n_fluid_ = 0;
  Real h_{};
  mutable std::vector<vec_t> r_, v_, dv_dt_;
  mutable std::vector<Real> rho_, drho_dt_;
  std::vector<Real> m_;
  tg_context* ctx_ = nullptr;
  mutable State state_ = State::host_only;
};

template<class Real, std::size_t Dim, class Integrator>
ParticleArray(Space<Real, Dim>, const Integrator&) -> ParticleArray<Real, Dim>;

} // namespace sph

// ---- fields (source/tit/sph/field.hpp:172-218) ------------------------------
namespace gpu_detail {
template<class Get>
struct Field {
  Get get;
  template<class PA>
  constexpr decltype(auto) operator[](sph::ParticleView<PA> a) const {
    return get(a.array(), a.index());
  }
};
struct UniformH {
  template<class PA>
  constexpr decltype(auto) operator[](sph::ParticleView<PA> a) const {
    return std::as_const(a.array()).uniform_h();
  }
  template<class Real, std::size_t Dim>
  constexpr auto operator[](sph::ParticleArray<Real, Dim>& particles) const
      -> Real& {
    return particles.uniform_h();
  }
};
} // namespace gpu_detail

namespace sph {
/// Particle position.
inline constexpr gpu_detail::Field r{
    [](auto& pa, std::size_t i) -> decltype(auto) { return pa.position(i); }};
} // namespace sph
/// Particle velocity.
inline constexpr gpu_detail::Field v{
    [](auto& pa, std::size_t i) -> decltype(auto) { return pa.velocity(i); }};
/// Particle acceleration.
inline constexpr gpu_detail::Field dv_dt{
    [](auto& pa, std::size_t i) -> decltype(auto) { return pa.accel(i); }};
/// Particle density.
inline constexpr gpu_detail::Field rho{
    [](auto& pa, std::size_t i) -> decltype(auto) { return pa.density(i); }};
/// Particle density time derivative (read-only on the host).
inline constexpr gpu_detail::Field drho_dt{
    [](auto& pa, std::size_t i) -> decltype(auto) {
      return std::as_const(pa).drho(i);
    }};
/// Particle mass.
inline constexpr gpu_detail::Field m{
    [](auto& pa, std::size_t i) -> decltype(auto) { return pa.mass(i); }};
/// Particle width (uniform over the array).
inline constexpr gpu_detail::UniformH h{};

} // namespace tit

#endif // TITGPU_HPP
