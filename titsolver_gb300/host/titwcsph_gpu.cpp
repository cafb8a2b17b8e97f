// titwcsph_gpu.cpp - the titwcsph dam break (source/titwcsph/wcsph.cpp:37-193)
// driven through the C++ mirror of titgpu.hpp: the same setup expressions,
// API calls and loop.  With --faces the walls are the reference's own: the
// tessellated pool surface, one fixed particle per vertex and a
// winding-number containment; by default three layers of fixed wall
// particles with an empty surface (particle walls).
//
// Usage: titwcsph_gpu [--nx N] [--steps S] [--end-time T] [--fp32c]
//                     [--integrator ssprk3|ssprk2|euler|verlet]
//                     [--no-shifting] [--faces] [--ttdb FILE] [--dump FILE]
//                     [--log] [--eos tait|linear] [--face-fp32]
//   --nx       particles per column height H (default 80, as wcsph.cpp:42)
//   --steps    stop after S steps (default: run to scaled time T)
//   --end-time scaled end time t sqrt(g/H) (default 10, as wcsph.cpp:183)
//   --fp32c    FP32-compensated pair sums instead of plain FP64
//   --face-fp32   with --fp32c --faces: face integrals in FP32
//   --integrator  time integrator (default ssprk3, as wcsph.cpp:92)
//   --no-shifting skip the post-step shifting and free-surface correction
//                 (the reference always runs them)
//   --faces    the reference's face walls
//   --ttdb     write frames every 100 steps to this .ttdb file
//   --dump     write the initial and final state as raw binary (see below)
//   --eos      equation of state: TaitEquationOfState (default, as
//              wcsph.cpp:83) or LinearTaitEquationOfState
//   --log      print the reference's per-step line: step, scaled time, wall
//              seconds of the previous step and of the previous write
//              (wcsph.cpp:172-176)
//
// Dump layout (little-endian): int64 n, n_fluid, steps; float64 h, m, rho_0,
// cs_0, time; then r (n x 2), v (n x 2), rho (n) of the initial state and
// the same of the final state; with --faces then int64 n_faces, n_faces
// pairs of int32 fixed-particle indices, int64 n_poly and n_poly (x, y)
// float64 containment vertices.

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <numbers>
#include <optional>
#include <string>
#include <vector>

#include "titgpu.hpp"
#include "titgpu_data.hpp"

namespace tit::sph::wcsph {
namespace {

struct Options {
  int nx = 80;
  long steps = -1;
  double end_time = 10.0;
  bool fp32c = false;
  std::string integrator = "ssprk3";
  bool shifting = true;
  bool faces = false;
  std::string ttdb;
  std::string dump;
  bool log = false;
  std::string eos = "tait";
  bool face_fp32 = false;
};

auto parse(int argc, char** argv) -> Options {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    const auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw Exception{"missing value after " + a};
      return argv[++i];
    };
    if (a == "--nx") o.nx = std::stoi(next());
    else if (a == "--steps") o.steps = std::stol(next());
    else if (a == "--end-time") o.end_time = std::stod(next());
    else if (a == "--fp32c") o.fp32c = true;
    else if (a == "--integrator") o.integrator = next();
    else if (a == "--no-shifting") o.shifting = false;
    else if (a == "--faces") o.faces = true;
    else if (a == "--ttdb") o.ttdb = next();
    else if (a == "--dump") o.dump = next();
    else if (a == "--log") o.log = true;
    else if (a == "--eos") o.eos = next();
    else if (a == "--face-fp32") o.face_fp32 = true;
    else throw Exception{"unknown option " + a};
  }
  if (o.nx < 4) throw Exception{"--nx must be at least 4"};
  if (o.eos != "tait" && o.eos != "linear") throw Exception{"unknown --eos " + o.eos};
  if (o.face_fp32 && !o.fp32c) throw Exception{"--face-fp32 needs --fp32c"};
  if (o.integrator != "ssprk3" && o.integrator != "ssprk2" &&
      o.integrator != "euler" && o.integrator != "verlet") {
    throw Exception{"unknown integrator " + o.integrator};
  }
  return o;
}

template<class PA>
void dump_state(std::ofstream& out, PA& particles) {
  const auto& cp = std::as_const(particles);
  for (std::size_t i = 0; i < cp.size(); ++i) {
    const auto& x = cp.position(i);
    out.write(reinterpret_cast<const char*>(&x[0]), 2 * sizeof(double));
  }
  for (std::size_t i = 0; i < cp.size(); ++i) {
    const auto& x = cp.velocity(i);
    out.write(reinterpret_cast<const char*>(&x[0]), 2 * sizeof(double));
  }
  for (std::size_t i = 0; i < cp.size(); ++i) {
    const double d = cp.density(i);
    out.write(reinterpret_cast<const char*>(&d), sizeof(double));
  }
}

template<class Real, class Equations, class Integrator>
auto simulate(const Options& opt, const Equations& equations,
              const Integrator& time_integrator,
              const geom::Surface<Vec<Real, 2>>* domain) -> int;
template<class Real, class Equations>
auto run_integrator(const Options& opt, const Equations& equations,
                    const geom::Surface<Vec<Real, 2>>* domain) -> int;

template<class Real, class EOS>
auto sph_main_eos(const Options& opt, const EOS& eos) -> int {
  constexpr Real H = 0.6; // Water column height.

  constexpr Real g = 9.81;
  constexpr Real mu = 0.001;

  GpuOptions gpu;
  gpu.precision = opt.fp32c ? Precision::fp32_compensated : Precision::fp64;
  gpu.shifting = opt.shifting;
  gpu.face_fp32 = opt.face_fp32;
  if (opt.faces) {
    // The reference's walls (wcsph.cpp:55-77): the pool surface tessellated
    // at dr, and a winding-number containment of the pool.
    constexpr Real POOL_WIDTH = 5.366 * H;
    constexpr Real POOL_HEIGHT = 4.0 * H;
    const Real dr = H / opt.nx;
    geom::Surface<Vec<Real, 2>> domain;
    domain.append_vert({0.0, POOL_HEIGHT});
    domain.append_vert({POOL_WIDTH, POOL_HEIGHT});
    domain.append_vert({POOL_WIDTH, 0.0});
    domain.append_vert({0.0, 0.0});
    domain.append_face({0, 1});
    domain.append_face({1, 2});
    domain.append_face({2, 3});
    domain.append_face({3, 0});
    domain = geom::tessellate(domain, dr);
    geom::Surface<Vec<Real, 2>> domain2;
    domain2.append_vert({0.0, 0.0});
    domain2.append_vert({POOL_WIDTH, 0.0});
    domain2.append_vert({POOL_WIDTH, POOL_HEIGHT});
    domain2.append_vert({0.0, POOL_HEIGHT});
    domain2.append_face({0, 1});
    domain2.append_face({1, 2});
    domain2.append_face({2, 3});
    domain2.append_face({3, 0});
    const geom::MakeFastWinding<Real> make_winding;
    const auto containment = make_winding(domain2);
    const FluidEquations equations{
        g, mu, domain, containment, eos, SixthOrderWendlandKernel{}, gpu,
    };
    return run_integrator<Real>(opt, equations, &domain);
  }
  // Particle walls: the domain surface stays empty and every point is
  // inside the containment (gamma = 1, no face terms).
  const geom::Surface<Vec<Real, 2>> domain;
  const FluidEquations equations{
      // Constants.
      g,
      mu,
      // Wall boundary.
      domain,
      geom::AllInside{},
      // Weakly compressible equation of state.
      eos,
      // C4 Wendland's spline kernel.
      SixthOrderWendlandKernel{},
      gpu,
  };
  return run_integrator<Real>(opt, equations, nullptr);
}

template<class Real>
auto sph_main(int argc, char** argv) -> int {
  const Options opt = parse(argc, argv);
  constexpr Real H = 0.6;
  constexpr Real g = 9.81;
  constexpr Real rho_0 = 1000.0;
  const Real cs_0 = 20 * std::sqrt(g * H);
  if (opt.eos == "linear") {
    return sph_main_eos<Real>(opt, LinearTaitEquationOfState{cs_0, rho_0});
  }
  return sph_main_eos<Real>(opt, TaitEquationOfState{cs_0, rho_0});
}

template<class Real, class Equations>
auto run_integrator(const Options& opt, const Equations& equations,
                    const geom::Surface<Vec<Real, 2>>* domain) -> int {

  // Setup the time integrator.
  if (opt.integrator == "ssprk2") {
    return simulate<Real>(opt, equations,
                          SSPRKIntegrator{equations, SSPRKOrder::two}, domain);
  }
  if (opt.integrator == "euler") {
    return simulate<Real>(opt, equations, SymplecticEulerIntegrator{equations},
                          domain);
  }
  if (opt.integrator == "verlet") {
    return simulate<Real>(opt, equations, VelocityVerletIntegrator{equations},
                          domain);
  }
  return simulate<Real>(opt, equations,
                        SSPRKIntegrator{equations, SSPRKOrder::three}, domain);
}

template<class Real, class Equations, class Integrator>
auto simulate(const Options& opt, const Equations& equations,
              const Integrator& time_integrator,
              const geom::Surface<Vec<Real, 2>>* domain) -> int {
  constexpr Real H = 0.6;   // Water column height.
  constexpr Real L = 2 * H; // Water column length.

  constexpr Real POOL_WIDTH = 5.366 * H; // Pool width.
  constexpr Real POOL_HEIGHT = 4.0 * H;  // Pool height.

  const Real dr = H / opt.nx; // Initial particle spacing.
  const auto WATER_M = int(std::round(L / dr));
  const auto WATER_N = int(std::round(H / dr));

  constexpr Real g = 9.81;
  constexpr Real rho_0 = 1000.0;
  const Real cs_0 = 20 * std::sqrt(g * H);
  const Real h_0 = 2.0 * dr;
  const Real m_0 = rho_0 * pow2(dr);

  // Setup the particles array:
  ParticleArray particles{
      // 2D space.
      Space<Real, 2>{},
      // Set of fields is inferred from the time integrator.
      time_integrator,
  };

  // Generate individual particles.
  for (auto i = 0; i < WATER_M; ++i) {
    for (auto j = 0; j < WATER_N; ++j) {
      auto a = particles.append(ParticleType::fluid);
      r[a] = dr * Vec{i + Real{1.0}, j + Real{1.0}};
    }
  }
  if (domain != nullptr) {
    // One fixed particle per domain vertex (wcsph.cpp:109-112).
    for (std::size_t i = 0; i < domain->num_verts(); ++i) {
      auto a = particles.append(ParticleType::fixed);
      r[a] = domain->vert(i);
    }
  } else {
    // Three layers of fixed particles on the dr lattice: bottom and both
    // sides of the pool, open top.
    const auto nW = int(std::round(POOL_WIDTH / dr));
    const auto nH = int(std::round(POOL_HEIGHT / dr));
    for (auto j = -2; j <= nH; ++j) {
      for (auto i = -2; i <= nW + 2; ++i) {
        if (i > 0 && i < nW && j > 0) continue;
        auto a = particles.append(ParticleType::fixed);
        r[a] = dr * Vec{Real(i), Real(j)};
      }
    }
  }

  // Set global particle constants.
  h[particles] = h_0;
  for (const auto a : particles.all()) {
    m[a] = m_0;
    rho[a] = rho_0;
  }

  // Density hydrostatic initialization.
  for (const auto a : particles.all()) {
    if (a.has_type(ParticleType::fixed)) {
      rho[a] = rho_0;
      continue;
    }

    // Compute pressure from Poisson problem.
    const auto x = r[a][0];
    const auto y = r[a][1];
    auto p_a = rho_0 * g * (H - y);
    for (std::size_t k = 1; k < 100; k += 2) {
      constexpr auto pi = std::numbers::pi_v<Real>;
      const auto k_pi = static_cast<Real>(k) * pi;
      p_a -= 8 * rho_0 * g * H / pow2(k_pi) *
             (std::exp(k_pi * (x - L) / (2 * H)) * std::cos(k_pi * y / (2 * H)));
    }

    // Recalculate density.
    rho[a] = rho_0 + p_a / pow2(cs_0);
  }

  std::ofstream dump;
  if (!opt.dump.empty()) {
    dump.open(opt.dump, std::ios::binary);
    if (!dump) throw Exception{"cannot open " + opt.dump};
    const std::int64_t head[3] = {static_cast<std::int64_t>(particles.size()),
                                  static_cast<std::int64_t>(particles.num_fluid()),
                                  opt.steps};
    dump.write(reinterpret_cast<const char*>(head), sizeof(head));
    const double consts[5] = {h_0, m_0, rho_0, cs_0, 0.0};
    dump.write(reinterpret_cast<const char*>(consts), sizeof(consts));
    dump_state(dump, particles);
  }

  // Setup the particle mesh structure.
  ParticleMesh mesh{
      // Search for the particles using the grid search.
      geom::GridSearch{h_0},
      // Search for the boundary faces using the grid search.
      geom::GridFaceSearch{h_0},
      // Use RIB as the primary partitioning method.
      geom::RecursiveInertialBisection{},
      // Use pixelated K-means as the interface partitioning method.
      geom::PixelatedPartition{2 * h_0, geom::KMeansClustering{}},
  };

  // Initialize the particles.
  equations.initialize(mesh, particles);

  // Store only the last run, as the reference driver does.
  std::optional<data::Storage> storage;
  std::optional<data::SeriesView> series;
  if (!opt.ttdb.empty()) {
    storage.emplace(opt.ttdb);
    storage->set_max_series(1);
    series.emplace(storage->create_series());
    particles.write(0.0, *series);
  }

  // Run the simulation.
  Real time{};
  std::size_t step = 1;
  double exec_s = 0.0, print_s = 0.0;
  using clock = std::chrono::steady_clock;
  for (;; ++step) {
    const auto scaled_time = time * std::sqrt(g / H);
    if (opt.log) {
      std::printf("%15zu\t\t%10.5f\t\t%10.5f\t\t%10.5f\n", step,
                  static_cast<double>(scaled_time), exec_s, print_s);
    }
    const auto t0 = clock::now();
    const Real dt = time_integrator.step(mesh, particles);
    exec_s = std::chrono::duration<double>(clock::now() - t0).count();
    const bool end = opt.steps >= 0 ? static_cast<long>(step) >= opt.steps
                                    : scaled_time >= opt.end_time;
    if (series && ((step % 100 == 0) || end)) {
      const auto t1 = clock::now();
      particles.write(scaled_time + dt * std::sqrt(g / H), *series);
      print_s = std::chrono::duration<double>(clock::now() - t1).count();
    }
    time += dt;
    if (end) break;
  }
  if (storage) storage->wait();

  if (dump) {
    dump_state(dump, particles);
    if (domain != nullptr) {
      const std::int64_t nfaces = static_cast<std::int64_t>(domain->num_faces());
      dump.write(reinterpret_cast<const char*>(&nfaces), sizeof(nfaces));
      for (std::size_t fi = 0; fi < domain->num_faces(); ++fi) {
        for (const auto v : domain->face_verts(fi)) {
          const std::int32_t vi = static_cast<std::int32_t>(v);
          dump.write(reinterpret_cast<const char*>(&vi), sizeof(vi));
        }
      }
      const double poly[8] = {0.0, 0.0, POOL_WIDTH, 0.0, POOL_WIDTH, POOL_HEIGHT,
                              0.0, POOL_HEIGHT};
      const std::int64_t npoly = 4;
      dump.write(reinterpret_cast<const char*>(&npoly), sizeof(npoly));
      dump.write(reinterpret_cast<const char*>(poly), sizeof(poly));
    }
    dump.seekp(3 * sizeof(std::int64_t) + 4 * sizeof(double));
    const double t = time;
    dump.write(reinterpret_cast<const char*>(&t), sizeof(t));
  }
  std::printf("titwcsph_gpu: %zu steps, time %.6f, %zu particles (%zu fluid)\n",
              step, static_cast<double>(time), particles.size(),
              particles.num_fluid());
  return 0;
}

} // namespace
} // namespace tit::sph::wcsph

auto main(int argc, char** argv) -> int {
  try {
    return tit::sph::wcsph::sph_main<double>(argc, argv);
  } catch (const tit::Exception& e) {
    std::fprintf(stderr, "titwcsph_gpu: %s\n", e.what());
    return 1;
  }
}
