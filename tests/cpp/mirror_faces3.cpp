// The C++ mirror in 3D with face walls: the titwcsph dam break extruded to
// 3D (column 2H x H x H at dr (i + 1, j + 1, k + 1), pool W x Ht x (K + 1) dr)
// set up through the reference-style API (geom::Surface of triangles,
// geom::tessellate, geom::MakeFastWinding, FluidEquations, SSPRKIntegrator,
// ParticleArray, ParticleMesh), run for a few steps on the GPU.  Writes the
// initial and final state, the face vertex triples and the containment
// triangles to argv[1] for a comparison with the oracle.
//
// Usage: mirror_faces3 OUT [--fp32c] [--nx N] [--steps S]
//
// Layout (little-endian): int64 n, n_fluid, steps; float64 h, m, rho_0,
// cs_0; r (n x 3), v (n x 3), rho (n) initial, the same final; int64
// n_faces, n_faces x 3 int32 fixed-particle indices; int64 n_tris,
// n_tris x 9 float64 containment triangles.

#include <cmath>
#include <cstdio>
#include <fstream>
#include <numbers>
#include <string>
#include <vector>

#include "titgpu.hpp"

namespace {

using namespace tit;
using namespace tit::sph;

template<class PA>
void write_state(std::ofstream& out, PA& particles) {
  const auto& cp = std::as_const(particles);
  for (std::size_t i = 0; i < cp.size(); ++i) {
    out.write(reinterpret_cast<const char*>(&cp.position(i)[0]), 3 * sizeof(double));
  }
  for (std::size_t i = 0; i < cp.size(); ++i) {
    out.write(reinterpret_cast<const char*>(&cp.velocity(i)[0]), 3 * sizeof(double));
  }
  for (std::size_t i = 0; i < cp.size(); ++i) {
    const double d = cp.density(i);
    out.write(reinterpret_cast<const char*>(&d), sizeof(double));
  }
}

// An axis-aligned box [0, X] x [0, Y] x [0, Z] as 12 triangles; outward
// normals, or inward (each triangle reversed).
auto box(double X, double Y, double Z, bool outward) -> geom::Surface<Vec<double, 3>> {
  geom::Surface<Vec<double, 3>> s;
  for (int i = 0; i < 8; ++i) {
    s.append_vert({(i & 1) ? X : 0.0, (i & 2) ? Y : 0.0, (i & 4) ? Z : 0.0});
  }
  const std::size_t quads[6][4] = {{0, 2, 3, 1}, {4, 5, 7, 6}, {0, 1, 5, 4},
                                   {2, 6, 7, 3}, {1, 3, 7, 5}, {0, 4, 6, 2}};
  for (const auto& q : quads) {
    if (outward) {
      s.append_face({q[0], q[1], q[2]});
      s.append_face({q[0], q[2], q[3]});
    } else {
      s.append_face({q[2], q[1], q[0]});
      s.append_face({q[3], q[2], q[0]});
    }
  }
  return s;
}

auto run(int argc, char** argv) -> int {
  if (argc < 2) throw Exception{"usage: mirror_faces3 OUT [--fp32c] [--nx N] [--steps S]"};
  bool fp32c = false;
  int nx = 6;
  long steps = 3;
  for (int i = 2; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--fp32c") fp32c = true;
    else if (a == "--nx" && i + 1 < argc) nx = std::stoi(argv[++i]);
    else if (a == "--steps" && i + 1 < argc) steps = std::stol(argv[++i]);
    else throw Exception{"unknown option " + a};
  }
  using Real = double;
  const Real H = 0.6, L = 2 * H;
  const Real dr = H / nx;
  const int M = static_cast<int>(std::round(L / dr));
  const int N = static_cast<int>(std::round(H / dr));
  const int K = N;
  const Real W = 3.0 * H, Ht = 1.5 * H, D = (K + 1) * dr;
  const Real g = 9.81, rho_0 = 1000.0, mu = 0.001;
  const Real cs_0 = 20 * std::sqrt(g * H);
  const Real h_0 = 1.3 * dr;
  const Real m_0 = rho_0 * dr * dr * dr;

  // Walls: the pool tessellated at dr with normals into the fluid; the
  // containment: the pool box, outward.
  const auto domain = geom::tessellate(box(W, Ht, D, false), dr);
  const geom::MakeFastWinding<Real> make_winding;
  const auto containment = make_winding(box(W, Ht, D, true));
  GpuOptions gpu;
  gpu.precision = fp32c ? Precision::fp32_compensated : Precision::fp64;
  gpu.autotune = false;
  const FluidEquations equations{g, mu, domain, containment,
                                 TaitEquationOfState{cs_0, rho_0},
                                 SixthOrderWendlandKernel{}, gpu};
  const SSPRKIntegrator integrator{equations, SSPRKOrder::three};
  ParticleArray particles{Space<Real, 3>{}, integrator};
  for (int i = 0; i < M; ++i) {
    for (int j = 0; j < N; ++j) {
      for (int k = 0; k < K; ++k) {
        auto a = particles.append(ParticleType::fluid);
        r[a] = dr * Vec{i + Real{1}, j + Real{1}, k + Real{1}};
      }
    }
  }
  for (std::size_t i = 0; i < domain.num_verts(); ++i) {
    auto a = particles.append(ParticleType::fixed);
    r[a] = domain.vert(i);
  }
  h[particles] = h_0;
  for (const auto a : particles.all()) {
    m[a] = m_0;
    rho[a] = rho_0;
    if (a.has_type(ParticleType::fixed)) continue;
    // Hydrostatic pressure of the 2D column (wcsph.cpp:123-142), constant
    // across the depth.
    const auto x = r[a][0], y = r[a][1];
    auto p_a = rho_0 * g * (H - y);
    for (std::size_t q = 1; q < 100; q += 2) {
      const auto k_pi = static_cast<Real>(q) * std::numbers::pi_v<Real>;
      p_a -= 8 * rho_0 * g * H / (k_pi * k_pi) *
             (std::exp(k_pi * (x - L) / (2 * H)) * std::cos(k_pi * y / (2 * H)));
    }
    rho[a] = rho_0 + p_a / (cs_0 * cs_0);
  }

  std::ofstream out(argv[1], std::ios::binary);
  if (!out) throw Exception{std::string{"cannot open "} + argv[1]};
  const std::int64_t head[3] = {static_cast<std::int64_t>(particles.size()),
                                static_cast<std::int64_t>(particles.num_fluid()), steps};
  out.write(reinterpret_cast<const char*>(head), sizeof(head));
  const double consts[4] = {h_0, m_0, rho_0, cs_0};
  out.write(reinterpret_cast<const char*>(consts), sizeof(consts));
  write_state(out, particles);

  ParticleMesh mesh{geom::GridSearch{h_0}, geom::GridFaceSearch{h_0},
                    geom::RecursiveInertialBisection{},
                    geom::PixelatedPartition{2 * h_0, geom::KMeansClustering{}}};
  equations.initialize(mesh, particles);
  for (long s = 0; s < steps; ++s) integrator.step(mesh, particles);

  write_state(out, particles);
  const std::int64_t nfaces = static_cast<std::int64_t>(domain.num_faces());
  out.write(reinterpret_cast<const char*>(&nfaces), sizeof(nfaces));
  for (std::size_t fi = 0; fi < domain.num_faces(); ++fi) {
    for (const auto v : domain.face_verts(fi)) {
      const std::int32_t vi = static_cast<std::int32_t>(v);
      out.write(reinterpret_cast<const char*>(&vi), sizeof(vi));
    }
  }
  const std::vector<double> tris = containment.surface_data();
  const std::int64_t ntris = static_cast<std::int64_t>(tris.size() / 9);
  out.write(reinterpret_cast<const char*>(&ntris), sizeof(ntris));
  out.write(reinterpret_cast<const char*>(tris.data()),
            static_cast<std::streamsize>(tris.size() * sizeof(double)));
  std::printf("ok %zu particles, %zu faces\n", particles.size(), domain.num_faces());
  return 0;
}

}  // namespace

auto main(int argc, char** argv) -> int {
  try {
    return run(argc, argv);
  } catch (const tit::Exception& e) {
    std::fprintf(stderr, "mirror_faces3: %s\n", e.what());
    return 1;
  }
}
