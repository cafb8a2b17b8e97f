// Host-only checks of the C++ mirror (titgpu.hpp) and the .ttdb writer
// (titgpu_data.hpp); no kernel runs.  Writes a storage to argv[1] for the
// Python side to read back.  Prints "ok" and exits 0 when every check holds.

#include <array>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "titgpu.hpp"
#include "titgpu_data.hpp"

using namespace tit;
using namespace tit::sph;

#define CHECK(cond)                                                   \
  do {                                                                \
    if (!(cond)) {                                                    \
      std::fprintf(stderr, "check failed at line %d: %s\n", __LINE__, \
                   #cond);                                            \
      return 1;                                                       \
    }                                                                 \
  } while (0)

template<class F>
auto throws(F&& f) -> bool {
  try {
    f();
  } catch (const Exception&) {
    return true;
  }
  return false;
}

auto main(int argc, char** argv) -> int {
  if (argc < 2) return 2;

  // Vec arithmetic and deduction.
  const Vec a{1.0, 2.0};
  const Vec b = 2.0 * a + Vec{0.5, 0.25};
  CHECK(b[0] == 2.5 && b[1] == 4.25);
  static_assert(std::is_same_v<decltype(Vec{1.0, 2.0, 3.0}), Vec<double, 3>>);

  // Equations, integrator and array types as a driver spells them.
  const geom::Surface<Vec<double, 2>> domain;
  const FluidEquations equations{9.81, 0.001, domain, geom::AllInside{},
                                 TaitEquationOfState{20.0, 1000.0},
                                 QuarticWendlandKernel{}};
  const SSPRKIntegrator rk3{equations, SSPRKOrder::three};
  const SSPRKIntegrator rk2{equations, SSPRKOrder::two};
  CHECK(rk3.gpu_integrator() == TG_SSPRK3 && rk2.gpu_integrator() == TG_SSPRK2);
  CHECK(SymplecticEulerIntegrator{equations}.gpu_integrator() == TG_EULER);
  CHECK(VelocityVerletIntegrator{equations}.gpu_integrator() == TG_VERLET);
  ParticleArray particles{Space<double, 2>{}, rk3};
  static_assert(std::is_same_v<decltype(particles), ParticleArray<double, 2>>);

  // Fluid particles go before the fixed ones, whatever the append order.
  auto w0 = particles.append(ParticleType::fixed);
  r[w0] = Vec{-1.0, -1.0};
  auto f0 = particles.append(ParticleType::fluid);
  r[f0] = Vec{0.5, 0.5};
  auto f1 = particles.append(ParticleType::fluid);
  r[f1] = Vec{0.75, 0.5};
  CHECK(particles.size() == 3 && particles.num_fluid() == 2);
  CHECK(particles.position(0) == (Vec{0.5, 0.5}));
  CHECK(particles.position(1) == (Vec{0.75, 0.5}));
  CHECK(particles.position(2) == (Vec{-1.0, -1.0}));
  std::size_t nfix = 0;
  for (const auto p : particles.fixed()) {
    CHECK(p.has_type(ParticleType::fixed));
    ++nfix;
  }
  CHECK(nfix == 1);
  h[particles] = 0.1;
  for (const auto p : particles.all()) {
    m[p] = 1.0;
    rho[p] = 1000.0;
    CHECK(h[p] == 0.1);
  }

  // A surface with faces is refused (the GPU path has particle walls only).
  geom::Surface<Vec<double, 2>> faces;
  faces.append_vert({0.0, 0.0});
  faces.append_vert({1.0, 0.0});
  faces.append_face({0, 1});
  CHECK(throws([&] {
    FluidEquations bad{9.81, 0.001, faces, geom::AllInside{},
                       TaitEquationOfState{20.0, 1000.0},
                       QuarticWendlandKernel{}};
  }));
  CHECK(throws([] { TaitEquationOfState{-1.0, 1000.0}; }));
  {
    // The reference's other equation of state (equation_of_state.hpp:78-122).
    const LinearTaitEquationOfState lin{20.0, 1000.0};
    CHECK(lin.pressure_from_density(1001.0) == 400.0 * 1.0);
    CHECK(lin.sound_speed_from_density(1100.0) == 20.0);
    CHECK(lin.density_from_pressure(400.0) == 1001.0);
    const FluidEquations linear{9.81, 0.001, domain, geom::AllInside{}, lin,
                                QuarticWendlandKernel{}};
    CHECK(linear.eos().cs_0() == 20.0);
    CHECK(throws([] { LinearTaitEquationOfState{20.0, -1.0}; }));
  }

  // Face walls: tessellation as the reference splits faces and the
  // winding-number containment.
  {
    geom::Surface<Vec<double, 2>> pool;
    pool.append_vert({0.0, 1.0});
    pool.append_vert({2.0, 1.0});
    pool.append_vert({2.0, 0.0});
    pool.append_vert({0.0, 0.0});
    pool.append_face({0, 1});
    pool.append_face({1, 2});
    pool.append_face({2, 3});
    pool.append_face({3, 0});
    const auto t = geom::tessellate(pool, 0.25);
    CHECK(t.num_verts() == 24 && t.num_faces() == 24);
    CHECK(t.vert(4) == (Vec{0.25, 1.0}));  // first new vertex of face 0-1
    geom::Surface<Vec<double, 2>> ccw;
    ccw.append_vert({0.0, 0.0});
    ccw.append_vert({2.0, 0.0});
    ccw.append_vert({2.0, 1.0});
    ccw.append_vert({0.0, 1.0});
    for (std::size_t i = 0; i < 4; ++i) ccw.append_face({i, (i + 1) % 4});
    const geom::MakeFastWinding<double> make_winding;
    const auto inside = make_winding(ccw);
    CHECK(inside.contains(Vec{1.0, 0.5}) && !inside.contains(Vec{3.0, 0.5}));
    CHECK(inside.polygon().size() == 8);
    const FluidEquations faced{9.81, 0.001, t, inside,
                               TaitEquationOfState{20.0, 1000.0},
                               SixthOrderWendlandKernel{}};
    (void)faced;
    // Faces need a polygon containment: an all-inside functor is refused.
    CHECK(throws([&] {
      FluidEquations bad{9.81, 0.001, t, geom::AllInside{},
                         TaitEquationOfState{20.0, 1000.0}, SixthOrderWendlandKernel{}};
    }));
  }
  // geom::tessellate against the reference's known answers
  // (geom/tessellation.test.cpp): a 3-4-5 triangle outline at d_max = 1, and
  // red refinement of a tetrahedron at d_max = 2, uniform and with the z edge
  // twice as long (vertex order and face order included).
  {
    const auto same_verts = [](const auto& surf, const auto& want) {
      if (surf.num_verts() != want.size()) return false;
      for (std::size_t i = 0; i < want.size(); ++i) {
        for (std::size_t k = 0; k < want[i].size(); ++k) {
          if (std::abs(surf.vert(i)[k] - want[i][k]) > 1e-12) return false;
        }
      }
      return true;
    };
    const auto same_faces = [](const auto& surf, const auto& want) {
      if (surf.num_faces() != want.size()) return false;
      for (std::size_t i = 0; i < want.size(); ++i) {
        const auto f = surf.face_verts(i);
        for (std::size_t k = 0; k < want[i].size(); ++k) {
          if (f[k] != want[i][k]) return false;
        }
      }
      return true;
    };
    geom::Surface<Vec<double, 2>> tri;
    tri.append_vert({0.0, 0.0});
    tri.append_vert({3.0, 0.0});
    tri.append_vert({0.0, 4.0});
    tri.append_face({0, 1});
    tri.append_face({1, 2});
    tri.append_face({2, 0});
    const auto t2 = geom::tessellate(tri, 1.0);
    const std::vector<std::array<double, 2>> v2 = {
        {0.0, 0.0}, {3.0, 0.0}, {0.0, 4.0}, {1.0, 0.0}, {2.0, 0.0}, {2.4, 0.8},
        {1.8, 1.6}, {1.2, 2.4}, {0.6, 3.2}, {0.0, 3.0}, {0.0, 2.0}, {0.0, 1.0}};
    const std::vector<std::array<std::size_t, 2>> f2 = {
        {0, 3}, {3, 4}, {4, 1}, {1, 5}, {5, 6}, {6, 7},
        {7, 8}, {8, 2}, {2, 9}, {9, 10}, {10, 11}, {11, 0}};
    CHECK(same_verts(t2, v2) && same_faces(t2, f2));
    const auto tetra = [](double z) {
      geom::Surface<Vec<double, 3>> t;
      t.append_vert({0.0, 0.0, 0.0});
      t.append_vert({2.0, 0.0, 0.0});
      t.append_vert({0.0, 2.0, 0.0});
      t.append_vert({0.0, 0.0, z});
      t.append_face({0, 2, 1});
      t.append_face({0, 1, 3});
      t.append_face({0, 3, 2});
      t.append_face({1, 2, 3});
      return t;
    };
    const auto u = geom::tessellate(tetra(2.0), 2.0);
    const std::vector<std::array<double, 3>> uv = {
        {0.0, 0.0, 0.0}, {2.0, 0.0, 0.0}, {0.0, 2.0, 0.0}, {0.0, 0.0, 2.0},
        {1.0, 1.0, 0.0}, {1.0, 0.0, 1.0}, {0.0, 1.0, 1.0}};
    const std::vector<std::array<std::size_t, 3>> uf = {
        {2, 4, 0}, {4, 1, 0}, {1, 5, 0}, {5, 3, 0}, {3, 6, 0},
        {6, 2, 0}, {1, 4, 5}, {4, 2, 6}, {5, 6, 3}, {4, 6, 5}};
    CHECK(same_verts(u, uv) && same_faces(u, uf));
    const auto zl = geom::tessellate(tetra(4.0), 2.0);
    const std::vector<std::array<double, 3>> zv = {
        {0.0, 0.0, 0.0}, {2.0, 0.0, 0.0}, {0.0, 2.0, 0.0}, {0.0, 0.0, 4.0},
        {1.0, 1.0, 0.0}, {1.0, 0.0, 2.0}, {0.0, 0.0, 2.0}, {0.0, 1.0, 2.0},
        {1.5, 0.0, 1.0}, {0.5, 0.0, 1.0}, {0.5, 0.0, 3.0}, {0.0, 1.0, 1.0},
        {0.0, 1.5, 1.0}, {0.0, 0.5, 3.0}, {1.0, 0.5, 1.0}, {0.5, 1.0, 1.0}};
    const std::vector<std::array<std::size_t, 3>> zf = {
        {2, 4, 0},   {4, 1, 0},   {1, 8, 0},   {8, 9, 0},   {8, 5, 9},   {0, 9, 6},
        {9, 5, 6},   {5, 10, 6},  {10, 3, 6},  {6, 11, 0},  {11, 2, 0},  {7, 12, 6},
        {12, 11, 6}, {12, 2, 11}, {3, 13, 6},  {13, 7, 6},  {4, 14, 1},  {14, 8, 1},
        {14, 5, 8},  {2, 12, 4},  {12, 15, 4}, {12, 7, 15}, {7, 13, 5},  {13, 10, 5},
        {13, 3, 10}, {5, 14, 7},  {14, 15, 7}, {14, 4, 15}};
    CHECK(same_verts(zl, zv) && same_faces(zl, zf));
  }

  // Winding containment against the reference's known answers
  // (geom/winding.test.cpp): the unit square with its faces listed forwards
  // and backwards (the same counter-clockwise loop), the outward tetrahedron
  // and its reversal, coarse and tessellated at 0.05; a degenerate pair of
  // faces winds 0.
  {
    const geom::MakeFastWinding<double> make_winding;
    const auto square = [](bool reverse) {
      geom::Surface<Vec<double, 2>> s;
      s.append_vert({0.0, 0.0});
      s.append_vert({1.0, 0.0});
      s.append_vert({1.0, 1.0});
      s.append_vert({0.0, 1.0});
      if (reverse) {
        s.append_face({3, 0});
        s.append_face({2, 3});
        s.append_face({1, 2});
        s.append_face({0, 1});
      } else {
        s.append_face({0, 1});
        s.append_face({1, 2});
        s.append_face({2, 3});
        s.append_face({3, 0});
      }
      return s;
    };
    const auto tetra = [](bool reverse) {
      geom::Surface<Vec<double, 3>> s;
      s.append_vert({0.0, 0.0, 0.0});
      s.append_vert({1.0, 0.0, 0.0});
      s.append_vert({0.0, 1.0, 0.0});
      s.append_vert({0.0, 0.0, 1.0});
      if (reverse) {
        s.append_face({0, 1, 2});
        s.append_face({0, 3, 1});
        s.append_face({0, 2, 3});
        s.append_face({1, 3, 2});
      } else {
        s.append_face({0, 2, 1});
        s.append_face({0, 1, 3});
        s.append_face({0, 3, 2});
        s.append_face({1, 2, 3});
      }
      return s;
    };
    for (const bool reverse : {false, true}) {
      const double sign = reverse ? -1.0 : 1.0;
      for (const auto& sq : {square(reverse), geom::tessellate(square(reverse), 0.05)}) {
        const auto w = make_winding(sq);
        CHECK(std::abs(w(Vec{0.5, 0.5}) - 1.0) < 1e-12);
        CHECK(std::abs(w(Vec{0.1, 0.1}) - 1.0) < 1e-12);
        CHECK(std::abs(w(Vec{1.5, 0.5})) < 1e-12 && std::abs(w(Vec{100.0, 100.0})) < 1e-12);
        CHECK(w.contains(Vec{0.9, 0.75}));
        CHECK(w.surface_data().size() == 2 * sq.num_faces());
      }
      for (const auto& te : {tetra(reverse), geom::tessellate(tetra(reverse), 0.05)}) {
        const auto w = make_winding(te);
        CHECK(std::abs(w(Vec{0.25, 0.25, 0.25}) - sign) < 1e-12);
        CHECK(std::abs(w(Vec{0.1, 0.1, 0.1}) - sign) < 1e-12);
        CHECK(std::abs(w(Vec{1.0, 1.0, 1.0})) < 1e-12);
        CHECK(std::abs(w(Vec{3.0, 2.0, 1.0})) < 1e-12);
        CHECK(w.contains(Vec{0.25, 0.25, 0.25}) == !reverse);
        CHECK(!w.contains(Vec{100.0, 100.0, 100.0}));
      }
    }
    geom::Surface<Vec<double, 3>> flat;
    flat.append_vert({0.0, 0.0, 0.0});
    flat.append_vert({1.0, 0.0, 0.0});
    flat.append_vert({2.0, 0.0, 0.0});
    flat.append_face({0, 1, 2});
    flat.append_face({2, 1, 0});
    CHECK(std::abs(make_winding(flat)(Vec{0.0, 1.0, 0.0})) < 1e-12);
    CHECK(std::abs(make_winding(geom::Surface<Vec<double, 2>>{})(Vec{0.0, 0.0})) < 1e-12);
  }

  // 3D face walls: red refinement of a box keeps it closed and oriented,
  // with every edge at most d_max; the winding number of the outward box.
  {
    geom::Surface<Vec<double, 3>> box;
    const double X = 2.0, Y = 1.0, Z = 0.5;
    for (int i = 0; i < 8; ++i) {
      box.append_vert({(i & 1) ? X : 0.0, (i & 2) ? Y : 0.0, (i & 4) ? Z : 0.0});
    }
    // Outward quads split into two triangles each.
    const std::size_t quads[6][4] = {{0, 2, 3, 1}, {4, 5, 7, 6}, {0, 1, 5, 4},
                                     {2, 6, 7, 3}, {1, 3, 7, 5}, {0, 4, 6, 2}};
    for (const auto& q : quads) {
      box.append_face({q[0], q[1], q[2]});
      box.append_face({q[0], q[2], q[3]});
    }
    const geom::MakeFastWinding<double> make_winding;
    const auto inside = make_winding(box);
    CHECK(inside.contains(Vec{1.0, 0.5, 0.25}) && !inside.contains(Vec{2.5, 0.5, 0.25}));
    CHECK(std::abs(inside(Vec{1.0, 0.5, 0.25}) - 1.0) < 1e-12);
    CHECK(inside.surface_data().size() == 12 * 9);
    const auto t = geom::tessellate(box, 0.3);
    CHECK(t.num_verts() > 8 && t.num_faces() > 12);
    std::map<std::pair<std::size_t, std::size_t>, int> edges;
    double area = 0.0;
    for (std::size_t fi = 0; fi < t.num_faces(); ++fi) {
      const auto f = t.face_verts(fi);
      for (int k = 0; k < 3; ++k) {
        const auto d = t.vert(f[(k + 1) % 3]) - t.vert(f[k]);
        CHECK(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] <= 0.3 * 0.3);
        ++edges[{f[k], f[(k + 1) % 3]}];
      }
      const auto u = t.vert(f[1]) - t.vert(f[0]), v = t.vert(f[2]) - t.vert(f[0]);
      const double cx = u[1] * v[2] - u[2] * v[1], cy = u[2] * v[0] - u[0] * v[2],
                   cz = u[0] * v[1] - u[1] * v[0];
      area += std::sqrt(cx * cx + cy * cy + cz * cz) / 2.0;
    }
    for (const auto& [e, n] : edges) CHECK(n == 1 && edges.count({e.second, e.first}) == 1);
    CHECK(std::abs(area - 2.0 * (X * Y + X * Z + Y * Z)) < 1e-12);
    CHECK(std::abs(make_winding(t)(Vec{1.0, 0.5, 0.25}) - 1.0) < 1e-12);
  }
  CHECK(throws([] { geom::GridSearch{0.0}; }));
  // A k-d tree search selects the default GPU grid (same neighbour sets).
  CHECK(ParticleMesh{geom::kd_tree_indexing}.spacing() == 0.0);
  {
    const ParticleMesh kd_mesh{geom::KDTreeSearch{}, geom::GridFaceSearch{0.1}};
    CHECK(kd_mesh.spacing() == 0.0);
  }

  // A fluid particle outside the containment is refused before any device
  // call; mixed masses too.
  const auto outside = [](const Vec<double, 2>& x) { return x[0] < 0.6; };
  const FluidEquations fenced{9.81, 0.001, domain, outside,
                              TaitEquationOfState{20.0, 1000.0},
                              QuarticWendlandKernel{}};
  ParticleMesh mesh{geom::GridSearch{0.1}};
  CHECK(throws([&] { fenced.initialize(mesh, particles); }));
  m[f1] = 2.0;
  CHECK(throws([&] { particles.attach_(tg_params{}, 1000.0, 20.0, true, false); }));
  m[f1] = 1.0;

  // .ttdb writer: two series with max_series 1 keeps the last one; frames
  // and arrays of every kind the particle writer uses.
  {
    data::Storage storage{argv[1]};
    storage.set_max_series(1);
    (void)storage.create_series("first");
    const auto series = storage.create_series("second");
    CHECK(storage.num_series() == 1);
    CHECK(storage.max_series() == 1);
    const auto frame = series.create_frame(0.0);
    const std::vector<Vec<double, 2>> rs{{1.0, 2.0}, {3.0, 4.0}, {5.0, 6.0}};
    frame.write_array("r", std::span<const Vec<double, 2>>{rs});
    const std::vector<double> dens{1000.0, 1001.5, 999.25};
    frame.write_array("rho", std::span<const double>{dens});
    const std::vector<float> f32{1.5f, -2.0f};
    frame.write_array("f32", std::span<const float>{f32});
    const std::vector<std::int32_t> ids{7, 8, 9, 10};
    frame.write_array("ids", std::span<const std::int32_t>{ids});
    // A payload over one 128 KiB block.
    std::vector<double> big(40000);
    for (std::size_t i = 0; i < big.size(); ++i) big[i] = 0.5 * double(i);
    frame.write_array("big", std::span<const double>{big});
    const std::vector<double> none;
    frame.write_array("empty", std::span<const double>{none});
    // Background frame write, then a time that does not increase.
    std::vector<data::ArrayBlob> arrays;
    arrays.push_back(data::ArrayBlob::of(std::string{"rho"},
                                         std::span<const double>{dens}));
    storage.write_frame_async(series.id(), 0.5, std::move(arrays));
    CHECK(series.num_frames() == 2);
    CHECK(throws([&] { (void)series.create_frame(0.25); }));
  }
  std::printf("ok\n");
  return 0;
}
