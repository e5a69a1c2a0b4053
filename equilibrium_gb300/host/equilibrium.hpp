// C++ host-side mirror of the reference's src/simulation API over the C ABI
// (include/eqfluid.h). Same names and argument meanings as the Rust crate
// vkabadzhova/equilibrium; where the reference panics this throws
// equilibrium::Panic.
//
//   configs.rs:5-60        -> SimulationConfigs, FluidConfigs (defaults kept)
//   obstacle.rs:29-87     -> Rectangle (validated in the constructor)
//   fluid.rs:10-17         -> ContainerWall
//   fluid.rs:51-620        -> Fluid (new, default, step, fill_obstacle,
//                             add_density, add_velocity, clone, pub fields)
//   renderer_helpers.rs:29-81 -> CurrentSimulation::simulate / mark_fluid_obstacles
#pragma once
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/eqfluid.h"

namespace equilibrium {

struct Panic : std::runtime_error {
  int status;
  Panic(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(int rc) {
  if (rc != EQ_OK) throw Panic(rc, eq_last_error());
}

namespace simulation {

struct SimulationConfigs {
  float delta_t = 0.02f;
  int64_t frames = 16;
  uint32_t size = 128;
  static SimulationConfigs make(float dt, int64_t frames, uint32_t size) {
    return SimulationConfigs{dt, frames, size};
  }
};

struct FluidConfigs {
  float diffusion = 0.0f;
  float viscousity = 0.001f;
  bool has_perlin_noise = true;
  uint8_t fluid_color[4] = {208, 88, 157, 220};
  uint8_t world_color[4] = {94, 146, 162, 128};
};

enum class ContainerWall : uint8_t { NoWall = 0, DefaultWall = 1 };

using Point = std::pair<int64_t, int64_t>;

class Rectangle {
 public:
  Point down_left_point, up_right_point;
  Rectangle(Point dl, Point ur, uint32_t fluid_container_size)
      : down_left_point(dl), up_right_point(ur), approximate_points_{dl, ur} {
    check(eq_rectangle_check(dl.first, dl.second, ur.first, ur.second,
                             fluid_container_size));
  }
  static Rectangle make_default() { return Rectangle({80, 80}, {110, 110}, 128); }
  const std::vector<Point>& get_approximate_points() const { return approximate_points_; }

 private:
  std::vector<Point> approximate_points_;
};

class Fluid {
 public:
  FluidConfigs fluid_configs;
  SimulationConfigs simulation_configs;

  Fluid(FluidConfigs f, SimulationConfigs s, int device = -1)
      : fluid_configs(f), simulation_configs(s) {
    eq_fluid_configs fc{f.diffusion, f.viscousity, f.has_perlin_noise ? 1 : 0};
    eq_simulation_configs sc{s.delta_t, s.frames, s.size};
    check(eq_fluid_new(&fc, &sc, device, &h_));
  }
  static Fluid make_default(int device = -1) {
    eq_fluid* h = nullptr;
    check(eq_fluid_default(device, &h));
    return Fluid(h, FluidConfigs{}, SimulationConfigs{});
  }
  Fluid(const Fluid& o) : fluid_configs(o.fluid_configs), simulation_configs(o.simulation_configs) {
    check(eq_fluid_clone(o.h_, &h_));
  }
  Fluid(Fluid&& o) noexcept
      : fluid_configs(o.fluid_configs), simulation_configs(o.simulation_configs), h_(o.h_) {
    o.h_ = nullptr;
  }
  Fluid& operator=(const Fluid&) = delete;
  ~Fluid() { eq_fluid_free(h_); }

  void step() {
    push_configs();
    check(eq_fluid_step(h_));
  }
  void fill_obstacle(const Rectangle& r) {
    const auto& p = r.get_approximate_points();
    check(eq_fluid_fill_obstacle(h_, p[0].first, p[0].second, p[1].first, p[1].second));
  }
  void add_density(uint32_t x, uint32_t y, float amount) {
    check(eq_fluid_add_density(h_, x, y, amount));
  }
  void add_velocity(uint32_t x, uint32_t y, float ax, float ay) {
    check(eq_fluid_add_velocity(h_, x, y, ax, ay));
  }
  std::vector<float> density() const { return field(EQ_FIELD_DENSITY); }
  std::vector<float> velocities_x() const { return field(EQ_FIELD_VX); }
  std::vector<float> velocities_y() const { return field(EQ_FIELD_VY); }
  std::vector<ContainerWall> cells_type() const {
    std::vector<uint8_t> raw((size_t)simulation_configs.size * simulation_configs.size);
    check(eq_fluid_read_cells(h_, raw.data(), raw.size()));
    std::vector<ContainerWall> out(raw.size());
    for (size_t q = 0; q < raw.size(); ++q)
      out[q] = raw[q] ? ContainerWall::DefaultWall : ContainerWall::NoWall;
    return out;
  }
  eq_fluid* handle() const { return h_; }

 private:
  Fluid(eq_fluid* h, FluidConfigs f, SimulationConfigs s)
      : fluid_configs(f), simulation_configs(s), h_(h) {}
  void push_configs() {
    eq_fluid_configs fc{fluid_configs.diffusion, fluid_configs.viscousity,
                        fluid_configs.has_perlin_noise ? 1 : 0};
    eq_simulation_configs sc{simulation_configs.delta_t, simulation_configs.frames,
                             simulation_configs.size};
    check(eq_fluid_set_configs(h_, &fc, &sc));
  }
  std::vector<float> field(int f) const {
    std::vector<float> out((size_t)simulation_configs.size * simulation_configs.size);
    check(eq_fluid_read_field(h_, f, out.data(), out.size()));
    return out;
  }
  eq_fluid* h_ = nullptr;
};

struct FluidStep {
  Fluid fluid;
  int64_t frame_number;
};

struct CurrentSimulation {
  Fluid fluid;
  std::vector<Rectangle> obstacles;

  void mark_fluid_obstacles() {
    for (const auto& o : obstacles) fluid.fill_obstacle(o);
  }
  // renderer_helpers.rs:52-72; noise is applied by the caller's hook when
  // has_perlin_noise is set (the reference draws it from thread_rng).
  void simulate(const std::function<void(FluidStep&&)>& tx,
                const std::function<void(Fluid&)>& add_noise = nullptr) {
    mark_fluid_obstacles();
    for (int64_t i = 0; i < fluid.simulation_configs.frames; ++i) {
      if (fluid.fluid_configs.has_perlin_noise && add_noise) add_noise(fluid);
      fluid.step();
      tx(FluidStep{Fluid(fluid), i});
    }
  }
};

}  // namespace simulation
}  // namespace equilibrium
