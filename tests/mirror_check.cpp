// The reference's own unit tests, restated against the C++ host mirror:
//   renderer_helpers.rs:222-252  mark_fluid_obstacles_default_current_simulation (1408 walls)
//   obstacle.rs:97-115           rectangle_wrong_parameters / swapped_parameters panic
// plus one frame loop of renderer_helpers.rs:52-72. Needs a GPU (Fluid owns
// device state). Exit status 0 = all checks passed.
#include <cstdio>

#include "equilibrium.hpp"

using namespace equilibrium::simulation;

static int fails = 0;
#define EXPECT(c)                                              \
  do {                                                         \
    if (!(c)) {                                                \
      std::printf("FAILED: %s (line %d)\n", #c, __LINE__);     \
      ++fails;                                                 \
    }                                                          \
  } while (0)

int main() {
  // obstacle.rs:97-115
  bool panicked = false;
  try {
    Rectangle({50, 120}, {127, 110}, 128);
  } catch (const equilibrium::Panic&) {
    panicked = true;
  }
  EXPECT(panicked);
  panicked = false;
  try {
    Rectangle({12, 12}, {10, 10}, 128);
  } catch (const equilibrium::Panic&) {
    panicked = true;
  }
  EXPECT(panicked);

  // renderer_helpers.rs:222-252
  CurrentSimulation cs{Fluid::make_default(0), {Rectangle::make_default()}};
  cs.mark_fluid_obstacles();
  size_t walls = 0;
  for (auto c : cs.fluid.cells_type()) walls += (c == ContainerWall::DefaultWall);
  const uint32_t size = cs.fluid.simulation_configs.size;
  EXPECT(walls == 2 * (size + (size - 2)) + 30 * 30);

  // a short frame loop with noise off: one snapshot per frame
  cs.fluid.fluid_configs.has_perlin_noise = false;
  cs.fluid.simulation_configs.frames = 3;
  int64_t last = -1;
  cs.simulate([&](FluidStep&& st) {
    EXPECT(st.frame_number == last + 1);
    last = st.frame_number;
    EXPECT(st.fluid.density().size() == (size_t)size * size);
  });
  EXPECT(last == 2);
  std::printf(fails ? "mirror_check: %d failure(s)\n" : "mirror_check: ok\n", fails);
  return fails ? 1 : 0;
}
