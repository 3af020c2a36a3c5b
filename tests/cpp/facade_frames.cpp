// The reference's frame loop in its own random sequence through
// include/shy_world.hpp: srand(seed), then frames of World::erode(drops) with
// rand() spawns and Vegetation::grow() (SimpleHydrology.cpp:318-320).
// Arguments: map side, frames, drops per frame, seed; the library generates
// the terrain (value noise, seed 4).  Prints the plant list and the height
// sum as one JSON line.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "shy_world.hpp"

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 96;
  const int frames = argc > 2 ? std::atoi(argv[2]) : 30;
  const int drops = argc > 3 ? std::atoi(argv[3]) : 40;
  const unsigned seed = argc > 4 ? (unsigned)std::atoi(argv[4]) : 3u;
  try {
    shy_ref::World::init(n, n, 1);
    shy_ref::check(shy_terrain_generate(shy_ref::World::map.w, 0, 4, 8));
    shy_ref::World::srand(seed);
    for (int f = 0; f < frames; ++f) {
      shy_ref::World::erode_sequential(drops);
      shy_ref::Vegetation::grow();
    }
    const std::vector<shy_ref::Plant> plants = shy_ref::Vegetation::plants();
    shy_ref::World::map.pull();
    double hsum = 0.0;
    for (int x = 0; x < n; ++x)
      for (int y = 0; y < n; ++y) hsum += shy_ref::World::map.height({(float)x, (float)y});
    std::printf("{\"height_sum\": %.17g, \"plants\": [", hsum);
    for (size_t i = 0; i < plants.size(); ++i)
      std::printf("%s[%.9g, %.9g, %.9g]", i ? ", " : "", plants[i].pos.x, plants[i].pos.y, plants[i].size);
    std::printf("]}\n");
    shy_ref::World::shutdown();
  } catch (const shy_ref::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 2;
  }
  return 0;
}
