// A front-end style loop written against the reference's names (the shape of
// SimpleHydrology.cpp:314-356) through include/shy_world.hpp: erode, pull the
// maps, read cells.  Prints one line: frames, drop steps, height sum and the
// discharge-texture alpha sum (erf(0.4 d), SimpleHydrology.cpp:341-346).
#include <cstdio>
#include <vector>

#include "shy_world.hpp"

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 256;
  const int frames = argc > 2 ? std::atoi(argv[2]) : 10;
  const int drops = argc > 3 ? std::atoi(argv[3]) : 512;
  try {
    shy_ref::World::init(n, n, 7);
    shy_ref::check(shy_terrain_generate(shy_ref::World::map.w, 0, 7, 8));
    for (int f = 0; f < frames; ++f) {
      shy_ref::World::erode(drops);  // world.erode(quad::tilesize)
    }
    shy_ref::World::map.pull();
    double hsum = 0.0, alpha = 0.0;
    for (int x = 0; x < n; ++x)
      for (int y = 0; y < n; ++y) {
        const shy_ref::vec2 p = {(float)x, (float)y};
        hsum += shy_ref::World::map.height(p);
        alpha += shy_ref::World::map.discharge(p);
      }
    shy_stats st;
    shy_ref::check(shy_world_stats(shy_ref::World::map.w, &st));
    std::printf("{\"frames\": %d, \"drop_steps\": %llu, \"height_sum\": %.17g, \"alpha_sum\": %.17g}\n", frames,
                (unsigned long long)st.drop_steps, hsum, alpha);
    shy_ref::World::shutdown();
  } catch (const shy_ref::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 2;
  }
  return 0;
}
