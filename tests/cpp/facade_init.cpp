// World::init through the facade (include/shy_world.hpp) starts from the
// reference's own terrain, as World::map.init does (source/cellpool.h:323).
// Writes the nx x ny heights, x-major float32, to the file named by argv[4].
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "shy_world.hpp"

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]);
  const unsigned seed = (unsigned)std::strtol(argv[3], nullptr, 10);
  try {
    shy_ref::World::init(nx, ny, seed);
    shy_ref::World::map.pull();
    std::vector<float> h((size_t)nx * ny);
    for (int x = 0; x < nx; ++x)
      for (int y = 0; y < ny; ++y) h[(size_t)x * ny + y] = shy_ref::World::map.height({(float)x, (float)y});
    std::FILE* f = std::fopen(argv[4], "wb");
    if (!f || std::fwrite(h.data(), sizeof(float), h.size(), f) != h.size()) return 3;
    std::fclose(f);
    shy_ref::World::shutdown();
  } catch (const shy_ref::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 2;
  }
  return 0;
}
