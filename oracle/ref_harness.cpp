// ref_harness.cpp -- test infrastructure, not product code.
//
// Compiles the UNMODIFIED erosion headers of the reference (source/world.h,
// which pulls in source/cellpool.h, source/water.h, source/vegetation.h,
// source/include/math.h and source/include/FastNoiseLite.h) against the
// glm subset in glm_subset.h and a no-op vertex pool, and exposes the
// reference's own erosion entry points through a small C ABI so that tests
// can pin the CPU restatement in hydro_oracle.cpp against it.
//
// The include path to the reference's source/ directory is given on the
// compiler command line (see oracle/Makefile); nothing from the reference is
// copied. The reference's map size is the compile-time constant
// quad::tilesize (source/cellpool.h:167), 512 x 512.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <iostream>
#include <sys/types.h>
#include <vector>

#include "glm_subset.h"

using namespace std;
using namespace glm;

// Stand-ins for the render-side types that source/cellpool.h:252-340 calls
// while building its map (the reference gets these from TinyEngine).  fill()
// records the vertex that updatenode (source/cellpool.h:286-317) writes, 12
// floats per vertex index, when a recording buffer is set.
struct Vertex {
  Vertex(vec3, vec3, vec3, vec3) {}
};
float* g_fill_out = nullptr;
int g_fill_max = 0;
template <typename T> struct Vertexpool {
  std::vector<uint> indices;
  uint slot = 0;
  uint* section(size_t, int, glm::vec3, size_t) { return &slot; }
  void resize(uint*, size_t) {}
  void index() {}
  void update() {}
  void fill(uint*, int i, vec3 p, vec3 n, vec3 t, vec3 b) {
    if (!g_fill_out || i < 0 || i >= g_fill_max) return;
    float* o = g_fill_out + 12 * (size_t)i;
    const vec3 v[4] = {p, n, t, b};
    for (int k = 0; k < 4; ++k) {
      o[3 * k] = v[k].x;
      o[3 * k + 1] = v[k].y;
      o[3 * k + 2] = v[k].z;
    }
  }
};

#include "world.h"

namespace {
mappool::pool<quad::cell> g_cellpool;
Vertexpool<Vertex> g_vertexpool;
bool g_ready = false;

float* field_ptr(quad::cell* c, int field) {
  switch (field) {
    case 0: return &c->height;
    case 1: return &c->discharge;
    case 2: return &c->momentumx;
    case 3: return &c->momentumy;
    case 4: return &c->discharge_track;
    case 5: return &c->momentumx_track;
    case 6: return &c->momentumy_track;
    default: return &c->rootdensity;
  }
}
}  // namespace

extern "C" {

int ref_tilesize() { return quad::tilesize; }

// World::map.init (source/cellpool.h:323) builds the map once per process;
// the noise terrain it generates is overwritten by ref_set_field afterwards.
int ref_init(unsigned seed) {
  if (g_ready) return 0;
  std::streambuf* saved = std::cout.rdbuf(nullptr);  // init prints progress
  World::SEED = seed;
  g_cellpool.reserve(quad::area);
  World::map.init(g_vertexpool, g_cellpool, seed);
  std::cout.rdbuf(saved);
  g_ready = true;
  return 0;
}

// field: 0 height, 1 discharge, 2 momentumx, 3 momentumy, 4..6 tracks,
// 7 rootdensity.  Arrays are x-major: index = x * size + y
// (math::flatten, source/include/math.h:11-14).
void ref_set_field(int field, const float* src) {
  const int n = quad::size;
  for (int x = 0; x < n; ++x)
    for (int y = 0; y < n; ++y)
      *field_ptr(World::map.getCell(ivec2(x, y)), field) = src[(size_t)x * n + y];
}

void ref_get_field(int field, float* dst) {
  const int n = quad::size;
  for (int x = 0; x < n; ++x)
    for (int y = 0; y < n; ++y)
      dst[(size_t)x * n + y] = *field_ptr(World::map.getCell(ivec2(x, y)), field);
}

void ref_srand(unsigned s) { srand(s); }
int ref_rand() { return rand(); }

// 0 if ivec2(rand()%a, rand()%b) draws its x first (left to right), 1 if y
// first; source/world.h:69 leaves this to the compiler.
int ref_spawn_arg_order() {
  srand(12345u);
  ivec2 v(rand() % 1000003, rand() % 1000003);
  srand(12345u);
  int first = rand() % 1000003;
  return v.x == first ? 0 : 1;
}

// World::erode(cycles), source/world.h:54-88.
void ref_erode(int cycles) { World::erode(cycles); }

// World::cascade(pos), source/world.h:90-168.
void ref_cascade(float x, float y) { World::cascade(vec2(x, y)); }

// quad::map::normal(p), source/cellpool.h:445 -> _normal :182-204.
void ref_normal(int x, int y, float* out3) {
  vec3 n = World::map.normal(ivec2(x, y));
  out3[0] = n.x;
  out3[1] = n.y;
  out3[2] = n.z;
}

// One droplet: Drop d(pos); while (d.descend()); (source/world.h:74-76),
// recording the state after every descend() call as 8 floats:
// returned, age, pos.x, pos.y, speed.x, speed.y, volume, sediment.
int ref_descend_trace(float px, float py, float* out, int max_records) {
  Drop d(vec2(px, py));
  int n = 0;
  for (;;) {
    bool more = d.descend();
    if (n < max_records) {
      float* r = out + 8 * (size_t)n;
      r[0] = more ? 1.0f : 0.0f;
      r[1] = (float)d.age;
      r[2] = d.pos.x;
      r[3] = d.pos.y;
      r[4] = d.speed.x;
      r[5] = d.speed.y;
      r[6] = d.volume;
      r[7] = d.sediment;
    }
    ++n;
    if (!more) break;
  }
  return n;
}

// Vegetation::grow(), source/vegetation.h:122-188. Returns the plant count.
int ref_veg_grow() {
  Vegetation::grow();
  return (int)Vegetation::plants.size();
}

void ref_veg_clear() { Vegetation::plants.clear(); }

// Plants as (pos.x, pos.y, size) triples, in list order.
int ref_veg_get(float* out, int max_plants) {
  int n = (int)Vegetation::plants.size();
  for (int i = 0; i < n && i < max_plants; ++i) {
    out[3 * i + 0] = Vegetation::plants[i].pos.x;
    out[3 * i + 1] = Vegetation::plants[i].pos.y;
    out[3 * i + 2] = Vegetation::plants[i].size;
  }
  return n;
}

// The front end's per-frame data (SimpleHydrology.cpp:322-355): the mesh
// through the reference's own updatenode (its vertex index is
// math::flatten(pos, tileres), x-major like the maps), and the two texture
// lambdas of SimpleHydrology.cpp:341-354 (which need TinyEngine to compile)
// restated over the reference's map accessors, with waterColor of
// source/model.h:22.
void ref_frame(float* vert12, float* dis4, float* mom4) {
  const int n = quad::tilesize * quad::tilesize;
  g_fill_out = vert12;
  g_fill_max = n;
  for (auto& node : World::map.nodes) updatenode(g_vertexpool, node);
  g_fill_out = nullptr;
  const vec3 waterColor = vec3(92, 133, 142) / 255.0f;
  for (int x = 0; x < quad::tilesize; ++x)
    for (int y = 0; y < quad::tilesize; ++y) {
      const ivec2 p(x, y);
      const size_t i = (size_t)x * quad::tilesize + y;
      double d = World::map.discharge(p);
      const vec4 dc = vec4(waterColor, d);
      auto node = World::map.get(p);
      auto cell = node->get(p);
      float mx = cell->momentumx;
      float my = cell->momentumy;
      const vec4 mc = vec4(0.5f * (1.0f + erf(mx)), 0.5f * (1.0f + erf(my)), 0.5f, 1.0);
      dis4[4 * i] = dc.x; dis4[4 * i + 1] = dc.y; dis4[4 * i + 2] = dc.z; dis4[4 * i + 3] = dc.w;
      mom4[4 * i] = mc.x; mom4[4 * i + 1] = mc.y; mom4[4 * i + 2] = mc.z; mom4[4 * i + 3] = mc.w;
    }
}

}  // extern "C"
