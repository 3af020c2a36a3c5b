// shy_world.hpp -- header-only C++ facade over the C ABI in shy.h with the
// reference's erosion names, so that a front-end loop written against the
// reference (SimpleHydrology.cpp:314-356: world.erode(quad::tilesize);
// Vegetation::grow(); reads of map cells) keeps its shape:
//
//   shy_ref::World::init(512, 512, seed);          // World::map.init, source/cellpool.h:323
//                                                  //   (the reference's terrain for seed)
//   shy_ref::World::map.set_heights(h);            // inject a terrain
//   shy_ref::World::erode(512);                    // World::erode, source/world.h:54-88
//   shy_ref::World::cascade({x, y});               // World::cascade, source/world.h:90-168
//   shy_ref::Drop d({x, y}); while (d.descend());  // source/water.h:58-156
//   float h = shy_ref::World::map.height({x, y});  // quad::map::height, source/cellpool.h:433-437
//   shy_ref::World::srand(s);                      // the reference's own sequence:
//   shy_ref::World::erode_sequential(512);         //   World::erode with rand() spawns
//   shy_ref::Vegetation::grow();                   //   Vegetation::grow, plant agents
//
// World::erode runs the batched GPU mode (all drops of the call at once);
// World::erode_exact runs the reference's sequential semantics on the GPU.
// The map accessors read a host mirror refreshed by World::map.pull() (the
// reference's front end reads cells after each erode call in the same way).
// Errors throw shy_ref::Error (the C ABI itself never throws).
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "shy.h"

namespace shy_ref {

struct vec2 {
  float x, y;
};
struct vec3 {
  float x, y, z;
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
  if (rc != SHY_OK) throw Error(rc, std::string("shy: ") + shy_last_error());
}

// quad::map (source/cellpool.h:319-449) over a host mirror of the device maps.
class Map {
 public:
  shy_world* w = nullptr;
  int nx = 0, ny = 0;
  std::vector<float> height_, discharge_, momx_, momy_, root_;

  void set_heights(const std::vector<float>& h) {
    check(shy_world_set_field(w, SHY_FIELD_HEIGHT, h.data(), h.size()));
    height_ = h;
  }
  // refresh the mirror after erosion (the reference's front end reads cells
  // directly; here one call copies the maps back)
  void pull() {
    const size_t n = (size_t)nx * ny;
    height_.resize(n);
    discharge_.resize(n);
    momx_.resize(n);
    momy_.resize(n);
    root_.resize(n);
    check(shy_terrain_get_state(w, 0, height_.data(), discharge_.data(), momx_.data(), momy_.data(), n));
    check(shy_world_get_field(w, SHY_FIELD_ROOT_DENSITY, root_.data(), n));
  }
  // quad::map::oob, source/cellpool.h:413-419 (positions truncate like glm::ivec2)
  bool oob(vec2 p) const {
    const int x = (int)p.x, y = (int)p.y;
    return x < 0 || y < 0 || x >= nx || y >= ny;
  }
  size_t at(vec2 p) const { return (size_t)(int)p.x * ny + (int)p.y; }
  // quad::map::height, source/cellpool.h:433-437
  float height(vec2 p) const { return oob(p) ? 0.0f : height_[at(p)]; }
  // quad::map::discharge = erf(0.4 d), source/cellpool.h:439-443, 242-244
  float discharge(vec2 p) const { return oob(p) ? 0.0f : std::erf(0.4f * discharge_[at(p)]); }
  float momentumx(vec2 p) const { return oob(p) ? 0.0f : momx_[at(p)]; }
  float momentumy(vec2 p) const { return oob(p) ? 0.0f : momy_[at(p)]; }
  float rootdensity(vec2 p) const { return oob(p) ? 0.0f : root_[at(p)]; }
};

// class World, source/world.h:17-36, with its process-wide state.
class World {
 public:
  static inline Map map;
  static inline uint64_t SEED = 1;

  static void init(int nx, int ny, uint64_t seed, const shy_params* p = nullptr) {
    if (map.w) shy_world_destroy(map.w);
    map = Map();
    SEED = seed;
    check(shy_world_create(nx, ny, p, seed, &map.w));
    map.nx = nx;
    map.ny = ny;
    // the reference's terrain: quad::map::init(..., int SEED), cellpool.h:323-411
    check(shy_terrain_init(map.w, 0, (int32_t)seed));
  }
  static void shutdown() {
    if (map.w) shy_world_destroy(map.w);
    map.w = nullptr;
  }
  // World::erode(int cycles): `cycles` drops (the reference's name), batched.
  static void erode(int cycles) { check(shy_erode(map.w, cycles, 1)); }
  // World::erode with the reference's sequential semantics and given spawns.
  static void erode_exact(const std::vector<int32_t>& spawn_xy) {
    check(shy_erode_exact(map.w, spawn_xy.data(), (int)(spawn_xy.size() / 2)));
  }
  // World::cascade(vec2 pos)
  static void cascade(vec2 pos) { check(shy_cascade(map.w, pos.x, pos.y)); }
  // srand(seed) and World::erode(n) in the reference's own sequence: spawns
  // drawn from the world's C-library rand() stream, drops run one after
  // another (source/world.h:64-78)
  static void srand(unsigned seed) { check(shy_world_srand(map.w, seed)); }
  static void erode_sequential(int drops) { check(shy_erode_rand(map.w, drops)); }
};

// struct Plant (source/vegetation.h:12-36), as the plant list returns it.
struct Plant {
  vec2 pos;
  float size;
};

// struct Vegetation (source/vegetation.h:45-50): grow() runs the reference's
// plant agents on the world's rand() stream; plants() reads the list.
struct Vegetation {
  static void grow() { check(shy_vegetation_grow(World::map.w)); }
  static std::vector<Plant> plants() {
    int n = 0;
    check(shy_plants(World::map.w, nullptr, 0, &n));
    std::vector<float> buf(3 * (size_t)n);
    if (n) check(shy_plants(World::map.w, buf.data(), n, &n));
    std::vector<Plant> out((size_t)n);
    for (int i = 0; i < n; ++i) out[i] = {{buf[3 * i], buf[3 * i + 1]}, buf[3 * i + 2]};
    return out;
  }
};

// struct Drop, source/water.h:12-39.
struct Drop {
  shy_drop s;
  explicit Drop(vec2 pos) {
    s.age = 0;
    s.pos[0] = pos.x;
    s.pos[1] = pos.y;
    s.speed[0] = s.speed[1] = 0.0f;
    s.volume = 1.0f;
    s.sediment = 0.0f;
  }
  bool descend() {
    int more = 0;
    check(shy_drop_descend(World::map.w, &s, &more));
    return more != 0;
  }
  vec2 pos() const { return {s.pos[0], s.pos[1]}; }
  vec2 speed() const { return {s.speed[0], s.speed[1]}; }
  int age() const { return s.age; }
  float volume() const { return s.volume; }
  float sediment() const { return s.sediment; }
};

}  // namespace shy_ref
