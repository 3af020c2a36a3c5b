// hydro_oracle.cpp -- TEST INFRASTRUCTURE: the CPU oracle of the erosion path.
//
// Only the test suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// may load this library.  It is a checker, never part of the product: the
// product is the CUDA engine in simplehydrology_gb300/csrc.
//
// Two families of functions:
//
//  1. A restatement of the reference's sequential erosion algorithm
//     (weigert/SimpleHydrology, header-only C++), templated on the scalar type.
//     The float instance is pinned bit for bit against the reference compiled
//     here (oracle/ref_harness.cpp); the double instance is the FP64 error
//     reference.  Each function cites the reference lines it follows.
//     erf_mode selects the erf of erf(0.4 * discharge): ORC_ERF_LIBM is the
//     C library's erff, exactly what the reference calls; ORC_ERF_SHY is the
//     library's own erf (shy_math.h), which the GPU evaluates to the same bits.
//
//  2. A restatement of the batched cycle the GPU engine runs (drops advance
//     in lock step; per-step erosion, cascade and height updates summed in
//     32.32 fixed point).  That schedule has no reference counterpart; its
//     physics is the reference's, cited per line, and its oracle is this code.
//
//  3. The rest of the reference's frame: its plant agents (Vegetation::grow)
//     on the C-library rand() stream that World::erode's spawns share, the
//     front end's per-frame buffers, and the per-cell vegetation of the
//     batched mode.  The first two are pinned against the reference build
//     (tests/golden/ref_frames.json, ref_feed.json).
//
//  4. The reference's terrain: quad::map::init's OpenSimplex2 FBm layers
//     (source/cellpool.h:323-411), through the vendored FastNoiseLite
//     library's noise as that call configures it.  Pinned against the
//     reference build (tests/golden/ref_terrain.json).
//
// Built with -ffp-contract=off so that no multiply-add is fused (the
// reference's x86 build has no FMA either).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/shy.h"
#include "../simplehydrology_gb300/csrc/shy_math.h"

extern "C" {

#define ORC_ERF_LIBM 0
#define ORC_ERF_SHY 1

typedef struct orc_acc {
  uint64_t drops;       // drops that started descending
  uint64_t skipped;     // spawns below height 0.1
  uint64_t oob;         // drops that left the map
  uint64_t steps;       // descend() calls past the termination checks
  double gain;          // sediment created by evaporation
  double loss;          // sediment carried off the map
  int64_t gain_q;       // batched mode: per-drop gains in 32.32 fixed point
  int64_t loss_q;
} orc_acc;

// Field pointers in quad::cell order (source/cellpool.h:207-220), x-major.
typedef struct orc_grid_f32 {
  int nx, ny;
  float* f[8];
} orc_grid_f32;
typedef struct orc_grid_f64 {
  int nx, ny;
  double* f[8];
} orc_grid_f64;

}  // extern "C"

namespace {

template <class T> struct V2 { T x, y; };
template <class T> struct V3 { T x, y, z; };

// glm semantics: component-wise ops; dot sums left to right;
// length = sqrt(dot); normalize = v * (1 / sqrt(dot)).
template <class T> T dot2(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> T dot3(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T len2(V2<T> a) { return std::sqrt(dot2(a, a)); }
template <class T> V2<T> norm2(V2<T> a) {
  const T r = T(1) / std::sqrt(dot2(a, a));
  return {a.x * r, a.y * r};
}
template <class T> V3<T> cross3(V3<T> a, V3<T> b) {
  return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
template <class T> V3<T> mul3(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }

template <class T> struct Grid {
  int nx, ny;
  T *h, *d, *mx, *my, *td, *tmx, *tmy, *root;
  size_t at(int x, int y) const { return (size_t)x * ny + y; }
  // quad::map::oob, source/cellpool.h:413-419
  bool oob(int x, int y) const { return x < 0 || y < 0 || x >= nx || y >= ny; }
  // quad::map::height, source/cellpool.h:433-437 (0 outside the map)
  T height(int x, int y) const { return oob(x, y) ? T(0) : h[at(x, y)]; }
};

template <class T, class G> Grid<T> make_grid(const G* g) {
  Grid<T> r;
  r.nx = g->nx;
  r.ny = g->ny;
  r.h = g->f[0]; r.d = g->f[1]; r.mx = g->f[2]; r.my = g->f[3];
  r.td = g->f[4]; r.tmx = g->f[5]; r.tmy = g->f[6]; r.root = g->f[7];
  return r;
}

inline float erf_of(float x, int mode) { return mode == ORC_ERF_SHY ? shy_erff(x) : std::erf(x); }
inline double erf_of(double x, int mode) { return mode == ORC_ERF_SHY ? shy_erf_d(x) : std::erf(x); }

// glm::ivec2(vec2): truncation toward zero.
template <class T> inline int trunc_i(T v) { return (int)v; }

// quad::_normal, source/cellpool.h:182-204.
template <class T> V3<T> normal(const Grid<T>& g, int px, int py, T mapscale) {
  V3<T> n = {T(0), T(0), T(0)};
  const V3<T> s = {T(1), mapscale, T(1)};
  const T hp = g.height(px, py);
  auto add = [&](V3<T> a, V3<T> b) {
    const V3<T> c = cross3(mul3(s, a), mul3(s, b));
    n = {n.x + c.x, n.y + c.y, n.z + c.z};
  };
  if (!g.oob(px + 1, py + 1))
    add({T(0), g.height(px, py + 1) - hp, T(1)}, {T(1), g.height(px + 1, py) - hp, T(0)});
  if (!g.oob(px - 1, py - 1))
    add({T(0), g.height(px, py - 1) - hp, T(-1)}, {T(-1), g.height(px - 1, py) - hp, T(0)});
  if (!g.oob(px + 1, py - 1))
    add({T(1), g.height(px + 1, py) - hp, T(0)}, {T(0), g.height(px, py - 1) - hp, T(-1)});
  if (!g.oob(px - 1, py + 1))
    add({T(-1), g.height(px - 1, py) - hp, T(0)}, {T(0), g.height(px, py + 1) - hp, T(1)});
  if (std::sqrt(dot3(n, n)) > T(0)) {
    const T r = T(1) / std::sqrt(dot3(n, n));
    n = {n.x * r, n.y * r, n.z * r};
  }
  return n;
}

const int kNb[8][2] = {{-1, -1}, {-1, 0}, {-1, 1}, {0, -1}, {0, 1}, {1, -1}, {1, 0}, {1, 1}};

// World::cascade, source/world.h:90-168.
template <class T> void cascade(Grid<T>& g, const shy_params& P, V2<T> pos) {
  struct Pt { int x, y; T h, d; };
  Pt sn[8];
  int num = 0;
  const int ix = trunc_i(pos.x), iy = trunc_i(pos.y);
  for (int k = 0; k < 8; ++k) {  // :116-125
    const int x = ix + kNb[k][0], y = iy + kNb[k][1];
    if (g.oob(x, y)) continue;
    const V2<T> nn = {(T)kNb[k][0], (T)kNb[k][1]};
    sn[num++] = {x, y, g.h[g.at(x, y)], len2(nn)};
  }
  // :129-131; std::sort of <= 16 elements is libstdc++'s insertion sort,
  // which keeps equal heights in neighbour order (a stable sort).
  for (int i = 1; i < num; ++i) {
    Pt v = sn[i];
    int j = i;
    while (j > 0 && v.h < sn[j - 1].h) {
      sn[j] = sn[j - 1];
      --j;
    }
    sn[j] = v;
  }
  const size_t c = g.at(ix, iy);
  for (int i = 0; i < num; ++i) {  // :133-166
    const size_t n = g.at(sn[i].x, sn[i].y);
    const T diff = g.h[c] - sn[i].h;
    if (diff == T(0)) continue;
    T excess;
    if ((double)sn[i].h > 0.1)
      excess = std::abs(diff) - sn[i].d * (T)P.max_diff;  // * quad::lodsize (1)
    else
      excess = std::abs(diff);
    if (excess <= T(0)) continue;
    const T transfer = (T)P.settling * excess / T(2);
    if (diff > T(0)) {
      g.h[c] -= transfer;
      g.h[n] += transfer;
    } else {
      g.h[c] += transfer;
      g.h[n] -= transfer;
    }
  }
}

template <class T> struct Drop {
  int age = 0;
  V2<T> pos = {T(0), T(0)};
  V2<T> speed = {T(0), T(0)};
  T volume = T(1);
  T sediment = T(0);
};

// (float)((double)x / (1.0 - evap)) and (float)((double)x * (1.0 - evap)),
// source/water.h:135-136: the reference evaluates these in double.
template <class T> T evap_div(T s, float evap) { return (T)((double)s / (1.0 - (double)evap)); }
template <class T> T evap_mul(T v, float evap) { return (T)((double)v * (1.0 - (double)evap)); }

// Drop::descend, source/water.h:58-156.
template <class T>
bool descend(Grid<T>& g, const shy_params& P, Drop<T>& dr, int erf_mode, orc_acc* acc) {
  const int ix = trunc_i(dr.pos.x), iy = trunc_i(dr.pos.y);
  if (g.oob(ix, iy)) return false;  // :62-68
  const size_t c = g.at(ix, iy);
  const V3<T> n = normal(g, ix, iy, (T)P.map_scale);  // :70
  if ((T)dr.age > (T)P.max_age) {  // :74-77
    g.h[c] += dr.sediment;
    return false;
  }
  if (dr.volume < (T)P.min_vol) {  // :79-82
    g.h[c] += dr.sediment;
    return false;
  }
  acc->steps++;
  T effD = (T)P.deposition_rate * (T(1) - g.root[c]);  // :86-87
  if (effD < T(0)) effD = T(0);
  const T gs = (T)P.gravity;  // quad::lodsize * gravity, :95
  dr.speed.x = dr.speed.x + (gs * n.x) / dr.volume;
  dr.speed.y = dr.speed.y + (gs * n.z) / dr.volume;
  const V2<T> f = {g.mx[c], g.my[c]};  // :97-99
  if (len2(f) > T(0) && len2(dr.speed) > T(0)) {
    const T k = ((T)P.momentum_transfer * dot2(norm2(f), norm2(dr.speed))) / (dr.volume + g.d[c]);
    dr.speed.x = dr.speed.x + k * f.x;
    dr.speed.y = dr.speed.y + k * f.y;
  }
  if (len2(dr.speed) > T(0)) {  // :108-109
    const T root2 = std::sqrt(T(2));
    const V2<T> u = norm2(dr.speed);
    dr.speed = {root2 * u.x, root2 * u.y};
  }
  dr.pos = {dr.pos.x + dr.speed.x, dr.pos.y + dr.speed.y};  // :111
  g.td[c] += dr.volume;                                       // :115-117
  g.tmx[c] += dr.volume * dr.speed.x;
  g.tmy[c] += dr.volume * dr.speed.y;
  const int jx = trunc_i(dr.pos.x), jy = trunc_i(dr.pos.y);
  const bool out = g.oob(jx, jy);
  T h2;  // :120-124
  if (out)
    h2 = (T)((double)g.h[c] - 0.002);
  else
    h2 = g.h[g.at(jx, jy)];
  T ceq = (T(1) + (T)P.entrainment * erf_of((T)0.4f * g.d[c], erf_mode)) * (g.h[c] - h2);  // :127
  if (ceq < T(0)) ceq = T(0);
  const T cdiff = ceq - dr.sediment;  // :129-132
  dr.sediment += (effD * cdiff);
  g.h[c] -= (effD * cdiff);
  const T s0 = dr.sediment;  // :135-136
  dr.sediment = evap_div(dr.sediment, P.evap_rate);
  dr.volume = evap_mul(dr.volume, P.evap_rate);
  acc->gain += (double)dr.sediment - (double)s0;
  if (out) {  // :139-142
    dr.volume = T(0);
    acc->oob++;
    acc->loss += (double)dr.sediment;
    return false;
  }
  cascade(g, P, dr.pos);  // :151
  dr.age++;
  return true;
}

// World::erode, source/world.h:54-88, with the spawn positions given.
template <class T>
void erode_seq(Grid<T>& g, const shy_params& P, const int32_t* spawn_xy, int n, int erf_mode,
               orc_acc* acc) {
  const size_t N = (size_t)g.nx * g.ny;
  for (size_t i = 0; i < N; ++i) g.td[i] = g.tmx[i] = g.tmy[i] = T(0);  // :56-61
  for (int i = 0; i < n; ++i) {                                          // :64-78
    const int x = spawn_xy[2 * i], y = spawn_xy[2 * i + 1];
    if ((double)g.height(x, y) < 0.1) {  // :71
      acc->skipped++;
      continue;
    }
    Drop<T> dr;
    dr.pos = {(T)x, (T)y};
    acc->drops++;
    while (descend(g, P, dr, erf_mode, acc)) {
    }
  }
  const T a = T(1) - (T)P.lrate, b = (T)P.lrate;  // :81-86
  for (size_t i = 0; i < N; ++i) {
    g.d[i] = a * g.d[i] + b * g.td[i];
    g.mx[i] = a * g.mx[i] + b * g.tmx[i];
    g.my[i] = a * g.my[i] + b * g.tmy[i];
  }
}

template <class T>
int drop_run(Grid<T>& g, const shy_params& P, T x, T y, float* trace, int max_records,
             int erf_mode, orc_acc* acc) {
  Drop<T> dr;
  dr.pos = {x, y};
  int n = 0;
  for (;;) {
    const bool more = descend(g, P, dr, erf_mode, acc);
    if (n < max_records && trace) {
      float* r = trace + 8 * (size_t)n;
      r[0] = more ? 1.0f : 0.0f;
      r[1] = (float)dr.age;
      r[2] = (float)dr.pos.x;
      r[3] = (float)dr.pos.y;
      r[4] = (float)dr.speed.x;
      r[5] = (float)dr.speed.y;
      r[6] = (float)dr.volume;
      r[7] = (float)dr.sediment;
    }
    ++n;
    if (!more) break;
  }
  return n;
}

// ---------------------------------------------------------------------------
// Batched cycle: restatement of the GPU engine's lock-step design.
//
// All drops of a cycle spawn at once and advance in lock step.  Step t has
// three phases, each reading only state that the previous phase completed:
//  A  every live drop takes one Drop::descend step (source/water.h:58-156)
//     against the heights after step t-1.  A drop that shares its cell with
//     n-1 other live drops exchanges sediment at rate effD / n, so one cell
//     sees one drop's worth of exchange per step (n = 1 is the reference).
//     Height changes and the three tracks are summed in 32.32 fixed point.
//  C  World::cascade (source/world.h:90-168) runs once at every distinct cell
//     a drop moved to, on the heights after phase A's changes; its transfers
//     are summed in fixed point too.  Where the 3 x 3 blocks of k cascades
//     overlap, a pair's transfer is divided by k (the larger count of its two
//     cells), so overlapping cascades together move what one would; k = 1
//     (no overlap) is the reference.
//  D  heights take phase A's and then phase C's sums.
// Heights are held in 32.32 fixed point during batched cycles (hq), with the
// float maps holding their values rounded to float; the drops read the float
// values, and phase D adds the step's integer sums to hq.  Integer sums make
// the result independent of the order drops are visited, which is what lets
// the GPU reproduce it bit for bit.

const double kQ = 4294967296.0;  // 2^32: 32.32 fixed point
inline int64_t q32(float v) { return (int64_t)llrintf(v * 4294967296.0f); }
inline float unq(int64_t q) { return (float)((double)q * (1.0 / kQ)); }

struct LDrop {
  Drop<float> d;
  bool alive;
  int64_t gain_q;  // evaporation gain, 32.32, summed per step
};

struct Lockstep {
  Grid<float> g;
  shy_params P;
  std::vector<float> ceqfac, effd;
  std::vector<int64_t> hq, hqbuf;  // heights, 32.32 fixed point
  std::vector<int64_t> E, Cq, td, tmx, tmy;
  std::vector<int32_t> cnt;
  std::vector<int64_t> stamp;   // per-cell tag: changed this step (phase D list)
  std::vector<int64_t> cstamp;  // per-cell tag: cascade centre claimed this step
  std::vector<int32_t> cover;   // cascade centres whose 3 x 3 block holds the cell
  std::vector<int64_t> touched, centers, occupied;
  std::vector<unsigned char> mask;
  int64_t tag = 0;

  void rebuild_records() {
    const size_t N = (size_t)g.nx * g.ny;
    ceqfac.resize(N);
    effd.resize(N);
    for (size_t i = 0; i < N; ++i) {
      // (1 + entrainment * erf(0.4 d)): source/water.h:127 with
      // node::discharge, source/cellpool.h:242-244
      ceqfac[i] = 1.0f + P.entrainment * shy_erff(0.4f * g.d[i]);
      const float e = P.deposition_rate * (1.0f - g.root[i]);  // source/water.h:86-87
      effd[i] = e < 0.0f ? 0.0f : e;
    }
  }

  void touch(int64_t c) {
    if (stamp[c] != tag) {
      stamp[c] = tag;
      touched.push_back(c);
    }
  }

  // World::cascade at (ix, iy) on the heights h + E, transfers into Cq.
  void cascade_delta(int ix, int iy) {
    struct Pt { int x, y; float h, d; };
    Pt sn[8];
    int num = 0;
    for (int k = 0; k < 8; ++k) {
      const int x = ix + kNb[k][0], y = iy + kNb[k][1];
      if (g.oob(x, y)) continue;
      const V2<float> nn = {(float)kNb[k][0], (float)kNb[k][1]};
      const size_t n = g.at(x, y);
      sn[num++] = {x, y, unq(hq[n] + E[n]), len2(nn)};
    }
    for (int i = 1; i < num; ++i) {
      Pt v = sn[i];
      int j = i;
      while (j > 0 && v.h < sn[j - 1].h) {
        sn[j] = sn[j - 1];
        --j;
      }
      sn[j] = v;
    }
    const size_t c = g.at(ix, iy);
    const float h0 = unq(hq[c] + E[c]);
    float hc = h0;
    for (int i = 0; i < num; ++i) {
      const float diff = hc - sn[i].h;
      if (diff == 0.0f) continue;
      const float excess =
          (double)sn[i].h > 0.1 ? std::fabs(diff) - sn[i].d * P.max_diff : std::fabs(diff);
      if (excess <= 0.0f) continue;
      const size_t n = g.at(sn[i].x, sn[i].y);
      const int32_t k = cover[c] > cover[n] ? cover[c] : cover[n];
      const float transfer = P.settling * excess / 2.0f / (float)k;
      if (diff > 0.0f) {
        hc -= transfer;
        Cq[n] += q32(transfer);
      } else {
        hc += transfer;
        Cq[n] -= q32(transfer);
      }
      touch((int64_t)n);
    }
    Cq[c] += q32(hc - h0);
    touch((int64_t)c);
  }

  // Phase A for one drop; returns false when the drop ends this step.
  bool step(LDrop& ld, orc_acc* acc) {
    Drop<float>& dr = ld.d;
    const int ix = trunc_i(dr.pos.x), iy = trunc_i(dr.pos.y);
    const size_t c = g.at(ix, iy);
    const V3<float> n = normal(g, ix, iy, P.map_scale);
    if ((float)dr.age > P.max_age || dr.volume < P.min_vol) {  // water.h:74-83
      E[c] += q32(dr.sediment);
      touch((int64_t)c);
      return false;
    }
    acc->steps++;
    dr.speed.x = dr.speed.x + (P.gravity * n.x) / dr.volume;  // water.h:95
    dr.speed.y = dr.speed.y + (P.gravity * n.z) / dr.volume;
    const V2<float> f = {g.mx[c], g.my[c]};  // water.h:97-99
    if (len2(f) > 0.0f && len2(dr.speed) > 0.0f) {
      const float k = (P.momentum_transfer * dot2(norm2(f), norm2(dr.speed))) / (dr.volume + g.d[c]);
      dr.speed.x = dr.speed.x + k * f.x;
      dr.speed.y = dr.speed.y + k * f.y;
    }
    if (len2(dr.speed) > 0.0f) {  // water.h:108-109
      const float root2 = std::sqrt(2.0f);
      const V2<float> u = norm2(dr.speed);
      dr.speed = {root2 * u.x, root2 * u.y};
    }
    dr.pos = {dr.pos.x + dr.speed.x, dr.pos.y + dr.speed.y};  // water.h:111
    td[c] += q32(dr.volume);                                   // water.h:115-117
    tmx[c] += q32(dr.volume * dr.speed.x);
    tmy[c] += q32(dr.volume * dr.speed.y);
    const int jx = trunc_i(dr.pos.x), jy = trunc_i(dr.pos.y);
    const bool out = g.oob(jx, jy);
    const float hc = g.h[c];
    const float h2 = out ? (float)((double)hc - 0.002) : g.h[g.at(jx, jy)];  // water.h:120-124
    float ceq = ceqfac[c] * (hc - h2);                                        // water.h:127-128
    if (ceq < 0.0f) ceq = 0.0f;
    const float ed = effd[c] / (float)cnt[c];
    const float ex = ed * (ceq - dr.sediment);  // water.h:129-132
    dr.sediment += ex;
    E[c] -= q32(ex);
    touch((int64_t)c);
    const float s0 = dr.sediment;  // water.h:135-136
    dr.sediment = evap_div(dr.sediment, P.evap_rate);
    dr.volume = evap_mul(dr.volume, P.evap_rate);
    ld.gain_q += q32(dr.sediment - s0);  // exact difference (Sterbenz)
    if (out) {  // water.h:139-142
      acc->oob++;
      acc->loss += (double)dr.sediment;
      acc->loss_q += q32(dr.sediment);
      return false;
    }
    const int64_t cc = (int64_t)g.at(jx, jy);  // water.h:151 -> phase C
    if (cstamp[cc] != tag) {
      cstamp[cc] = tag;
      centers.push_back(cc);
    }
    dr.age++;
    return true;
  }

  void cycle(uint64_t seed, uint64_t cyc, int drops, orc_acc* acc) {
    const size_t N = (size_t)g.nx * g.ny;
    E.assign(N, 0);
    Cq.assign(N, 0);
    td.assign(N, 0);
    tmx.assign(N, 0);
    tmy.assign(N, 0);
    cnt.assign(N, 0);
    stamp.assign(N, -1);
    cstamp.assign(N, -1);
    cover.assign(N, 0);
    tag = 0;
    std::vector<LDrop> L;
    for (int k = 0; k < drops; ++k) {
      int x, y;
      shy_spawn_xy(seed, cyc, (uint32_t)k, g.nx, g.ny, &x, &y);
      if ((double)g.h[g.at(x, y)] < 0.1) {  // world.h:71
        acc->skipped++;
        continue;
      }
      acc->drops++;
      LDrop ld;
      ld.d.pos = {(float)x, (float)y};
      ld.alive = true;
      ld.gain_q = 0;
      L.push_back(ld);
    }
    size_t alive = L.size();
    while (alive > 0) {
      occupied.clear();
      for (auto& ld : L)
        if (ld.alive) {
          const int64_t c = (int64_t)g.at(trunc_i(ld.d.pos.x), trunc_i(ld.d.pos.y));
          if (cnt[c]++ == 0) occupied.push_back(c);
        }
      touched.clear();
      centers.clear();
      for (auto& ld : L) {  // phase A
        if (!ld.alive) continue;
        if (!step(ld, acc)) {
          ld.alive = false;
          --alive;
          acc->gain += (double)ld.gain_q / kQ;
          acc->gain_q += ld.gain_q;
        }
      }
      for (int64_t c : centers) {  // how many cascades reach each cell
        const int x = (int)(c / g.ny), y = (int)(c % g.ny);
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy)
            if (!g.oob(x + dx, y + dy)) cover[g.at(x + dx, y + dy)]++;
      }
      for (int64_t c : centers) cascade_delta((int)(c / g.ny), (int)(c % g.ny));  // phase C
      for (int64_t c : centers) {
        const int x = (int)(c / g.ny), y = (int)(c % g.ny);
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy)
            if (!g.oob(x + dx, y + dy)) cover[g.at(x + dx, y + dy)] = 0;
      }
      for (int64_t c : touched) {  // phase D
        hq[c] += E[c] + Cq[c];
        g.h[c] = unq(hq[c]);
        E[c] = 0;
        Cq[c] = 0;
      }
      for (int64_t c : occupied) cnt[c] = 0;
      tag += 1;
    }
    // world.h:81-86: tracks to float, lrate blend
    mask.assign(N, 0);
    const float a = 1.0f - P.lrate, b = P.lrate;
    for (size_t i = 0; i < N; ++i) {
      const float fd = unq(td[i]), fx = unq(tmx[i]), fy = unq(tmy[i]);
      g.td[i] = fd;
      g.tmx[i] = fx;
      g.tmy[i] = fy;
      g.d[i] = a * g.d[i] + b * fd;
      g.mx[i] = a * g.mx[i] + b * fx;
      g.my[i] = a * g.my[i] + b * fy;
      mask[i] = td[i] != 0;
    }
    for (int p = 0; p < P.cascade_passes; ++p) relax_pass();
    rebuild_records();
  }

  // Optional end-of-cycle slope relaxation: World::cascade's transfer rule
  // (source/world.h:138-164) as a symmetric Jacobi stencil over every pair of
  // neighbours at least one of which a drop visited this cycle, each pair
  // moving cascade_weight * settling * excess / 2.  Off by default.
  void relax_pass() {
    const size_t N = (size_t)g.nx * g.ny;
    hqbuf.resize(N);
    for (int x = 0; x < g.nx; ++x)
      for (int y = 0; y < g.ny; ++y) {
        const size_t c = g.at(x, y);
        const float hc = g.h[c];
        int64_t sum = 0;
        for (int k = 0; k < 8; ++k) {
          const int x2 = x + kNb[k][0], y2 = y + kNb[k][1];
          if (g.oob(x2, y2)) continue;
          const size_t n = g.at(x2, y2);
          if (!(mask[c] | mask[n])) continue;
          const float hn = g.h[n];
          const float diff = hc - hn;
          if (diff == 0.0f) continue;
          const float dist = (kNb[k][0] != 0 && kNb[k][1] != 0) ? std::sqrt(2.0f) : 1.0f;
          const float lo = hc < hn ? hc : hn;
          const float excess =
              (double)lo > 0.1 ? std::fabs(diff) - dist * P.max_diff : std::fabs(diff);
          if (excess <= 0.0f) continue;
          const float transfer = P.cascade_weight * (P.settling * excess / 2.0f);
          sum += diff > 0.0f ? -q32(transfer) : q32(transfer);
        }
        hqbuf[c] = hq[c] + sum;
      }
    hq.swap(hqbuf);
    for (size_t i = 0; i < N; ++i) g.h[i] = unq(hq[i]);
  }
};

// ---------------------------------------------------------------------------
// The reference's plant agents (source/vegetation.h:12-188) and its frame
// loop's random stream.  Vegetation::grow draws from the same C-library
// rand() as World::erode's spawns (source/world.h:69), so a frame
// `World::erode(n); Vegetation::grow();` after srand(seed) is one sequence of
// draws; shy_crand (shy_math.h) restates that generator.  `order` is the
// evaluation order of the two rand() arguments of one vector constructor
// (world.h:69 and vegetation.h:162): 0 left to right, 1 right to left (g++).

struct PlantA {
  float x, y, size;
};

// Plant::root(f), source/vegetation.h:87-118: the 3 x 3 kernel in the
// reference's order, skipping cells outside the map.
template <class T> void plant_root(Grid<T>& g, const PlantA& p, float f) {
  static const int off[9][2] = {{0, 0}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}, {-1, -1}, {1, -1}, {-1, 1}, {1, 1}};
  static const float wgt[9] = {1.0f, 0.6f, 0.6f, 0.6f, 0.6f, 0.4f, 0.4f, 0.4f, 0.4f};
  for (int k = 0; k < 9; ++k) {
    const int x = (int)(p.x + (float)off[k][0]), y = (int)(p.y + (float)off[k][1]);
    if (g.oob(x, y)) continue;
    g.root[g.at(x, y)] += f * wgt[k];
  }
}

// quad::map::discharge (source/cellpool.h:439-443): erf(0.4 d), 0 outside
template <class T> float map_discharge(const Grid<T>& g, int x, int y, int erf_mode) {
  return g.oob(x, y) ? 0.0f : erf_of(0.4f * (float)g.d[g.at(x, y)], erf_mode);
}

// Vegetation::grow, source/vegetation.h:122-188.
template <class T>
void vegetation_grow(Grid<T>& g, const shy_params& P, shy_crand* rnd, std::vector<PlantA>& plants, int order,
                     int erf_mode) {
  {  // :126-139, a random position
    const int x = shy_crand_next(rnd) % g.nx;
    const int y = shy_crand_next(rnd) % g.ny;
    // Plant::spawn, :76-85
    if (!(map_discharge(g, x, y, erf_mode) >= P.plant_max_discharge) &&
        !(normal(g, x, y, P.map_scale).y < P.plant_max_steep) && !(g.height(x, y) >= P.plant_max_height)) {
      plants.push_back({(float)x, (float)y, 0.0f});
      plant_root(g, plants.back(), 1.0f);
    }
  }
  for (size_t i = 0; i < plants.size(); ++i) {  // :143-183
    PlantA& p = plants[i];
    p.size = p.size + P.plant_grow_rate * (P.plant_max_size - p.size);  // Plant::grow, :63-65
    const int cx = (int)p.x, cy = (int)p.y;
    // Plant::die, :67-74 (short-circuit: rand() only when both tests pass)
    const bool die = map_discharge(g, cx, cy, erf_mode) >= P.plant_max_discharge ||
                     g.height(cx, cy) >= P.plant_max_height || shy_crand_next(rnd) % 1000 == 0;
    if (die) {
      plant_root(g, p, -1.0f);
      plants.erase(plants.begin() + (long)i);
      --i;
      continue;
    }
    if (shy_crand_next(rnd) % 20 != 0) continue;  // :160
    const int r1 = shy_crand_next(rnd), r2 = shy_crand_next(rnd);
    const int dx = (order == 0 ? r1 : r2) % 9 - 4, dy = (order == 0 ? r2 : r1) % 9 - 4;  // :162
    const float nx = p.x + (float)dx, ny = p.y + (float)dy;
    const int ix = (int)nx, iy = (int)ny;
    if (g.oob(ix, iy)) continue;                                                    // :165
    if (map_discharge(g, ix, iy, erf_mode) >= P.plant_max_discharge) continue;      // :168
    if ((double)(float)(shy_crand_next(rnd) % 1000) / 1000.0 <= (double)g.root[g.at(ix, iy)]) continue;  // :171
    if (normal(g, ix, iy, P.map_scale).y <= P.plant_max_steep) continue;            // :174-177
    plants.push_back({nx, ny, 0.0f});
    plant_root(g, plants.back(), 1.0f);
  }
}

// ---------------------------------------------------------------------------
// Per-cell vegetation: the GPU engine's restatement of Vegetation::grow
// (source/vegetation.h:122-188).  Every cell holds at most one plant (size
// > 0); one call is one grow() of every plant, in parallel, against the maps
// as they were at the start of the call:
//   grow      size += growRate * (maxSize - size)                  (:63-65)
//   die       erf(0.4 d) >= maxDischarge, height >= maxTreeHeight,
//             or a draw below plant_death_prob (1/1000)            (:67-74)
//             -> root(-1)
//   spread    with plant_spread_prob (1/20): a target cell offset by
//             (u9 - 4, u9 - 4); in the map, erf(0.4 d) < maxDischarge, a draw
//             u1000/1000 above its rootdensity, normal.y > maxSteep, empty
//             -> new plant, root(+1)                               (:160-183)
//   spawn     every empty cell with plant_spawn_prob where erf(0.4 d) <
//             maxDischarge, normal.y >= maxSteep, height < maxTreeHeight
//             -> new plant, root(+1)                               (:76-85)
// A new plant has had its first grow (the reference grows a plant in the
// call that adds it).  A cell that several spawns/spreads reach gets one
// plant.  root(f) adds f * {1, 0.6, 0.4} over the 3 x 3 block (:87-118),
// summed in 32.32 fixed point and added once per cell.
struct VegDraws {
  uint64_t seed, step;
  float u(size_t cell, uint32_t what) const { return shy_uniform24(seed, step, cell, what); }
};

inline float veg_weight(int dx, int dy) {
  const int n = (dx != 0) + (dy != 0);
  return n == 0 ? 1.0f : (n == 1 ? 0.6f : 0.4f);
}

void vegetation_step(Grid<float>& g, float* plant, const shy_params& P, uint64_t seed, uint64_t step) {
  const size_t N = (size_t)g.nx * g.ny;
  const VegDraws R = {seed, step};
  std::vector<float> p0(plant, plant + N);
  std::vector<int64_t> dq(N, 0);
  std::vector<unsigned char> taken(N, 0);
  auto erfd = [&](size_t c) { return shy_erff(0.4f * g.d[c]); };
  auto root = [&](int x, int y, float f) {
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        if (!g.oob(x + dx, y + dy)) dq[g.at(x + dx, y + dy)] += q32(f * veg_weight(dx, dy));
  };
  // a new plant, at most one per cell (the first claim wins; every claim
  // places the same plant)
  auto claim = [&](int x, int y) {
    const size_t t = g.at(x, y);
    if (taken[t]) return false;
    taken[t] = 1;
    plant[t] = P.plant_grow_rate * (P.plant_max_size - 0.0f);
    root(x, y, 1.0f);
    return true;
  };
  // The spread rule of source/vegetation.h:160-183 from cell (x, y) with the
  // draws of `c` (what = w0 .. w0 + 3), on the step's starting maps.
  auto spread_target = [&](int x, int y, size_t c, unsigned w0, int& tx, int& ty) {
    if (!(R.u(c, w0) < P.plant_spread_prob)) return false;
    tx = x + (int)(R.u(c, w0 + 1) * 9.0f) - 4;
    ty = y + (int)(R.u(c, w0 + 2) * 9.0f) - 4;
    if (g.oob(tx, ty)) return false;
    const size_t t = g.at(tx, ty);
    if (erfd(t) >= P.plant_max_discharge) return false;
    if ((float)(int)(R.u(c, w0 + 3) * 1000.0f) / 1000.0f <= g.root[t]) return false;
    if (!(normal(g, tx, ty, P.map_scale).y > P.plant_max_steep)) return false;
    if (p0[t] > 0.0f) return false;
    return true;
  };
  // The reference visits a plant appended during Vegetation::grow in the
  // same call (source/vegetation.h:138, plants.size() is re-read), so a new
  // plant may spread at once: the plant a claim places takes one spread
  // attempt in the same step, with draws keyed by its own cell (chains of
  // three or more new plants in one step are cut at two).
  auto place = [&](int x, int y) {
    if (!claim(x, y)) return;
    int tx, ty;
    if (spread_target(x, y, g.at(x, y), 6, tx, ty)) claim(tx, ty);
  };
  for (int x = 0; x < g.nx; ++x)
    for (int y = 0; y < g.ny; ++y) {
      const size_t c = g.at(x, y);
      if (p0[c] > 0.0f) {
        const float s = p0[c] + P.plant_grow_rate * (P.plant_max_size - p0[c]);
        if (erfd(c) >= P.plant_max_discharge || g.h[c] >= P.plant_max_height ||
            R.u(c, 0) < P.plant_death_prob) {
          plant[c] = 0.0f;
          root(x, y, -1.0f);
          continue;
        }
        plant[c] = s;
        int tx, ty;
        if (spread_target(x, y, c, 1, tx, ty)) place(tx, ty);
      } else {
        if (!(R.u(c, 5) < P.plant_spawn_prob)) continue;
        if (erfd(c) >= P.plant_max_discharge) continue;
        if (normal(g, x, y, P.map_scale).y < P.plant_max_steep) continue;
        if (g.h[c] >= P.plant_max_height) continue;
        place(x, y);
      }
    }
  for (size_t i = 0; i < N; ++i)
    if (dq[i] != 0) g.root[i] = g.root[i] + unq(dq[i]);
}

// ---- 4. the reference's terrain (source/cellpool.h:323-411) ----------------
//
// quad::map::init keeps one static FastNoiseLite object
// (source/include/FastNoiseLite.h) set to OpenSimplex2 noise with FBm
// fractals and otherwise at the library's defaults: noise seed 1337, three
// octaves, lacunarity 2, gain 0.5, weighted strength 0, fractal bounding
// 1 / 1.75, and the OpenSimplex2 3D rotation of the coordinates.  Integer
// arithmetic is done on uint32_t, which wraps as the library's int does.
//
// FnlNoise follows FastNoiseLite's OpenSimplex2 3D evaluation closely, as
// bit parity requires, so it is a derivative of that library and carries its
// licence:
//
//   MIT License
//   Copyright(c) 2020 Jordan Peck (jordan.me2@gmail.com)
//   Copyright(c) 2020 Contributors
//
//   Permission is hereby granted, free of charge, to any person obtaining a
//   copy of this software and associated documentation files(the
//   "Software"), to deal in the Software without restriction, including
//   without limitation the rights to use, copy, modify, merge, publish,
//   distribute, sublicense, and / or sell copies of the Software, and to
//   permit persons to whom the Software is furnished to do so, subject to
//   the following conditions :
//
//   The above copyright notice and this permission notice shall be included
//   in all copies or substantial portions of the Software.
//
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS
//   OR IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF
//   MERCHANTABILITY, FITNESS FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT.
//   IN NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR ANY
//   CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT,
//   TORT OR OTHERWISE, ARISING FROM, OUT OF OR IN CONNECTION WITH THE
//   SOFTWARE OR THE USE OR OTHER DEALINGS IN THE SOFTWARE.
struct FnlNoise {
  float frequency = 0.01f;
  static constexpr uint32_t kPx = 501125321u, kPy = 1136930381u, kPz = 1720413743u;

  // the library's 3D gradient set: its twelve cube-edge vectors five times
  // over, then edges 8, 1, 9 and 3
  static void gradient(int index, float g[3]) {
    static const signed char edge[12][3] = {{0, 1, 1},  {0, -1, 1},  {0, 1, -1},  {0, -1, -1},
                                            {1, 0, 1},  {-1, 0, 1},  {1, 0, -1},  {-1, 0, -1},
                                            {1, 1, 0},  {-1, 1, 0},  {1, -1, 0},  {-1, -1, 0}};
    static const int tail[4] = {8, 1, 9, 3};
    const int e = index < 60 ? index % 12 : tail[index - 60];
    for (int c = 0; c < 3; ++c) g[c] = (float)edge[e][c];
  }
  static float grad_coord(uint32_t seed, uint32_t xp, uint32_t yp, uint32_t zp, float xd, float yd, float zd) {
    uint32_t hash = (seed ^ xp ^ yp ^ zp) * 0x27d4eb2du;
    hash ^= hash >> 15;
    float g[3];
    gradient((int)((hash & (63u << 2)) >> 2), g);
    return xd * g[0] + yd * g[1] + zd * g[2];
  }
  static int round_half_away(float f) { return f >= 0 ? (int)(f + 0.5f) : (int)(f - 0.5f); }

  // one octave of 3D OpenSimplex2 (coordinates already rotated)
  static float opensimplex2(uint32_t seed, float x, float y, float z) {
    const int ri = round_half_away(x), rj = round_half_away(y), rk = round_half_away(z);
    float d[3] = {x - (float)ri, y - (float)rj, z - (float)rk};
    int sign[3];
    float ad[3];
    for (int c = 0; c < 3; ++c) {
      sign[c] = (int)(-1.0f - d[c]) | 1;
      ad[c] = (float)sign[c] * -d[c];
    }
    const uint32_t prime[3] = {kPx, kPy, kPz};
    uint32_t lat[3] = {(uint32_t)ri * kPx, (uint32_t)rj * kPy, (uint32_t)rk * kPz};
    float value = 0.0f;
    float a = (0.6f - d[0] * d[0]) - (d[1] * d[1] + d[2] * d[2]);
    for (int pass = 0;; ++pass) {
      if (a > 0) value += (a * a) * (a * a) * grad_coord(seed, lat[0], lat[1], lat[2], d[0], d[1], d[2]);
      // the next vertex along the coordinate of largest distance (ties: x
      // before y before z)
      const int c = (ad[0] >= ad[1] && ad[0] >= ad[2]) ? 0 : ((ad[1] > ad[0] && ad[1] >= ad[2]) ? 1 : 2);
      float b = a + 1;
      float d1[3] = {d[0], d[1], d[2]};
      uint32_t lat1[3] = {lat[0], lat[1], lat[2]};
      d1[c] += (float)sign[c];
      b -= (float)(sign[c] * 2) * d1[c];
      lat1[c] -= (uint32_t)sign[c] * prime[c];
      if (b > 0) value += (b * b) * (b * b) * grad_coord(seed, lat1[0], lat1[1], lat1[2], d1[0], d1[1], d1[2]);
      if (pass == 1) break;
      for (int k = 0; k < 3; ++k) {
        ad[k] = 0.5f - ad[k];
        d[k] = (float)sign[k] * ad[k];
      }
      a += (0.75f - ad[0]) - (ad[1] + ad[2]);
      for (int k = 0; k < 3; ++k) {
        if (sign[k] < 0) lat[k] += prime[k];
        sign[k] = -sign[k];
      }
      seed = ~seed;
    }
    return value * 32.69428253173828125f;
  }

  // GetNoise(x, y, z): frequency, the OpenSimplex2 rotation, FBm octaves
  float get(float x, float y, float z) const {
    x *= frequency;
    y *= frequency;
    z *= frequency;
    const float r = (x + y + z) * (float)(2.0 / 3.0);
    x = r - x;
    y = r - y;
    z = r - z;
    uint32_t seed = 1337u;
    float sum = 0.0f, amp = 1 / 1.75f;
    for (int o = 0; o < 3; ++o) {
      const float n = opensimplex2(seed++, x, y, z);
      sum += n * amp;
      amp *= 1.0f + 0.0f * ((n + 1) * 0.5f - 1.0f);  // Lerp with weighted strength 0
      x *= 2.0f;
      y *= 2.0f;
      z *= 2.0f;
      amp *= 0.5f;
    }
    return sum;
  }
};

}  // namespace

extern "C" {

int orc_params_default(shy_params* p) {
  std::memset(p, 0, sizeof(*p));
  p->evap_rate = 0.001f;         // source/water.h:43
  p->deposition_rate = 0.1f;     // :44
  p->min_vol = 0.01f;            // :45
  p->max_age = 500.0f;           // :46
  p->entrainment = 10.0f;        // :48
  p->gravity = 1.0f;             // :49
  p->momentum_transfer = 1.0f;   // :50
  p->lrate = 0.1f;               // source/world.h:42
  p->max_diff = 0.01f;           // :43
  p->settling = 0.8f;            // :44
  p->map_scale = 80.0f;          // source/cellpool.h:165
  p->plant_max_size = 1.5f;      // source/vegetation.h:38
  p->plant_grow_rate = 0.05f;    // :39
  p->plant_max_steep = 0.8f;     // :40
  p->plant_max_discharge = 0.3f; // :41
  p->plant_max_height = 0.8f;    // :42
  p->plant_spawn_prob = 1e-4f;
  p->plant_death_prob = 0.001f;  // :71
  p->plant_spread_prob = 0.05f;  // :160
  p->cascade_weight = 0.125f;
  p->cascade_passes = 0;
  return 0;
}

int orc_erode_seq_f32(orc_grid_f32* gr, const shy_params* p, const int32_t* spawn_xy, int n,
                      int erf_mode, orc_acc* acc) {
  Grid<float> g = make_grid<float>(gr);
  erode_seq(g, *p, spawn_xy, n, erf_mode, acc);
  return 0;
}

int orc_erode_seq_f64(orc_grid_f64* gr, const shy_params* p, const int32_t* spawn_xy, int n,
                      int erf_mode, orc_acc* acc) {
  Grid<double> g = make_grid<double>(gr);
  erode_seq(g, *p, spawn_xy, n, erf_mode, acc);
  return 0;
}

int orc_drop_run_f32(orc_grid_f32* gr, const shy_params* p, float x, float y, float* trace,
                     int max_records, int erf_mode, orc_acc* acc) {
  Grid<float> g = make_grid<float>(gr);
  return drop_run(g, *p, x, y, trace, max_records, erf_mode, acc);
}

int orc_drop_run_f64(orc_grid_f64* gr, const shy_params* p, double x, double y, float* trace,
                     int max_records, int erf_mode, orc_acc* acc) {
  Grid<double> g = make_grid<double>(gr);
  return drop_run(g, *p, x, y, trace, max_records, erf_mode, acc);
}

// One Drop::descend() call on a caller-held drop (int age + 6 floats).
int orc_drop_descend_f32(orc_grid_f32* gr, const shy_params* p, shy_drop* d, int erf_mode,
                         orc_acc* acc) {
  Grid<float> g = make_grid<float>(gr);
  Drop<float> dr;
  dr.age = d->age;
  dr.pos = {d->pos[0], d->pos[1]};
  dr.speed = {d->speed[0], d->speed[1]};
  dr.volume = d->volume;
  dr.sediment = d->sediment;
  const bool more = descend(g, *p, dr, erf_mode, acc);
  d->age = dr.age;
  d->pos[0] = dr.pos.x; d->pos[1] = dr.pos.y;
  d->speed[0] = dr.speed.x; d->speed[1] = dr.speed.y;
  d->volume = dr.volume;
  d->sediment = dr.sediment;
  return more ? 1 : 0;
}

void orc_cascade_f32(orc_grid_f32* gr, const shy_params* p, float x, float y) {
  Grid<float> g = make_grid<float>(gr);
  cascade(g, *p, V2<float>{x, y});
}

void orc_normals_f32(orc_grid_f32* gr, const shy_params* p, float* out3) {
  Grid<float> g = make_grid<float>(gr);
  for (int x = 0; x < g.nx; ++x)
    for (int y = 0; y < g.ny; ++y) {
      const V3<float> n = normal(g, x, y, p->map_scale);
      float* o = out3 + 3 * g.at(x, y);
      o[0] = n.x; o[1] = n.y; o[2] = n.z;
    }
}

// The front end's per-frame buffers (SimpleHydrology.cpp:341-354; updatenode,
// source/cellpool.h:286-317): kind 0 the discharge texture
// vec4(waterColor, erf(0.4 d)) with waterColor = vec3(92, 133, 142) / 255
// (source/model.h:22), kind 1 the momentum texture
// vec4(0.5 (1 + erf(mx)), 0.5 (1 + erf(my)), 0.5, 1), kind 2 the mesh
// vertex of each cell: P = (x, mapscale h, y), quad::_normal, T - P, B - P.
void orc_feed_f32(orc_grid_f32* gr, const shy_params* p, int kind, int erf_mode, float* out) {
  Grid<float> g = make_grid<float>(gr);
  const float ms = p->map_scale;
  for (int x = 0; x < g.nx; ++x)
    for (int y = 0; y < g.ny; ++y) {
      const size_t c = g.at(x, y);
      if (kind == 0) {
        float* o = out + 4 * c;
        o[0] = 92.0f / 255.0f;
        o[1] = 133.0f / 255.0f;
        o[2] = 142.0f / 255.0f;
        o[3] = (float)(double)erf_of(0.4f * g.d[c], erf_mode);  // map.discharge, stored via double
      } else if (kind == 1) {
        float* o = out + 4 * c;
        o[0] = 0.5f * (1.0f + erf_of(g.mx[c], erf_mode));
        o[1] = 0.5f * (1.0f + erf_of(g.my[c], erf_mode));
        o[2] = 0.5f;
        o[3] = 1.0f;
      } else {
        float* o = out + 12 * c;
        const float px = (float)x, py = (float)y;
        const float hp = ms * g.height(x, y);
        const V3<float> n = normal(g, x, y, ms);
        const float tx = (float)(x + 1), ty = ms * g.height(x + 1, y);
        const float bx = (float)x, by = ms * g.height(x, y + 1), bz = (float)(y + 1);
        o[0] = px; o[1] = hp; o[2] = py;
        o[3] = n.x; o[4] = n.y; o[5] = n.z;
        o[6] = tx - px; o[7] = ty - hp; o[8] = py - py;
        o[9] = bx - px; o[10] = by - hp; o[11] = bz - py;
      }
    }
}

// The restated C-library generator: n outputs after seeding.
void orc_crand(unsigned seed, int n, int* out) {
  shy_crand g;
  shy_crand_seed(&g, seed);
  for (int i = 0; i < n; ++i) out[i] = shy_crand_next(&g);
}

// The reference's frame loop from srand(seed): `frames` times
// World::erode(drops) with spawns from the stream (source/world.h:64-78),
// then Vegetation::grow().  The plant list starts empty; it comes back as
// (x, y, size) triples in list order (at most max_plants); returns its size.
int orc_frames_f32(orc_grid_f32* gr, const shy_params* p, unsigned seed, int frames, int drops, int order,
                   int erf_mode, float* plants_out, int max_plants, orc_acc* acc) {
  Grid<float> g = make_grid<float>(gr);
  shy_crand rnd;
  shy_crand_seed(&rnd, seed);
  std::vector<PlantA> plants;
  std::vector<int32_t> sp((size_t)2 * (drops > 0 ? drops : 0));
  for (int f = 0; f < frames; ++f) {
    for (int i = 0; i < drops; ++i) {
      const int r1 = shy_crand_next(&rnd), r2 = shy_crand_next(&rnd);
      sp[2 * i] = (order == 0 ? r1 : r2) % g.nx;
      sp[2 * i + 1] = (order == 0 ? r2 : r1) % g.ny;
    }
    erode_seq(g, *p, sp.data(), drops, erf_mode, acc);
    vegetation_grow(g, *p, &rnd, plants, order, erf_mode);
  }
  for (size_t i = 0; i < plants.size() && (int)i < max_plants; ++i) {
    plants_out[3 * i] = plants[i].x;
    plants_out[3 * i + 1] = plants[i].y;
    plants_out[3 * i + 2] = plants[i].size;
  }
  return (int)plants.size();
}

// Spawn positions as World::erode draws them (source/world.h:69):
// srand(seed), then two rand() per drop; `order` 0 gives the first draw to x,
// 1 gives it to y (the compiler picks the argument evaluation order).
void orc_rand_spawns(unsigned seed, int n, int nx, int ny, int order, int32_t* out) {
  srand(seed);
  for (int i = 0; i < n; ++i) {
    const int r1 = rand();
    const int r2 = rand();
    out[2 * i] = order == 0 ? r1 % nx : r2 % nx;
    out[2 * i + 1] = order == 0 ? r2 % ny : r1 % ny;
  }
}

// `cycles` batched cycles of `drops` drops each, starting at cycle index
// `cycle0`.  Tracks come back as the last cycle's sums (as floats).  The
// fixed-point heights can be carried between calls in `hq_io` (nx * ny
// int64): used as the starting state when `hq_in` is nonzero (else derived
// from the float heights), and written back when `hq_io` is not null.
int orc_erode_batched_f32(orc_grid_f32* gr, const shy_params* p, uint64_t seed, uint64_t cycle0,
                          int drops, int cycles, orc_acc* acc, int64_t* hq_io, int hq_in) {
  Lockstep b;
  b.g = make_grid<float>(gr);
  b.P = *p;
  b.rebuild_records();
  const size_t N = (size_t)b.g.nx * b.g.ny;
  b.hq.resize(N);
  for (size_t i = 0; i < N; ++i) {  // heights to 32.32 fixed point
    b.hq[i] = (hq_io && hq_in) ? hq_io[i] : q32(b.g.h[i]);
    b.g.h[i] = unq(b.hq[i]);
  }
  for (int c = 0; c < cycles; ++c) b.cycle(seed, cycle0 + (uint64_t)c, drops, acc);
  if (hq_io) std::memcpy(hq_io, b.hq.data(), N * sizeof(int64_t));
  return 0;
}

// One per-cell vegetation step (see vegetation_step); `plant` is nx * ny
// plant sizes, updated in place with the root-density field.
void orc_vegetation_step_f32(orc_grid_f32* gr, float* plant, const shy_params* p, uint64_t seed, uint64_t step) {
  Grid<float> g = make_grid<float>(gr);
  vegetation_step(g, plant, *p, seed, step);
}

// Seeded fractal value noise normalised to [0, 1]: the terrain recipe.
void orc_value_noise(int nx, int ny, uint64_t seed, int octaves, float* out) {
  const size_t N = (size_t)nx * ny;
  std::vector<double> v(N);
  const int side = nx > ny ? nx : ny;
  double lo = 0.0, hi = 0.0;
  for (int x = 0; x < nx; ++x)
    for (int y = 0; y < ny; ++y) {
      const double t = shy_value_noise(seed, x, y, side, octaves);
      v[(size_t)x * ny + y] = t;
      if (x == 0 && y == 0) lo = hi = t;
      lo = t < lo ? t : lo;
      hi = t > hi ? t : hi;
    }
  const double span = hi - lo;
  for (size_t i = 0; i < N; ++i) out[i] = span > 0.0 ? (float)((v[i] - lo) / span) : 0.0f;
}

// quad::map::init's terrain (source/cellpool.h:349-409) for an nx x ny map:
// eight layers at frequencies 2^o, weights from 0.6 times 0.6 per layer, at
// (x / nx, y / ny, SEED % 10000), then min-max normalised with both bounds
// starting at 0.
void orc_terrain_init(int nx, int ny, int32_t seed, float* out) {
  FnlNoise noise;
  const size_t N = (size_t)nx * ny;
  for (size_t i = 0; i < N; ++i) out[i] = 0.0f;
  float frequency = 1.0f, scale = 0.6f;
  const float zc = (float)(seed % 10000);
  for (int o = 0; o < 8; ++o) {
    noise.frequency = frequency;
    for (int x = 0; x < nx; ++x)
      for (int y = 0; y < ny; ++y) {
        const float px = (float)x / (float)nx, py = (float)y / (float)ny;
        out[(size_t)x * ny + y] += scale * noise.get(px, py, zc);
      }
    frequency *= 2;
    scale *= 0.6;
  }
  float lo = 0.0f, hi = 0.0f;
  for (size_t i = 0; i < N; ++i) {
    lo = (lo < out[i]) ? lo : out[i];
    hi = (hi > out[i]) ? hi : out[i];
  }
  for (size_t i = 0; i < N; ++i) out[i] = (out[i] - lo) / (hi - lo);
}

// The integer routines the GPU's batched kernels use, for the tests.
int64_t orc_q32_int(float v) { return shy_q32(v); }
float orc_unq_int(int64_t q) { return shy_unq(q); }
float orc_evap_div_int(float s, float evap) {
  const shy_evap E = shy_evap_make(evap);
  return shy_evap_div(s, &E);
}

float orc_erff_libm(float x) { return std::erf(x); }
float orc_erff_shy(float x) { return shy_erff(x); }
double orc_erf_shy_d(double x) { return shy_erf_d(x); }

}  // extern "C"
