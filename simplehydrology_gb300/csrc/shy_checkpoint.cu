// shy_checkpoint.cu -- save a world's state to a file and resume from it.
//
// The reference keeps its state in process memory only; a world here can be
// written out between calls and reopened, and the resumed world continues
// bit for bit as the original would have (same maps, same fixed-point
// heights, same spawn-stream position).
//
// Format (version 1, little-endian):
//   header    char magic[8] = "SHYCKPT\0"; u32 version; u32 abi version;
//             u32 n_terrains; u32 flags (bit 0: fixed-point heights valid);
//             u64 cycle; u64 vegetation step; i32 erf source; i32 erf source
//             of the records; i32 track mode; u32 sizeof(shy_params);
//             u32 sizeof(cell record); i32 rand() argument order; u64 cells
//   params    shy_params as in shy.h
//   terrains  per terrain: i32 nx, i32 ny, i32 drops per cycle, u32 0,
//             u64 seed
//   counters  u64 cycles, drops, skipped, oob, steps; i64 gain and loss in
//             32.32 fixed point; f64 exact-mode gain and loss
//   arrays    per array: u32 id, u32 0, u64 bytes, data; all terrains back to
//             back, cells x-major: 1 heights f32, 2 root density f32, 3 plant
//             size f32, 4 tracks 3 x f32, 5 records 4 x f32 (momentum x, y,
//             discharge, 1 + entrainment erf(0.4 d)), 6 deposition rate f32,
//             7 cell records (i64 fixed-point height, i64 0, f32 deposition
//             rate, i32 0, i32 0, i32 0); then 8 the C-library random stream
//             (31 x i32 state, i32 front, i32 back; 0 bytes if never used) and
//             9 the plant agents (x, y, size) x f32 in list order
//   trailer   u64 FNV-1a hash of every byte before it
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "shy_device.cuh"

namespace shy {

namespace {

const char kMagic[8] = {'S', 'H', 'Y', 'C', 'K', 'P', 'T', '\0'};
const uint32_t kVersion = 1;

struct Header {
  char magic[8];
  uint32_t version, abi, n_terrains, flags;
  uint64_t cycle, veg_step;
  int32_t erf_source, ceq_source, track_mode;
  uint32_t params_size, cellq_size;
  int32_t rand_order;
  uint64_t cells;
};
struct TerrainRec {
  int32_t nx, ny, drops;
  uint32_t zero;
  uint64_t seed;
};
struct Counters {
  uint64_t cycles, drops, skipped, oob, steps;
  int64_t gain_q, loss_q;
  double gain_exact, loss_exact;
};

uint64_t fnv1a(uint64_t h, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

struct Writer {
  std::vector<unsigned char> buf;
  void put(const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    buf.insert(buf.end(), b, b + n);
  }
};

struct Reader {
  const unsigned char* p;
  size_t n, off = 0;
  bool get(void* dst, size_t k) {
    if (k > n - off) return false;
    std::memcpy(dst, p + off, k);
    off += k;
    return true;
  }
};

enum ArrayId : uint32_t { A_H = 1, A_ROOT, A_PLANT, A_TRACKS, A_REC, A_EFFD, A_CELLQ, A_CRAND, A_AGENTS };

struct ArrayDesc {
  uint32_t id;
  void* dev;
  size_t bytes;
};

std::vector<ArrayDesc> arrays(shy_world* w) {
  const size_t N = (size_t)w->cells;
  return {{A_H, w->h, 4 * N},          {A_ROOT, w->root, 4 * N},      {A_PLANT, w->plant, 4 * N},
          {A_TRACKS, w->track_f, 12 * N}, {A_REC, w->rec, 16 * N},     {A_EFFD, w->effd, 4 * N},
          {A_CELLQ, w->cq, sizeof(CellQ) * N}};
}

}  // namespace

}  // namespace shy

using namespace shy;

extern "C" int shy_world_save(shy_world* w, const char* path) {
  if (!w || !path) {
    set_error("shy_world_save: null world or path");
    return SHY_ERR_INVALID_ARG;
  }
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "shy_world_save: synchronize");
  Header h;
  std::memset(&h, 0, sizeof(h));
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.abi = SHY_ABI_VERSION;
  h.n_terrains = (uint32_t)w->terrains.size();
  h.flags = w->hq_stale ? 0u : 1u;
  GridBar bar;
  SHY_CHECK_CUDA(cudaMemcpy(&bar, w->bar, sizeof(bar), cudaMemcpyDeviceToHost), "shy_world_save: read state");
  h.cycle = bar.cycle;
  h.veg_step = w->veg_step;
  h.erf_source = w->erf_source;
  h.ceq_source = w->ceq_source;
  h.track_mode = w->track_mode;
  h.params_size = sizeof(shy_params);
  h.cellq_size = sizeof(CellQ);
  h.rand_order = w->rand_order;
  h.cells = (uint64_t)w->cells;
  Writer out;
  out.put(&h, sizeof(h));
  out.put(&w->P, sizeof(shy_params));
  for (const auto& T : w->terrains) {
    TerrainRec r = {T.nx, T.ny, T.drops, 0u, T.seed};
    out.put(&r, sizeof(r));
  }
  DevStats st;
  SHY_CHECK_CUDA(cudaMemcpy(&st, w->stats, sizeof(st), cudaMemcpyDeviceToHost), "shy_world_save: read counters");
  Counters c = {st.cycles, st.drops, st.skipped, st.oob, st.steps, st.gain_q, st.loss_q, st.gain_exact,
                st.loss_exact};
  out.put(&c, sizeof(c));
  std::vector<unsigned char> tmp;
  for (const auto& a : arrays(w)) {
    tmp.resize(a.bytes);
    SHY_CHECK_CUDA(cudaMemcpy(tmp.data(), a.dev, a.bytes, cudaMemcpyDeviceToHost), "shy_world_save: read maps");
    if (a.id == A_CELLQ) {  // between calls only the height and deposition rate are state
      CellQ* q = reinterpret_cast<CellQ*>(tmp.data());
      for (long long i = 0; i < w->cells; ++i) {
        q[i].e = 0;
        q[i].spare = 0;
        q[i].cnt[0] = q[i].cnt[1] = 0;
      }
    }
    const uint32_t id[2] = {a.id, 0u};
    const uint64_t bytes = a.bytes;
    out.put(id, sizeof(id));
    out.put(&bytes, sizeof(bytes));
    out.put(tmp.data(), a.bytes);
  }
  {  // the random stream and the plant agents
    const uint32_t id[2] = {A_CRAND, 0u};
    const uint64_t bytes = w->crand ? sizeof(shy_crand) : 0;
    out.put(id, sizeof(id));
    out.put(&bytes, sizeof(bytes));
    if (bytes) {
      shy_crand g;
      SHY_CHECK_CUDA(cudaMemcpy(&g, w->crand, sizeof(g), cudaMemcpyDeviceToHost), "shy_world_save: read stream");
      out.put(&g, sizeof(g));
    }
    const uint32_t id2[2] = {A_AGENTS, 0u};
    const uint64_t pbytes = sizeof(float3) * (uint64_t)w->plant_count;
    out.put(id2, sizeof(id2));
    out.put(&pbytes, sizeof(pbytes));
    if (pbytes) {
      tmp.resize(pbytes);
      SHY_CHECK_CUDA(cudaMemcpy(tmp.data(), w->plants, pbytes, cudaMemcpyDeviceToHost), "shy_world_save: read plants");
      out.put(tmp.data(), pbytes);
    }
  }
  const uint64_t hash = fnv1a(1469598103934665603ull, out.buf.data(), out.buf.size());
  out.put(&hash, sizeof(hash));

  const std::string tmp_path = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp_path.c_str(), "wb");
  if (!f) {
    set_error("shy_world_save: cannot open %s for writing", tmp_path.c_str());
    return SHY_ERR_IO;
  }
  const bool ok = std::fwrite(out.buf.data(), 1, out.buf.size(), f) == out.buf.size();
  const bool closed = std::fclose(f) == 0;
  if (!ok || !closed || std::rename(tmp_path.c_str(), path) != 0) {
    std::remove(tmp_path.c_str());
    set_error("shy_world_save: writing %s failed", path);
    return SHY_ERR_IO;
  }
  return SHY_OK;
}

extern "C" int shy_world_load(const char* path, shy_world** out) {
  if (!path || !out) {
    set_error("shy_world_load: null path or output");
    return SHY_ERR_INVALID_ARG;
  }
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) {
    set_error("shy_world_load: cannot open %s", path);
    return SHY_ERR_IO;
  }
  std::vector<unsigned char> buf;
  unsigned char chunk[1 << 16];
  size_t k;
  while ((k = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + k);
  const bool rd_err = std::ferror(f) != 0;
  std::fclose(f);
  if (rd_err || buf.size() < sizeof(Header) + 8) {
    set_error("shy_world_load: %s is not a checkpoint (too short)", path);
    return SHY_ERR_IO;
  }
  uint64_t stored;
  std::memcpy(&stored, buf.data() + buf.size() - 8, 8);
  if (fnv1a(1469598103934665603ull, buf.data(), buf.size() - 8) != stored) {
    set_error("shy_world_load: %s is damaged (hash mismatch)", path);
    return SHY_ERR_IO;
  }
  Reader r{buf.data(), buf.size() - 8};
  Header h;
  r.get(&h, sizeof(h));
  if (std::memcmp(h.magic, kMagic, 8) != 0 || h.version != kVersion || h.params_size != sizeof(shy_params) ||
      h.cellq_size != sizeof(CellQ) || h.n_terrains == 0 || h.n_terrains > 65536) {
    set_error("shy_world_load: %s has an unknown format", path);
    return SHY_ERR_IO;
  }
  shy_params P;
  std::vector<int> nx(h.n_terrains), ny(h.n_terrains), drops(h.n_terrains);
  std::vector<uint64_t> seeds(h.n_terrains);
  bool ok = r.get(&P, sizeof(P));
  uint64_t cells = 0;
  for (uint32_t t = 0; ok && t < h.n_terrains; ++t) {
    TerrainRec tr = {};
    if (!(ok = r.get(&tr, sizeof(tr)))) break;
    nx[t] = tr.nx;
    ny[t] = tr.ny;
    drops[t] = tr.drops;
    seeds[t] = tr.seed;
    cells += (uint64_t)tr.nx * (uint64_t)tr.ny;
  }
  Counters c;
  ok = ok && r.get(&c, sizeof(c));
  if (!ok || cells != h.cells) {
    set_error("shy_world_load: %s is truncated or inconsistent", path);
    return SHY_ERR_IO;
  }
  shy_world* w = nullptr;
  int rc = world_create((int)h.n_terrains, nx.data(), ny.data(), drops.data(), seeds.data(), &P, &w);
  if (rc != SHY_OK) return rc;
  auto fail = [&](int code, const char* msg) {
    set_error("shy_world_load: %s", msg);
    world_free(w);
    return code;
  };
  for (const auto& a : arrays(w)) {
    uint32_t id[2];
    uint64_t bytes;
    if (!r.get(id, sizeof(id)) || !r.get(&bytes, sizeof(bytes)) || id[0] != a.id || bytes != a.bytes ||
        bytes > r.n - r.off)
      return fail(SHY_ERR_IO, "map arrays truncated or out of order");
    cudaError_t e = cudaMemcpy(a.dev, buf.data() + r.off, a.bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(cuda_fail(e, "shy_world_load: upload"), cudaGetErrorString(e));
    r.off += a.bytes;
  }
  {  // the random stream and the plant agents
    uint32_t id[2];
    uint64_t bytes;
    if (!r.get(id, sizeof(id)) || !r.get(&bytes, sizeof(bytes)) || id[0] != A_CRAND ||
        (bytes != 0 && bytes != sizeof(shy_crand)) || bytes > r.n - r.off)
      return fail(SHY_ERR_IO, "random stream record damaged");
    if (bytes) {
      cudaError_t e = cudaMalloc((void**)&w->crand, sizeof(shy_crand));
      if (e == cudaSuccess) e = cudaMemcpy(w->crand, buf.data() + r.off, sizeof(shy_crand), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return fail(cuda_fail(e, "shy_world_load: upload"), cudaGetErrorString(e));
      r.off += bytes;
    }
    if (!r.get(id, sizeof(id)) || !r.get(&bytes, sizeof(bytes)) || id[0] != A_AGENTS ||
        bytes % sizeof(float3) != 0 || bytes > r.n - r.off || bytes / sizeof(float3) > (1u << 30))
      return fail(SHY_ERR_IO, "plant list record damaged");
    const long long np = (long long)(bytes / sizeof(float3));
    if (np > 0) {
      const long long cap = 4 * (np + 1) + 4096;
      cudaError_t e = cudaMalloc((void**)&w->plants, sizeof(float3) * (size_t)cap);
      if (e == cudaSuccess) e = cudaMemcpy(w->plants, buf.data() + r.off, bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return fail(cuda_fail(e, "shy_world_load: upload"), cudaGetErrorString(e));
      w->plant_cap = (int)cap;
      w->plant_count = (int)np;
      r.off += bytes;
    }
  }
  if (r.off != r.n) return fail(SHY_ERR_IO, "trailing bytes");
  GridBar bar;
  std::memset(&bar, 0, sizeof(bar));
  bar.cycle = h.cycle;
  DevStats st;
  std::memset(&st, 0, sizeof(st));
  st.cycles = c.cycles;
  st.drops = c.drops;
  st.skipped = c.skipped;
  st.oob = c.oob;
  st.steps = c.steps;
  st.gain_q = c.gain_q;
  st.loss_q = c.loss_q;
  st.gain_exact = c.gain_exact;
  st.loss_exact = c.loss_exact;
  cudaError_t e = cudaMemcpy(w->bar, &bar, sizeof(bar), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(w->stats, &st, sizeof(st), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(cuda_fail(e, "shy_world_load: upload"), cudaGetErrorString(e));
  w->veg_step = h.veg_step;
  w->erf_source = h.erf_source;
  w->ceq_source = h.ceq_source;
  w->track_mode = h.track_mode;
  w->rand_order = h.rand_order == 0 ? 0 : 1;
  w->hq_stale = (h.flags & 1u) == 0;
  *out = w;
  return SHY_OK;
}
