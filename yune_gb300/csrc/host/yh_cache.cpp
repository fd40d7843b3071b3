// yh_cache.cpp -- binary scene cache: one file with everything a caller hands to the
// core for one scene (triangles, materials, quad lights, the BVH node array and its
// depth, the camera) plus opaque caller bytes, so that a large procedural scene is read
// back instead of generated and built again. Yune itself re-reads its OBJ file and
// rebuilds the BVH on every start (src/Scene.cpp:133-383, src/BVH.cpp:56-173); the
// cache is new.
//
// File layout (little-endian; sizes in bytes):
//   [0, 256)  header: magic "YUNESCEN", format version, a byte-order word, the record
//             size of each array type, the counts, the caller's 64-bit key, the BVH
//             depth, the offset of each section, the file size, a hash of the payload
//             and a hash of the header itself
//   sections  triangles, materials, lights, nodes, camera, caller bytes: each starts on
//             a 64-byte boundary, the gaps are zero
// The payload hash combines one hash per section (in that order); each section's hash
// is an FNV-1a over its 64-bit words (the last word zero-padded), taken in 4 MiB chunks
// whose hashes are then folded in order by the same FNV-1a step, so that large sections
// are hashed on several threads with a result independent of the thread count.
//
// A file is written under a temporary name in the same directory and renamed into
// place, so a reader sees either the old file or the complete new one.
#include "yune_host.h"
#include "host/yh_threads.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr char MAGIC[8] = {'Y', 'U', 'N', 'E', 'S', 'C', 'E', 'N'};
constexpr uint32_t VERSION = 1;
constexpr uint32_t BYTE_ORDER_WORD = 0x01020304u;
constexpr uint64_t HEADER_BYTES = 256;
constexpr uint64_t ALIGN = 64;
constexpr uint64_t FNV_OFFSET = 0xcbf29ce484222325ull;
constexpr uint64_t FNV_PRIME = 0x100000001b3ull;
constexpr size_t CHUNK = (size_t)4 << 20;   // bytes hashed (and read) per task
constexpr int N_SECT = 6;                     // tris, mats, lights, nodes, cam, meta

struct Header {
  char magic[8];
  uint32_t version, byte_order;
  uint32_t sz_tri, sz_mat, sz_light, sz_node, sz_cam;
  int32_t depth;
  uint64_t key;
  uint64_t count[N_SECT];     // records per section (bytes for the caller's section)
  uint64_t offset[N_SECT];
  uint64_t file_bytes;
  uint64_t payload_hash;
  uint64_t header_hash;       // of the 256 header bytes with this field zero
};
static_assert(sizeof(Header) <= HEADER_BYTES, "header must fit its 256 bytes");

inline uint64_t fnv_step(uint64_t h, uint64_t w) { return (h ^ w) * FNV_PRIME; }

uint64_t hash_words(const unsigned char* p, size_t n) {
  uint64_t h = FNV_OFFSET;
  size_t i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    std::memcpy(&w, p + i, 8);
    h = fnv_step(h, w);
  }
  if (i < n) {
    uint64_t w = 0;
    std::memcpy(&w, p + i, n - i);
    h = fnv_step(h, w);
  }
  return h;
}

int host_threads() { return std::max(1, std::min(16, yh::host_threads())); }

// f(k) for k in [0, n) on up to host_threads() threads, one index at a time
template <class F>
void run_tasks(size_t n, F f) {
  const int t = (int)std::min<size_t>((size_t)host_threads(), n);
  if (t <= 1) {
    for (size_t k = 0; k < n; ++k) f(k);
    return;
  }
  std::vector<std::thread> pool;
  for (int w = 0; w < t; ++w)
    pool.emplace_back([&, w] {
      for (size_t k = (size_t)w; k < n; k += (size_t)t) f(k);
    });
  for (auto& th : pool) th.join();
}

// hash of one section: chunk hashes folded in order
uint64_t hash_section(const void* data, size_t n) {
  const size_t chunks = (n + CHUNK - 1) / CHUNK;
  std::vector<uint64_t> part(chunks);
  run_tasks(chunks, [&](size_t k) {
    const size_t b = k * CHUNK, e = std::min(n, b + CHUNK);
    part[k] = hash_words((const unsigned char*)data + b, e - b);
  });
  uint64_t h = FNV_OFFSET;
  h = fnv_step(h, (uint64_t)n);
  for (uint64_t x : part) h = fnv_step(h, x);
  return h;
}

uint64_t combine(const uint64_t* sect) {
  uint64_t h = FNV_OFFSET;
  for (int k = 0; k < N_SECT; ++k) h = fnv_step(h, sect[k]);
  return h;
}

uint64_t header_hash(Header hd) {
  hd.header_hash = 0;
  unsigned char raw[HEADER_BYTES] = {};
  std::memcpy(raw, &hd, sizeof(hd));
  return hash_words(raw, HEADER_BYTES);
}

inline uint64_t round_up(uint64_t x) { return (x + ALIGN - 1) / ALIGN * ALIGN; }

bool write_all(int fd, const void* p, size_t n, uint64_t off) {
  const unsigned char* c = (const unsigned char*)p;
  while (n > 0) {
    const ssize_t w = pwrite(fd, c, std::min(n, (size_t)1 << 30), (off_t)off);
    if (w <= 0) return false;
    c += w; n -= (size_t)w; off += (uint64_t)w;
  }
  return true;
}

bool read_all(int fd, void* p, size_t n, uint64_t off) {
  unsigned char* c = (unsigned char*)p;
  while (n > 0) {
    const ssize_t r = pread(fd, c, std::min(n, (size_t)1 << 30), (off_t)off);
    if (r <= 0) return false;
    c += r; n -= (size_t)r; off += (uint64_t)r;
  }
  return true;
}

// a section read in CHUNK pieces on several threads
bool read_section(int fd, void* dst, size_t n, uint64_t off) {
  const size_t chunks = (n + CHUNK - 1) / CHUNK;
  std::vector<char> ok(chunks, 1);
  run_tasks(chunks, [&](size_t k) {
    const size_t b = k * CHUNK, e = std::min(n, b + CHUNK);
    ok[k] = read_all(fd, (unsigned char*)dst + b, e - b, off + b) ? 1 : 0;
  });
  return std::all_of(ok.begin(), ok.end(), [](char c) { return c != 0; });
}

struct Fd {
  int fd = -1;
  ~Fd() { if (fd >= 0) close(fd); }
};

// reads and checks the header (magic, version, byte order, record sizes, section bounds)
int read_header(int fd, Header& hd) {
  unsigned char raw[HEADER_BYTES];
  if (!read_all(fd, raw, HEADER_BYTES, 0)) return YH_E_FORMAT;
  std::memcpy(&hd, raw, sizeof(hd));
  if (std::memcmp(hd.magic, MAGIC, 8) != 0 || hd.version != VERSION || hd.byte_order != BYTE_ORDER_WORD)
    return YH_E_FORMAT;
  if (hd.header_hash != header_hash(hd)) return YH_E_FORMAT;
  if (hd.sz_tri != sizeof(yc_triangle) || hd.sz_mat != sizeof(yc_material) || hd.sz_light != sizeof(yc_quad_light) ||
      hd.sz_node != sizeof(yc_bvh_node) || hd.sz_cam != sizeof(yc_cam))
    return YH_E_FORMAT;
  struct stat st;
  if (fstat(fd, &st) != 0 || (uint64_t)st.st_size != hd.file_bytes) return YH_E_FORMAT;
  const uint64_t rec[N_SECT] = {hd.sz_tri, hd.sz_mat, hd.sz_light, hd.sz_node, hd.sz_cam, 1};
  uint64_t end = HEADER_BYTES;
  for (int k = 0; k < N_SECT; ++k) {
    if (hd.count[k] > (uint64_t)INT_MAX || (k == 4 && hd.count[k] > 1)) return YH_E_FORMAT;
    if (hd.offset[k] != round_up(end)) return YH_E_FORMAT;
    end = hd.offset[k] + hd.count[k] * rec[k];
  }
  if (round_up(end) != hd.file_bytes) return YH_E_FORMAT;
  return YH_OK;
}

}  // namespace

extern "C" {

int yh_cache_save(const char* path, uint64_t key, const yc_triangle* tris, int n_tri, const yc_material* mats,
                  int n_mat, const yc_quad_light* lights, int n_light, const yc_bvh_node* nodes, int n_node,
                  int depth, const yc_cam* cam, const void* meta, int meta_bytes) {
  if (!path || n_tri < 0 || n_mat < 0 || n_light < 0 || n_node < 0 || meta_bytes < 0) return YH_E_INVALID;
  if ((n_tri && !tris) || (n_mat && !mats) || (n_light && !lights) || (n_node && !nodes) || (meta_bytes && !meta))
    return YH_E_INVALID;
  Header hd;
  std::memset(&hd, 0, sizeof(hd));
  std::memcpy(hd.magic, MAGIC, 8);
  hd.version = VERSION;
  hd.byte_order = BYTE_ORDER_WORD;
  hd.sz_tri = sizeof(yc_triangle); hd.sz_mat = sizeof(yc_material); hd.sz_light = sizeof(yc_quad_light);
  hd.sz_node = sizeof(yc_bvh_node); hd.sz_cam = sizeof(yc_cam);
  hd.depth = depth;
  hd.key = key;
  const void* src[N_SECT] = {tris, mats, lights, nodes, cam, meta};
  const uint64_t cnt[N_SECT] = {(uint64_t)n_tri, (uint64_t)n_mat, (uint64_t)n_light, (uint64_t)n_node,
                                cam ? 1u : 0u, (uint64_t)meta_bytes};
  const uint64_t rec[N_SECT] = {hd.sz_tri, hd.sz_mat, hd.sz_light, hd.sz_node, hd.sz_cam, 1};
  uint64_t sect_hash[N_SECT];
  uint64_t end = HEADER_BYTES;
  for (int k = 0; k < N_SECT; ++k) {
    hd.count[k] = cnt[k];
    hd.offset[k] = round_up(end);
    end = hd.offset[k] + cnt[k] * rec[k];
    sect_hash[k] = hash_section(src[k], (size_t)(cnt[k] * rec[k]));
  }
  hd.file_bytes = round_up(end);
  hd.payload_hash = combine(sect_hash);
  hd.header_hash = header_hash(hd);

  // unique per process and call, so concurrent writers of one path never share a file
  static std::atomic<unsigned> serial{0};
  const std::string tmp = std::string(path) + ".tmp." + std::to_string((long long)getpid()) + "." +
                          std::to_string(serial.fetch_add(1));
  int rc = YH_OK;
  {
    Fd f;
    f.fd = open(tmp.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (f.fd < 0) return YH_E_IO;
    unsigned char raw[HEADER_BYTES] = {};
    std::memcpy(raw, &hd, sizeof(hd));
    bool ok = write_all(f.fd, raw, HEADER_BYTES, 0);
    // gaps and the tail: ftruncate extends the file with zeros
    ok = ok && ftruncate(f.fd, (off_t)hd.file_bytes) == 0;
    for (int k = 0; ok && k < N_SECT; ++k) {
      const size_t n = (size_t)(cnt[k] * rec[k]);
      const size_t chunks = (n + CHUNK - 1) / CHUNK;
      std::vector<char> good(chunks, 1);
      run_tasks(chunks, [&](size_t c) {
        const size_t b = c * CHUNK, e = std::min(n, b + CHUNK);
        good[c] = write_all(f.fd, (const unsigned char*)src[k] + b, e - b, hd.offset[k] + b) ? 1 : 0;
      });
      ok = std::all_of(good.begin(), good.end(), [](char g) { return g != 0; });
    }
    if (!ok) rc = YH_E_IO;
  }
  if (rc == YH_OK && std::rename(tmp.c_str(), path) != 0) rc = YH_E_IO;
  if (rc != YH_OK) unlink(tmp.c_str());
  return rc;
}

int yh_cache_query(const char* path, yh_cache_info* info) {
  if (!path || !info) return YH_E_INVALID;
  Fd f;
  f.fd = open(path, O_RDONLY);
  if (f.fd < 0) return YH_E_IO;
  Header hd;
  const int rc = read_header(f.fd, hd);
  if (rc != YH_OK) return rc;
  info->key = hd.key;
  info->n_tri = (int)hd.count[0];
  info->n_mat = (int)hd.count[1];
  info->n_light = (int)hd.count[2];
  info->n_node = (int)hd.count[3];
  info->has_cam = (int)hd.count[4];
  info->meta_bytes = (int)hd.count[5];
  info->depth = hd.depth;
  return YH_OK;
}

int yh_cache_load(const char* path, uint64_t key, yc_triangle* tris, int cap_tri, yc_material* mats, int cap_mat,
                  yc_quad_light* lights, int cap_light, yc_bvh_node* nodes, int cap_node, yc_cam* cam, void* meta,
                  int cap_meta) {
  if (!path || cap_tri < 0 || cap_mat < 0 || cap_light < 0 || cap_node < 0 || cap_meta < 0) return YH_E_INVALID;
  Fd f;
  f.fd = open(path, O_RDONLY);
  if (f.fd < 0) return YH_E_IO;
  Header hd;
  int rc = read_header(f.fd, hd);
  if (rc != YH_OK) return rc;
  if (hd.key != key) return YH_E_STALE;
  void* dst[N_SECT] = {tris, mats, lights, nodes, cam, meta};
  const uint64_t cap[N_SECT] = {(uint64_t)cap_tri, (uint64_t)cap_mat, (uint64_t)cap_light, (uint64_t)cap_node,
                                cam ? 1u : 0u, (uint64_t)cap_meta};
  const uint64_t rec[N_SECT] = {hd.sz_tri, hd.sz_mat, hd.sz_light, hd.sz_node, hd.sz_cam, 1};
  for (int k = 0; k < N_SECT; ++k) {
    if (hd.count[k] > cap[k]) return YH_E_RANGE;
    if (hd.count[k] && !dst[k]) return YH_E_INVALID;
  }
  uint64_t sect_hash[N_SECT];
  for (int k = 0; k < N_SECT; ++k) {
    const size_t n = (size_t)(hd.count[k] * rec[k]);
    if (!read_section(f.fd, dst[k], n, hd.offset[k])) return YH_E_FORMAT;
    sect_hash[k] = hash_section(dst[k], n);
  }
  if (combine(sect_hash) != hd.payload_hash) return YH_E_FORMAT;
  return YH_OK;
}

}  // extern "C"
