// noalloc.cu -- render pass over one image tile that allocates nothing.
//
// Some callers cannot allocate device memory at the time they render: a real-time loop
// where cudaMalloc's implicit device synchronisation would stall the frame, or a host
// whose device memory belongs to its own allocator and forbids driver allocations
// after start-up. yc_render_pass sizes its wavefront state to the image on first use
// (cudaMalloc); this variant keeps that state -- the per-path records, the ray queues and
// the round counters -- in one file-scope __device__ array of NOALLOC_BYTES instead, so
// a tile of at most NOALLOC_MAX_PATHS pixels renders with no allocation at all. The
// array is part of the library image: every GPU that loads the library holds it until
// the process exits.
//
// Every call shares that one array, and it keeps the previous call's contents: the round
// counters are cleared on each pass, everything else is written before it is read. Two
// calls whose work overlaps on the GPU (two contexts on one device, on different
// streams) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include "yc_internal.h"
#include "yc_noalloc.h"
#include "yc_shade.cuh"

namespace yc {

// per-path bytes: the path record (PS_STRIDE float4, 224) + 4 queue slots (16)
constexpr size_t NOALLOC_PATH_BYTES = PS_STRIDE * 16 + 4 * 4;
constexpr size_t NOALLOC_BYTES = (size_t)NOALLOC_MAX_PATHS * NOALLOC_PATH_BYTES + 2 * sizeof(RoundCounters);

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {

// Device address of the scratch array on the current device. In host code the array's
// name is only a host-side stand-in, so the address comes from cudaGetSymbolAddress. It
// is looked up on every call (a call already synchronises its stream, and the lookup is
// a table read): after a cudaDeviceReset or a new primary context the module is loaded
// again and the array may have moved, so no address is kept from an earlier call.
int scratch_address(unsigned char** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return -1;
  *out = static_cast<unsigned char*>(p);
  return 0;
}

}  // namespace

// pathtracer prologue + createRay (kernels/legacy/udpt.cl:158-189, 213-238) for one
// tile; the path slot is the pixel's index inside the tile, so the state fits the
// tile-sized scratch.
__global__ void __launch_bounds__(256) k_raygen_tile(PassParams pp, PathState ps, int* q_closest, RoundCounters* rc,
                                                     DevStats* st) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = pp.tile_w * pp.tile_h;
  int px = 0, py = 0;
  bool active = false;
  if (gid < n) {
    px = gid % pp.tile_w + pp.off_x;
    py = gid / pp.tile_w + pp.off_y;
    active = px < pp.width && py < pp.height;
  }
  const int W = pp.width, H = pp.height;
  const int pix = py * W + px;
  if (active) {
    uint32_t seed = (uint32_t)((py + 1) * W + (px + 1));
    seed = pp.rand_seed * seed;
    seed = ym::wang_hash(seed);
    if (seed == 0) seed = ym::wang_hash(seed);
    const float r1 = draw(seed);
    const float r2 = draw(seed);
    const float fx = ym::add((float)px, r1), fy = ym::add((float)py, r2);
    const float aspect = pp.aspect;
    f4 dir;
    dir.x = (float)((double)aspect * ((2.0 * (double)fx / (double)W) - 1));
    dir.y = (float)((2.0 * (double)fy / (double)H) - 1);
    dir.z = -pp.cam.view_plane_dist;
    dir.w = 0.0f;
    f4 d;
    d.x = ym::dot(ld4(pp.cam.r1), dir);
    d.y = ym::dot(ld4(pp.cam.r2), dir);
    d.z = ym::dot(ld4(pp.cam.r3), dir);
    d.w = ym::dot(ld4(pp.cam.r4), dir);
    d = ym::normalize(d);
    const f4 o = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w);
    float len = __int_as_float(0x7f800000);
    int k = -1;
    light_test(pp.sc, o, d, len, k);
    ps.misc[gid] = make_int4((int)seed, pix, 0 | ((k + 1) << 20), 0);   // state S_PRIMARY, no flags, no light j
    ps.ro[gid] = make_float4(o.x, o.y, o.z, len);
    ps.rd[gid] = make_float4(d.x, d.y, d.z, d.w);
  }
  const unsigned m = __ballot_sync(0xffffffffu, active);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(&rc->n_closest, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (active) q_closest[base + __popc(m & ((1u << lane) - 1))] = gid;
  if (lane == 0 && m) {
    atomicAdd(&st->primary, (unsigned long long)__popc(m));
    atomicAdd(&st->rays, (unsigned long long)__popc(m));
    atomicAdd(&st->traversed, (unsigned long long)__popc(m));
  }
}

int noalloc_render(const NoallocPass& a, std::string& err) {
  const int n_paths = a.pp.tile_w * a.pp.tile_h;
  if (n_paths > NOALLOC_MAX_PATHS) {
    err = "tile of " + std::to_string(n_paths) + " pixels exceeds the " + std::to_string(NOALLOC_MAX_PATHS) +
          "-pixel scratch of yc_render_pass_noalloc; split the frame with block_x/block_y";
    return YC_E_INVALID;
  }
  unsigned char* base = nullptr;
  if (scratch_address(&base)) {
    err = "cudaGetSymbolAddress failed for the render scratch";
    return YC_E_LAUNCH;
  }
  // carve the scratch: the path records, 4 queues, 2 round-counter blocks
  const size_t N = NOALLOC_MAX_PATHS;
  float4* f = reinterpret_cast<float4*>(base);
  const PathState ps = path_state_at(f);
  int* q = reinterpret_cast<int*>(f + PS_STRIDE * N);
  int* qs[4] = {q, q + N, q + 2 * N, q + 3 * N};
  RoundCounters* rc = reinterpret_cast<RoundCounters*>(q + 4 * N);
  cudaStream_t s = a.stream;
  auto launch_failed = [&](const char* what) {
    const cudaError_t e = cudaPeekAtLastError();
    if (e == cudaSuccess) return false;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return true;
  };
  // the counters keep the previous call's values: clear both blocks first
  if (cudaMemsetAsync(rc, 0, 2 * sizeof(RoundCounters), s) != cudaSuccess) {
    err = "clearing the round counters failed";
    return YC_E_LAUNCH;
  }
  k_raygen_tile<<<(n_paths + 255) / 256, 256, 0, s>>>(a.pp, ps, qs[0], rc, a.stats);
  if (launch_failed("ray generation")) return YC_E_LAUNCH;
  const int grid_c = trace_grid_blocks(false, a.pp.sc.depth, a.pp.sc.wide != 0);
  const int grid_a = trace_grid_blocks(true, a.pp.sc.depth, a.pp.sc.wide != 0);
  if (grid_c <= 0 || grid_a <= 0) {
    err = "trace kernel cannot be resident (stack too deep)";
    return YC_E_LAUNCH;
  }
  int cur = 0;
  bool finished = false;
  for (int round = 0; round < a.max_rounds; ++round) {
    RoundCounters* rin = rc + cur;
    RoundCounters* rout = rc + (1 - cur);
    if (launch_trace(a.pp.sc, false, qs[2 * cur], &rin->n_closest, &rin->work_closest, ps.ro, ps.rd, ps.hit, a.stats,
                     grid_c, s) ||
        launch_trace(a.pp.sc, true, qs[2 * cur + 1], &rin->n_any, &rin->work_any, ps.ro, ps.rd, ps.hit, a.stats,
                     grid_a, s)) {
      launch_failed("trace kernel");
      if (err.empty()) err = "trace kernel launch failed";
      return YC_E_LAUNCH;
    }
    if (cudaMemsetAsync(rout, 0, sizeof(RoundCounters), s) != cudaSuccess) {
      err = "clearing the round counters failed";
      return YC_E_LAUNCH;
    }
    launch_logic(a.pp, ps, qs[2 * cur], qs[2 * cur + 1], rin, qs[2 * (1 - cur)], qs[2 * (1 - cur) + 1], rout,
                 a.stats, a.logic_grid, s);
    if (launch_failed("shading kernel")) return YC_E_LAUNCH;
    cur = 1 - cur;
    if ((round + 1) % 6 == 0 || round + 1 == a.max_rounds) {
      if (cudaMemcpyAsync(a.rc_host, rc + cur, sizeof(RoundCounters), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        launch_failed("render pass");
        if (err.empty()) err = "render pass failed";
        return YC_E_LAUNCH;
      }
      if (a.rc_host->n_closest == 0 && a.rc_host->n_any == 0) { finished = true; break; }
    }
  }
  if (!finished) {
    err = "pass not finished after " + std::to_string(a.max_rounds) + " rounds (YC_OPT_MAX_ROUNDS)";
    return YC_E_TIMEOUT;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    err = std::string("render pass failed: ") + cudaGetErrorString(e);
    return YC_E_LAUNCH;
  }
  return YC_OK;
}

}  // namespace yc
