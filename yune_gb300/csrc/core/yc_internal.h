// yc_internal.h -- host-side declarations shared by the core's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "yc_scene.h"
#include "yune_cuda.h"

namespace yc {

// ---- wavefront path state: one record of PS_STRIDE float4 (224 B, seven 32-byte
// sectors) per path slot ----
// The logic kernel reads and writes a path's whole record, and after the shade-queue
// sort neighbouring threads hold unrelated slots; one contiguous record per path keeps
// every sector it fetches fully used (a field per array would use half of each). The
// ray, the batch engine's (job, pass) pair and the hit come first, so the traversal
// kernels touch the first two sectors only.
// misc.x seed, misc.y pixel index, misc.z packed (state | flags << 4 | (j+1) << 12 |
// (k+1) << 20), misc.w bounce index.
constexpr int PS_STRIDE = 14;
enum { PSF_RO = 0, PSF_RD, PSF_JOB, PSF_HIT, PSF_MISC, PSF_THR, PSF_THR_NEXT, PSF_DIRECT, PSF_INDIRECT, PSF_LS,
       PSF_HP, PSF_NRM, PSF_WO, PSF_WI };

// one field of every record: slot i at p[i * PS_STRIDE]
template <class T>
struct SF {
  T* p;
  __host__ __device__ __forceinline__ T& operator[](size_t i) const { return p[i * PS_STRIDE]; }
};

struct PathState {
  SF<int4> misc;
  SF<float4> thr;        // throughput
  SF<float4> thr_next;   // throughput after the pending bounce (udpt.cl:504-507)
  SF<float4> direct;     // direct_color (udpt.cl:455)
  SF<float4> indirect;   // indirect_color
  SF<float4> ls;         // light_sample of the pending NEE (udpt.cl:562-563)
  SF<float4> hp;         // xyz hit point, w light_pdf
  SF<float4> nrm;        // xyz shading normal, w brdf_prob of the NEE lobe
  SF<float4> wo;         // xyz w_o, w brdf_pdf of the MIS sample
  SF<float4> wi;         // xyz NEE direction, w material index (int bits)
  SF<float4> ro;         // emitted ray: origin xyz, length
  SF<float4> rd;         // emitted ray: direction xyz
  SF<float4> hit;        // trace result: (t, u, v, tri) or (occluded, -, -, -)
  SF<int4> job;          // batch engine: (job, pass) of the slot's pixel task
};

// the path state of the records starting at rec (PS_STRIDE float4 per slot)
inline PathState path_state_at(float4* rec) {
  PathState ps;
  ps.misc = SF<int4>{reinterpret_cast<int4*>(rec + PSF_MISC)};
  ps.thr = SF<float4>{rec + PSF_THR};
  ps.thr_next = SF<float4>{rec + PSF_THR_NEXT};
  ps.direct = SF<float4>{rec + PSF_DIRECT};
  ps.indirect = SF<float4>{rec + PSF_INDIRECT};
  ps.ls = SF<float4>{rec + PSF_LS};
  ps.hp = SF<float4>{rec + PSF_HP};
  ps.nrm = SF<float4>{rec + PSF_NRM};
  ps.wo = SF<float4>{rec + PSF_WO};
  ps.wi = SF<float4>{rec + PSF_WI};
  ps.ro = SF<float4>{rec + PSF_RO};
  ps.rd = SF<float4>{rec + PSF_RD};
  ps.hit = SF<float4>{rec + PSF_HIT};
  ps.job = SF<int4>{reinterpret_cast<int4*>(rec + PSF_JOB)};
  return ps;
}

// queues of one round: path indices for the closest-hit and the any-hit kernels
struct Queues {
  int* closest;
  int* any;
};

// per-round device counters (cleared by one memset per round)
struct RoundCounters {
  int n_closest;      // entries appended to the closest queue
  int n_any;          // entries appended to the any-hit queue
  int work_closest;   // persistent-kernel work cursors
  int work_any;
  int work_logic;
  int pad[3];
};

// Sorting of a round's traversal work list by ray origin and direction (raysort.cu):
// `use` tells the trace kernel whether this round's list is the sorted one.
struct RaySortCtl {
  int use;
  int pad[3];
};
#ifdef __CUDACC__
// ---- ray-sort key (raysort.cu, and the batch engine's producers) ----
__device__ __forceinline__ unsigned rs_spread3(unsigned x) {   // bit i of x -> bit 3i (x < 8)
  return (x & 1u) | ((x & 2u) << 2) | ((x & 4u) << 4);
}
__device__ __forceinline__ unsigned rs_cell_of(float v, float scale, int n) {
  const float c = fminf(fmaxf(v * scale, 0.0f), (float)(n - 1));   // NaN -> 0
  return (unsigned)(int)c;
}
// Morton code of the origin's cell in the scene box (ob bits per axis), then of the
// direction's cell in [-1, 1]^3 (db bits per axis)
__device__ __forceinline__ unsigned ray_key(const float4& o, const float4& d, const float4& lo, const float4& hi,
                                            int ob, int db) {
  const int no = 1 << ob, nd = 1 << db;
  const float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = hi.z - lo.z;
  const unsigned ox = rs_cell_of(o.x - lo.x, ex > 0.0f ? (float)no / ex : 0.0f, no);
  const unsigned oy = rs_cell_of(o.y - lo.y, ey > 0.0f ? (float)no / ey : 0.0f, no);
  const unsigned oz = rs_cell_of(o.z - lo.z, ez > 0.0f ? (float)no / ez : 0.0f, no);
  const float hd = 0.5f * (float)nd;
  const unsigned dx = rs_cell_of(d.x + 1.0f, hd, nd), dy = rs_cell_of(d.y + 1.0f, hd, nd),
                 dz = rs_cell_of(d.z + 1.0f, hd, nd);
  const unsigned mo = rs_spread3(ox) | (rs_spread3(oy) << 1) | (rs_spread3(oz) << 2);
  const unsigned md = rs_spread3(dx) | (rs_spread3(dy) << 1) | (rs_spread3(dz) << 2);
  return (mo << (3 * db)) | md;
}
#endif

struct RaySortBufs {
  unsigned* keys;      // one per work-list entry (with keys_any: one per closest-hit queue entry)
  unsigned* keys_any;  // null, or the any-hit queue's keys (the batch engine's logic and fill
                       // kernels write both arrays and the histogram as they queue rays)
  unsigned* hist;      // raysort_bins(ob, db) counters, zero between rounds
  unsigned* cursor;    // scatter cursors (exclusive prefix of hist within its tile of 1024 bins)
  unsigned* blk_sum;   // tile totals (64 at most)
  int* sorted;         // the sorted work list (path indices)
  RaySortCtl* ctl;
  int ob, db;          // origin and direction bits per axis
  int jb;              // job bits of a batch's key (3 * (ob + db) + jb <= 15; 0 for one scene)
  int threshold;       // rounds with fewer rays are traced unsorted
};

// Sorting of the shade queue by the phase a path waits in (S_PRIMARY..S_EXT of the
// unidirectional path, B_LIGHT..B_CONN of BDPT) and material class (diffuse, glossy,
// mirror, dielectric, no surface): key = phase * 5 + class (engine.cu).
constexpr int SORT_KEYS = 25;
struct SortCtl {
  int use;                  // 1: this round's shade queue is the sorted one
  int pad_;
  int count[SORT_KEYS];     // paths per key
  int cursor[SORT_KEYS];    // scatter cursors (exclusive prefix of count)
};

// device-wide statistics (yc_stats layout, 64-bit counters); call_overflow counts the
// stack overflows of the current API call only (cleared when a call starts, read when it
// ends, so the call can return YC_E_OVERFLOW)
struct DevStats {
  unsigned long long rays, primary, extension, shadow, mis, connection, traversed, samples, stack_overflow;
  unsigned long long ext_rays, ext_boxes, ext_tris, any_rays, any_boxes, any_tris;
  unsigned long long call_overflow;
};

// the camera's aspect ratio as createRay computes it (udpt.cl:216-217, in double precision):
// one value per frame, computed on the host when a pass is set up
inline float frame_aspect(int width, int height) { return (float)(((double)width * 1.0) / (double)height); }

struct PassParams {
  DevScene sc;
  yc_cam cam;
  float4* accum;
  int width, height;
  float aspect;            // udpt.cl:216-217 in double precision, set by frame_aspect
  int tile_w, tile_h;      // work-item grid of one block launch
  int off_x, off_y;        // pixel offset of the block (udpt.cl:166-167)
  uint32_t rand_seed;
  int reset;
  int gi_check;
  int mis, rr_threshold, max_depth, brdf_model, mis_lobe_fix;
};

// refit.cu: the nodes of an uploaded scene grouped by depth, deepest level first: order
// (device) lists node indices, level_off (host) the start of each level in it
struct RefitPlan {
  int* order = nullptr;
  std::vector<int> level_off;
};
// rewrites the stream and shading records from new triangles (device) and, with
// refit_nodes, every child box level by level and the scene box (root_out: lo, hi)
int launch_refit(const RefitPlan& plan, const yc_triangle* tris_dev, int n_tri, float4* nodes, float4* stream,
                 int n_slots, float4* shade, bool wide, int root_link, bool refit_nodes, float4* root_out,
                 cudaStream_t s);

// launchers (udpt.cu / trace.cu)
void launch_raygen(const PassParams& pp, const PathState& ps, int* q_closest, RoundCounters* rc, DevStats* st,
                   cudaStream_t s);
// sorted/sctl: the round's shade queue sorted by phase and material class, used when
// sctl->use is set (null: the queues in order)
void launch_logic(const PassParams& pp, const PathState& ps, const int* in_closest, const int* in_any,
                  const RoundCounters* rc_in, int* out_closest, int* out_any, RoundCounters* rc_out,
                  DevStats* st, int grid, cudaStream_t s, const int* sorted = nullptr,
                  const SortCtl* sctl = nullptr);
int launch_trace(const DevScene& sc, bool any_hit, const int* queue, const int* count, int* work,
                 SF<float4> ro, SF<float4> rd, SF<float4> hit, DevStats* st, int grid_blocks,
                 cudaStream_t s);
void launch_tonemap(const float4* in, float4* out, int n, cudaStream_t s);
// tail.cu: finish a pass's paths one thread each once at most `threshold` are left
int tail_capacity(const DevScene& sc, int* grid_out);
int launch_tail(const PassParams& pp, const PathState& ps, const int* in_closest, const int* in_any,
                RoundCounters* rc_in, int threshold, DevStats* st, int grid, cudaStream_t s);
// direct query: rays as 9 floats each
int launch_trace_rays(const DevScene& sc, bool any_hit, const float* rays9, int n, int* tri_out, float* t_out,
                      int* work, DevStats* st, cudaStream_t s);
int trace_grid_blocks(bool any_hit, int depth, bool wide);
// one launch over both queues of a round (closest-hit entries, then any-hit); the work
// cursor is rc->work_closest. n_smem (< the stack depth, with spill): walk-stack entries in
// shared memory, the deeper ones in `spill` (grid_blocks * TRACE_TB columns of
// 2 * (depth - n_smem) ints); otherwise the whole stack is in shared memory.
int launch_trace_mixed(const DevScene& sc, const int* q_closest, const int* q_any, RoundCounters* rc,
                       SF<float4> ro, SF<float4> rd, SF<float4> hit, DevStats* st, int grid_blocks,
                       cudaStream_t s, const int* sorted = nullptr, const RaySortCtl* rs = nullptr, int n_smem = 0,
                       int* spill = nullptr);
// raysort.cu: sorts the round's work list (closest-hit queue, then any-hit queue) into
// b.sorted when the round has at least b.threshold rays, and sets b.ctl->use
int raysort_bins(int ob, int db, int jb = 0);
int launch_raysort(const DevScene& sc, const int* q_closest, const int* q_any, const RoundCounters* rc,
                   SF<float4> ro, SF<float4> rd, const RaySortBufs& b, int grid, cudaStream_t s);
int trace_mixed_grid_blocks(int depth, bool wide, int n_smem = 0);
int trace_stack_cap(int depth);   // walk-stack entries the per-pass kernels give a scene of this depth
constexpr int TRACE_TB_PASS = 128;   // block of the per-pass trace kernels (TRACE_TB of yc_trace_loop.cuh)
int l2_read_gbs(size_t bytes, int iters, cudaStream_t s, double* gbs);
// bvh_build.cu: BVH::createBVH on the device (the node array of the host builder)
// too_deep: the tree would pass 1024 levels (more than leaf_max triangles with one centroid)
cudaError_t bvh_build_device(const yc_triangle* tris_dev, int n, int bins, int leaf_max, cudaStream_t s,
                             std::vector<yc_bvh_node>& out, int& depth, bool& too_deep);

}  // namespace yc
