/* yune_cuda.h -- C-ABI of the GB300 path-tracing core (libyune_gb300.so).
 *
 * This replaces Yune's OpenCL dispatch: CLManager (include/CLManager.h:43-170) and the
 * OpenCL calls of RendererCore::setup / enqueueKernels / updateRenderKernelArgs /
 * updatePostProcessingKernelArgs (src/RendererCore.cpp:155-606). The caller keeps its
 * own Scene, BVH and Camera and hands over the same buffers it used to upload with
 * clCreateBuffer(COPY_HOST_PTR): TriangleGPU, Material and BVHNodeGPU arrays, the Cam
 * block, plus the per-pass arguments of the `pathtracer` kernel (GI_CHECK, reset, rand;
 * kernels/legacy/udpt.cl:158-160).
 *
 * Conventions: every function returns 0 (YC_OK) or a negative YC_E* code and never
 * throws; yc_last_error() gives the message of the most recent failure on the calling
 * thread. A context owns one CUDA stream and every device buffer it allocates; it is
 * not thread-safe (one host thread per context, as RendererCore drives CLManager from
 * the GUI thread). Pointers named *_host are host memory; the core copies them.
 */
#ifndef YUNE_CUDA_H
#define YUNE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#include "yune_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes, mirroring the classes CLManager::checkError maps cl_int codes to
 * (src/CLManager.cpp:755-855). */
enum {
  YC_OK = 0,
  YC_E_INVALID = -1,        /* bad argument (CL_INVALID_VALUE and friends) */
  YC_E_NOMEM = -2,          /* device or host allocation failed (CL_OUT_OF_*_MEMORY) */
  YC_E_LAUNCH = -3,         /* kernel launch or CUDA runtime failure */
  YC_E_TIMEOUT = -4,        /* a pass still had live paths after YC_OPT_MAX_ROUNDS rounds */
  YC_E_NODEVICE = -5,       /* no CUDA device */
  YC_E_OVERFLOW = -6,       /* a traversal reached its stack bound (YC_OPT_STACK_LIMIT, the
                               batch's stack_cap): its hit is wrong, so the call fails */
  YC_E_BUDGET = -7,         /* admission refused: the request exceeds the HBM budget */
  YC_E_NOTFOUND = -8        /* unknown scene / accumulator / job id */
};

/* integrators: the unidirectional tracer (udpt.cl), the naive bidirectional tracer
 * (bdpt.cl) and the bidirectional tracer with multiple importance sampling (power
 * heuristic over every strategy with at least two eye vertices; converges to the image of
 * YC_UDPT, which bdpt.cl's heuristic weights do not) */
enum { YC_UDPT = 0, YC_BDPT = 1, YC_BDPT_MIS = 2 };
/* diffuse BRDF: Lambert (udpt.cl:621-622) or the Oren-Nayar rule of
 * kernels/legacy/udpt-primitives.cl:673-686 */
enum { YC_BRDF_LAMBERT = 0, YC_BRDF_OREN_NAYAR = 1 };

/* Per-pass options. The reference fixes these with #defines in the kernel text
 * (udpt.cl:3-9, bdpt.cl:1-8) or with kernel arguments (udpt.cl:158-160). */
typedef struct yc_pass_cfg {
  int32_t integrator;      /* YC_UDPT, YC_BDPT or YC_BDPT_MIS */
  int32_t mis;             /* 1 = the MIS branch of evaluateDirectLighting (udpt.cl:570-608) */
  int32_t rr_threshold;    /* RR_THRESHOLD: roulette when bounce index > this (6 in udpt.cl;
                              YC_BDPT_MIS: subpath vertex index > this) */
  int32_t max_depth;       /* bound of the GI loop (100000 in udpt.cl:463) */
  int32_t brdf_model;      /* YC_BRDF_* */
  int32_t mis_lobe_fix;    /* 0 = reference behaviour; 1 = draw the lobe when the shadow
                              ray is blocked, so a MIS BRDF hit never divides by zero */
  int32_t bdpt_bounces;    /* BDPT_BOUNCES (20 in bdpt.cl:7); YC_BDPT_MIS: the longest path
                              in segments, camera to light (3..32) */
  int32_t block, block_x, block_y;   /* image tile of this launch (udpt.cl:166-167);
                                        block_x = block_y = 1 renders the whole frame */
} yc_pass_cfg;

/* Ray counters since the last yc_reset_stats: every traceRay-equivalent query of the
 * reference algorithm (primary, extension, NEE shadow, MIS BRDF, BDPT connection), and
 * how many of them needed a BVH traversal (a MIS ray whose closest light is not the
 * sampled one is settled analytically, as its outcome does not depend on the BVH). */
typedef struct yc_stats {
  uint64_t rays;            /* all queries */
  uint64_t primary, extension, shadow, mis, connection;
  uint64_t traversed;       /* queries that walked the BVH */
  uint64_t samples;         /* pixel paths completed */
  uint64_t stack_overflow;  /* traversals that hit the stack bound (must be 0) */
  /* work of the traversal kernels: rays walked, child boxes tested (32 B each; two per
   * two-child node, four per four-child node) and triangles tested (48 B each), for the
   * closest-hit (extend) and the any-hit (occlusion) kernel */
  uint64_t ext_rays, ext_boxes, ext_tris;
  uint64_t any_rays, any_boxes, any_tris;
} yc_stats;

/* Device time per kernel kind, summed over launches since the last reset, when
 * profiling is on (CUDA events around each launch on the context stream). */
typedef struct yc_kernel_times {
  double raygen_ms, extend_ms, occlusion_ms, logic_ms;
  uint64_t raygen_launches, extend_launches, occlusion_launches, logic_launches;
  uint64_t rounds;
  double sort_ms;              /* batch engine: shade-queue sort (histogram, scan, scatter) */
  uint64_t sort_launches;
  double tail_ms;              /* tail kernel (YC_OPT_TAIL) */
  uint64_t tail_launches;
  double trace_ms;             /* one launch over a round's closest-hit and any-hit rays
                                  (YC_OPT_MIXED_TRACE); extend_ms and occlusion_ms then stay 0 */
  uint64_t trace_launches;
  double raysort_ms;           /* sort of a round's rays before the trace (YC_OPT_RAY_SORT) */
  uint64_t raysort_launches;
} yc_kernel_times;

typedef struct yc_ctx yc_ctx;

/* ---- context (CLManager::setup, src/CLManager.cpp:118-156) ---- */
int yc_create(int device, yc_ctx** out);
int yc_destroy(yc_ctx* ctx);
const char* yc_last_error(void);
int yc_synchronize(yc_ctx* ctx);

/* ---- scene buffers (CLManager::setupVertexBuffer / setupMatBuffer / setupBVHBuffer,
 *      src/CLManager.cpp:420-484) ---- */
/* Copies and repacks one scene: triangles into a 48-byte (v1, e1, e2) stream in leaf
 * order, the BVH into 64-byte two-child nodes, normals into per-triangle shading
 * records. n_node = 0 means brute force over all triangles (traceRay, udpt.cl:280-284).
 * lights: the quad lights of the scene (1..16). */
int yc_upload_scene(yc_ctx* ctx, const yc_triangle* tris_host, int n_tri, const yc_material* mats_host,
                    int n_mat, const yc_bvh_node* nodes_host, int n_node, const yc_quad_light* lights_host,
                    int n_light, int* scene_id);
int yc_set_lights(yc_ctx* ctx, int scene_id, const yc_quad_light* lights_host, int n_light);

/* ---- BVH build on the device: BVH::createBVH (src/BVH.cpp:56-247) ----
 * Builds, on the context's GPU, the node array the reference builder makes for these
 * triangles (bins: BVH::bins, 20 in the reference; leaf_max: BVH::leaf_primitives, 1..10;
 * the root box is the union of the padded triangle boxes, as Scene::loadModel computes
 * it): breadth-first order, the same splits and the same refit; a bound that is zero is
 * stored as +0. *n_node and *depth receive the node count and the tree depth; the array
 * stays with the context until the next build and is read with yc_bvh_copy_nodes
 * (capacity >= *n_node), ready for yc_upload_scene. Synchronous. YC_E_INVALID when more
 * than leaf_max triangles share one centroid (the reference builder does not terminate). */
int yc_bvh_build(yc_ctx* ctx, const yc_triangle* tris_host, int n_tri, int bins, int leaf_max, int* n_node,
                 int* depth);
int yc_bvh_copy_nodes(yc_ctx* ctx, yc_bvh_node* nodes_host, int capacity);
/* Refit of an uploaded scene for moving geometry (BVH::resizeBvh, src/BVH.cpp:218-247,
 * and the vertex re-upload of CLManager::setupVertexBuffer), on the device: tris_host holds
 * new positions and normals of the same n_tri triangles (same order, materials in range);
 * the stream and shading records are rewritten from them and every box of the hierarchy
 * is recomputed bottom-up from the triangles' padded boxes (TriangleCPU::computeAABB). The
 * hierarchy's topology, leaves and tie-break ranks are kept, so a render equals the
 * reference's with its node array refitted by resizeBvh (yh_bvh_refit) -- as long as the
 * motion leaves the old hierarchy a fair fit; a large motion calls for a new build and
 * upload. The first refit of a scene groups its nodes by depth (one copy of the node
 * links to the host). Synchronous. */
int yc_refit_scene(yc_ctx* ctx, int scene_id, const yc_triangle* tris_host, int n_tri);
int yc_release_scene(yc_ctx* ctx, int scene_id);
/* bytes the scene holds on the device */
int yc_scene_bytes(yc_ctx* ctx, int scene_id, uint64_t* bytes);
/* interior levels of the uploaded hierarchy (a traversal stack needs depth + 2 slots) */
int yc_scene_depth(yc_ctx* ctx, int scene_id, int* depth);
/* FNV-1a digest of the uploaded scene's repacked arrays as they lie on the device (node,
 * triangle-stream and shading records, root box, root link), the digest yc_scene_layout
 * computes on the host for the same inputs. Synchronous. No reference counterpart (an
 * integrity check of the upload). */
int yc_scene_digest(yc_ctx* ctx, int scene_id, uint64_t* digest);

/* The device layout yc_upload_scene would build for these arrays, computed on the host
 * without a device or a context: the bytes the scene would hold (what yc_scene_bytes
 * reports after the upload, so a caller can admit a scene against an HBM budget first),
 * the traversal stack depth, and a digest of the repacked node, triangle-stream and
 * shading arrays (FNV-1a over their 64-bit words), equal for equal inputs whatever the
 * host thread count. tree_mode: the YC_OPT_TREE values. The same checks as the upload:
 * YC_E_INVALID with yc_last_error() naming the first bad triangle or node. No reference
 * counterpart (Yune learns its buffer sizes from clCreateBuffer). */
typedef struct yc_scene_layout_info {
  uint64_t device_bytes;
  uint64_t node_bytes, stream_bytes, shade_bytes;
  uint64_t digest;
  int32_t depth;            /* interior levels, as yc_scene_depth */
  int32_t wide;             /* 1: four-child nodes */
} yc_scene_layout_info;
int yc_scene_layout(const yc_triangle* tris_host, int n_tri, int n_mat, const yc_bvh_node* nodes_host, int n_node,
                    int tree_mode, yc_scene_layout_info* out);

/* The traversal's algorithmic work on explicit rays, counted on the host without a
 * device: the upload's repack of these arrays (tree_mode 0, 1 or 2), then each ray walked
 * alone in the device walk's order (nearer child first, the same distance cull, the
 * reference's slab and Moller-Trumbore arithmetic) but without the speculation of a warp
 * whose lanes walk together. *boxes and *tris_tested receive the child boxes (32 B each)
 * and triangles (48 B each) tested over all rays: the algorithmic bytes of the traversal
 * roofline. rays_host: 9 floats per ray as for yc_trace; any_hit: stop at the first hit
 * closer than the length. tri_out (original index, -1 none) and t_out (final length) may
 * be NULL. No reference counterpart (measurement). */
int yc_walk_counts(const yc_triangle* tris_host, int n_tri, const yc_bvh_node* nodes_host, int n_node, int tree_mode,
                   const float* rays_host, int n, int any_hit, uint64_t* boxes, uint64_t* tris_tested, int* tri_out,
                   float* t_out);

/* ---- camera (CLManager::setupCameraBuffer + the map/unmap of
 *      RendererCore::updateRenderKernelArgs, src/RendererCore.cpp:532-555) ---- */
int yc_set_camera(yc_ctx* ctx, const yc_cam* cam_host);

/* ---- accumulators (the RGBA32F images of CLManager::setupImageBuffers,
 *      src/CLManager.cpp:381-411; one device buffer, updated in place) ---- */
int yc_alloc_accum(yc_ctx* ctx, int width, int height, int* accum_id);
int yc_free_accum(yc_ctx* ctx, int accum_id);
int yc_read_accum(yc_ctx* ctx, int accum_id, float* rgba_host);
int yc_write_accum(yc_ctx* ctx, int accum_id, const float* rgba_host);
/* device address of the accumulator (width*height float4) for zero-copy consumers */
int yc_accum_device_ptr(yc_ctx* ctx, int accum_id, void** dptr);

/* ---- one render pass: the `pathtracer` launch of RendererCore::enqueueKernels
 *      (src/RendererCore.cpp:284-299), one sample per pixel of the tile, running mean
 *      into the accumulator (udpt.cl:196-210). Asynchronous on the context stream. ---- */
int yc_render_pass(yc_ctx* ctx, int scene_id, int accum_id, uint32_t rand_seed, int reset, int gi_check,
                   const yc_pass_cfg* cfg);
/* n_pass passes back to back (pass k uses rand_seeds[k]; reset applies to the first). */
int yc_render_passes(yc_ctx* ctx, int scene_id, int accum_id, const uint32_t* rand_seeds_host, int n_pass,
                     int reset_first, int gi_check, const yc_pass_cfg* cfg);

/* ---- allocation-free render pass over one tile ----
 * No counterpart in the reference. For callers that cannot allocate device memory when
 * they render: a real-time loop where cudaMalloc's implicit device synchronisation would
 * stall the frame, or a host whose device memory belongs to its own allocator and that
 * forbids driver allocations after start-up. yc_render_pass sizes its wavefront state
 * to the image on first use; this call keeps that state in a static device array of the
 * library (about 3.9 MB, held by every GPU that loads the library until exit) and so
 * renders one tile of at most 16384 pixels (cfg->block / block_x / block_y select it,
 * as for yc_render_pass) with no allocation. The scene and accumulator come from
 * yc_upload_scene / yc_alloc_accum, made beforehand. A larger tile is rejected with
 * YC_E_INVALID. Every call looks up the array's device address with
 * cudaGetSymbolAddress on the current device before it launches anything (so a module
 * reloaded after cudaDeviceReset is found again), and synchronises the context stream
 * before it returns. All calls share the array, which keeps the last call's contents
 * (the call clears what must start at zero): calls whose work overlaps on the GPU (two
 * contexts on one device) race and must be serialised. Results equal yc_render_pass with
 * the same arguments, with the same YC_E_TIMEOUT and YC_E_OVERFLOW rules. */
int yc_render_pass_noalloc(yc_ctx* ctx, int scene_id, int accum_id, uint32_t rand_seed, int reset, int gi_check,
                           const yc_pass_cfg* cfg);

/* ---- post pass: the `tonemap` launch (kernels/post-proc/tonemap.cl:14-35,
 *      src/RendererCore.cpp:340-371). out_host receives width*height float4. ---- */
int yc_tonemap(yc_ctx* ctx, int accum_id, float* rgba_out_host);

/* ---- direct ray queries (traceRay of udpt.cl:240-286 on explicit rays) ----
 * rays_host: n records of 9 floats (origin xyzw, dir xyzw, length). Closest query:
 * tri_out = closest triangle (original index, -1 none), light_out = light hit (-1
 * none), t_out = final ray length. Shadow query (any_hit = 1): tri_out = 1 if any
 * triangle or light closes the segment, else 0; light_out and t_out may be NULL. */
int yc_trace(yc_ctx* ctx, int scene_id, const float* rays_host, int n, int any_hit, int* tri_out,
             int* light_out, float* t_out);
/* Same query on device buffers: rays_dev as above, results written to device arrays.
 * Asynchronous on the context stream. */
int yc_trace_device(yc_ctx* ctx, int scene_id, const float* rays_dev, int n, int any_hit, int* tri_dev,
                    float* t_dev);

/* ---- batch and serving engine ----
 * No single counterpart in the reference, which renders one frame per launch. A batch
 * renders many jobs (scene, camera, accumulator, pass seeds) in one persistent
 * wavefront: a fixed pool of path slots takes pixel tasks from all jobs, renders each
 * pixel's passes in order (bit-identical per pixel to yc_render_pass with the same
 * seeds) and takes the next task, so jobs of any size and resolution keep the GPU full.
 * Rounds are captured in a CUDA graph. Jobs may be added while the batch runs
 * (serving). */
typedef struct yc_batch yc_batch;
typedef struct yc_batch_cfg {
  int32_t pool_paths;          /* path slots (wavefront size); 0 = 2,097,152 */
  int32_t rounds_per_launch;   /* rounds per graph launch (even); 0 = 8 */
  int32_t logic_blocks_per_sm; /* logic kernel CTAs per SM; 0 = 4 */
  int32_t use_graph;           /* 1 = capture the rounds in a CUDA graph */
  int32_t max_jobs;            /* capacity of the job table; 0 = 1024 */
  int32_t stack_cap;           /* traversal stack entries; 0 = from the first jobs' scenes */
  int32_t sort_threshold;      /* shade queues of at least this many paths are sorted by path
                                  phase and material class before the logic kernel; 0 = never */
  int32_t groups;              /* slot groups whose rounds run concurrently (1..8); 0 = 2 */
  int32_t ray_sort;            /* sort key of each round's rays: job bits * 100 + origin bits * 10
                                  + direction bits per axis (as YC_OPT_RAY_SORT, plus the low job
                                  bits of each ray's job, so that rays of different scenes do not
                                  share warps; 3 * (origin + direction) + job bits <= 15); 0 = the
                                  context's YC_OPT_RAY_SORT, -1 = rays in queue order */
  int32_t trace_block;         /* threads per block of the traversal kernels (a multiple of 32
                                  up to 256): with the stack columns of its threads it sets the
                                  shared memory per block and so the blocks and the L1 left
                                  per SM; 0 = 128 */
  int32_t stack_smem;          /* entries of each walk's stack kept in shared memory; deeper
                                  entries go to a global spill area of the batch (allocated
                                  when it first runs). Fewer entries leave more of the SM's L1
                                  to the node and triangle fetches; a value at or above the
                                  stack depth keeps the whole stack in shared memory; 0 = 12 */
  int32_t trace_share;         /* percent of the traversal blocks that fit on an SM that the
                                  persistent traversal grid launches (10..100): below 100 each
                                  SM keeps room for the other slot groups' kernels (ray sort,
                                  shading) to run beside a group's traversal; 0 = 100 */
} yc_batch_cfg;
int yc_batch_create(yc_ctx* ctx, const yc_batch_cfg* cfg, yc_batch** out);
/* Adds a job: n_pass passes of scene_id into accum_id seen from *cam, pass k with
 * pass_seeds_host[k]; reset_first = 1 restarts the accumulator (udpt.cl:196-199).
 * cfg: integrator must be YC_UDPT. */
int yc_batch_add_job(yc_batch* b, int scene_id, int accum_id, const yc_cam* cam, const uint32_t* pass_seeds_host,
                     int n_pass, int reset_first, const yc_pass_cfg* cfg, int* job_id);
/* Runs up to max_launches graph launches (0 = until every job is done) and reports how
 * many jobs are still unfinished. */
int yc_batch_run(yc_batch* b, int max_launches, int* unfinished_jobs);
/* pixels whose passes are all done, and the job's pixel count */
int yc_batch_job_progress(yc_batch* b, int job_id, int64_t* pixels_done, int64_t* pixels_total);
/* Cancels a job between runs: each of its pixels in flight stops after its current pass,
 * pixels not yet started are counted done without work (those handed to idle slots at
 * the start of the next launch run one pass), the other jobs are untouched.
 * The job reports done (pixels_done == pixels_total) once its work in flight drains; its
 * accumulator must stay allocated until then. */
int yc_batch_cancel_job(yc_batch* b, int job_id);
/* A batch belongs to its context: yc_destroy releases the context's remaining batches,
 * after which their handles must not be used. */
int yc_batch_destroy(yc_batch* b);

/* ---- launch-shape tuner of the batch engine ----
 * Times candidate shapes on the job mix itself and returns the fastest: every job renders
 * its calibration passes (seeds_host, n_pass; seeds of their own, not the jobs' real ones)
 * into scratch accumulators under each candidate, timed with CUDA events. The search runs
 * one parameter at a time from *start -- pool_paths (512K..4M, at most the mix's pixels
 * rounded up to a power of two), rounds_per_launch (4/8/16/32), logic_blocks_per_sm (2/4/8),
 * sort_threshold (0, 64K, 256K), groups and trace_share together (1/2/4 groups at 100%,
 * 2/4/8 groups at 50%, 4/8 groups at 25%), ray_sort (off, 32, 322), trace_block
 * (64/128/256 threads) and stack_smem (8/12/16 entries, or the whole stack) -- keeping the
 * best value of each, and sweeps again while a sweep
 * moved the shape (at most `sweeps` sweeps). start->stack_cap must hold the deepest
 * scene (depth + 2; the stack depth is not searched: a shorter stack fails the walks).
 * trials (capacity trial_cap) receive every timed shape in order; *n_trials their count.
 * No reference counterpart (the reference has one fixed launch per frame). */
typedef struct yc_tune_job {
  yc_cam cam;
  yc_pass_cfg cfg;             /* integrator YC_UDPT */
  int32_t scene_id, width, height, n_pass;
  const uint32_t* seeds_host;
} yc_tune_job;                 /* 144 bytes, no padding */
typedef struct yc_tune_trial {
  yc_batch_cfg cfg;
  float ms;
} yc_tune_trial;
int yc_batch_tune(yc_ctx* ctx, const yc_tune_job* jobs, int n_jobs, const yc_batch_cfg* start, int sweeps,
                  yc_batch_cfg* best, yc_tune_trial* trials, int trial_cap, int* n_trials);
/* The same search over a clock the caller supplies (host only, no device): clock(cfg,
 * user) returns the time of a candidate shape (any unit, lower is better; negative: an
 * error that ends the search with YC_E_LAUNCH). total_px bounds pool_paths as above.
 * yc_batch_tune is this search with the calibration run of the mix as the clock. */
typedef float (*yc_tune_clock)(const yc_batch_cfg* cfg, void* user);
int yc_tune_search(const yc_batch_cfg* start, int64_t total_px, int sweeps, yc_tune_clock clock, void* user,
                   yc_batch_cfg* best, yc_tune_trial* trials, int trial_cap, int* n_trials);

/* ---- serving: continuous batching of render requests ----
 * No counterpart in the reference, which renders one frame at a time from its GUI loop
 * (src/RendererCore.cpp:248-469); a host that serves many clients submits their frames
 * here. Requests (scene, frame size, passes, seeds, camera, options) are admitted while
 * their accumulators fit a device-memory budget and become jobs of one long-lived batch,
 * so requests that arrive while others run share its wavefront as slots and memory free
 * up. Each request's accumulator is bit-identical to rendering it alone with
 * yc_render_passes and the same seeds.
 *
 * The admission rules are a host-only object (yc_admission), usable without a device by
 * callers with their own scheduler: a request costs its accumulator (width * height * 16
 * bytes) plus its seeds (4 bytes per pass); one larger than the whole budget is rejected
 * at once, and so is one that arrives while max_queue requests already wait; waiting
 * requests are admitted in arrival order (the oldest first; a younger one never overtakes
 * it) whenever the bytes in use plus theirs fit the budget. A waiting request that is
 * cancelled is dropped; a running one is marked cancelling and finishes (cancelled) when
 * its work in flight drains, releasing its bytes. */
enum {
  YC_REQ_WAITING = 0,          /* queued for memory */
  YC_REQ_RUNNING = 1,          /* admitted: its job is in the batch */
  YC_REQ_CANCELLING = 2,       /* cancelled while running; its pixels in flight drain */
  YC_REQ_DONE = 3,             /* every pass of every pixel rendered */
  YC_REQ_CANCELLED = 4,
  YC_REQ_REJECTED_BUDGET = 5,  /* larger than the whole budget */
  YC_REQ_REJECTED_QUEUE = 6    /* max_queue requests were already waiting */
};
typedef struct yc_admission yc_admission;
/* max_queue < 0: no limit on waiting requests */
int yc_admission_create(uint64_t budget_bytes, int32_t max_queue, yc_admission** out);
/* A new request of `bytes`: *ticket identifies it, *state is YC_REQ_RUNNING (admitted at
 * once: nothing waits and it fits), YC_REQ_WAITING or a YC_REQ_REJECTED_* state. */
int yc_admission_submit(yc_admission* a, uint64_t bytes, int64_t* ticket, int32_t* state);
/* Admits the oldest waiting request if it fits now: *ticket = its ticket, or -1. */
int yc_admission_next(yc_admission* a, int64_t* ticket);
/* Cancels: waiting -> YC_REQ_CANCELLED (dropped), running -> YC_REQ_CANCELLING; other
 * states are left as they are. *state receives the new state. */
int yc_admission_cancel(yc_admission* a, int64_t ticket, int32_t* state);
/* The request's work is over (running -> DONE, cancelling -> CANCELLED); its bytes are
 * released. */
int yc_admission_finish(yc_admission* a, int64_t ticket, int32_t* state);
int yc_admission_state(const yc_admission* a, int64_t ticket, int32_t* state);
int yc_admission_usage(const yc_admission* a, uint64_t* bytes_in_use, int32_t* waiting, int32_t* running);
int yc_admission_destroy(yc_admission* a);

typedef struct yc_server yc_server;
typedef struct yc_serve_cfg {
  uint64_t budget_bytes;       /* device bytes of the requests in flight (accumulators, seeds) */
  int32_t max_queue;           /* waiting requests beyond this are rejected; < 0: no limit */
  int32_t keep_results;        /* 1: a finished request keeps its accumulator (and its bytes
                                  in the budget) until yc_serve_release; 0: freed at once */
  yc_batch_cfg batch;          /* the engine's launch shape (stack_cap 0: from the first
                                  requests' scenes; give the deepest resident scene's) */
} yc_serve_cfg;
typedef struct yc_request_desc {
  yc_cam cam;
  yc_pass_cfg cfg;             /* integrator YC_UDPT */
  int32_t scene_id;            /* a scene uploaded to the server's context */
  int32_t width, height;
  int32_t n_pass;
  const uint32_t* seeds_host;  /* n_pass pass seeds (copied by yc_serve_submit) */
} yc_request_desc;             /* 144 bytes, no padding */
typedef struct yc_request_info {
  int32_t state;               /* YC_REQ_* */
  int32_t accum_id;            /* while running and, with keep_results, once done; else -1 */
  int64_t pixels_done, pixels_total;
  double submit_s, admit_s, finish_s;   /* seconds on the server's steady clock (-1: not yet) */
} yc_request_info;
int yc_serve_create(yc_ctx* ctx, const yc_serve_cfg* cfg, yc_server** out);
/* Submits a request (seeds are copied); admitted at once when it fits. */
int yc_serve_submit(yc_server* s, const yc_request_desc* req, int64_t* request_id, int32_t* state);
int yc_serve_cancel(yc_server* s, int64_t request_id);
/* One scheduling step: admits waiting requests that fit, runs up to max_launches launches
 * of the batch (0: none, only admission and completion), then finishes every request whose
 * pixels are all done (freeing its accumulator unless keep_results). *running receives the
 * requests still running or cancelling, *waiting those queued. */
int yc_serve_step(yc_server* s, int max_launches, int32_t* running, int32_t* waiting);
int yc_serve_info(yc_server* s, int64_t request_id, yc_request_info* out);
/* The accumulator of a finished request (keep_results = 1): width * height float4. */
int yc_serve_read(yc_server* s, int64_t request_id, float* rgba_host);
/* Frees a finished request's accumulator (keep_results = 1) and its budget bytes. */
int yc_serve_release(yc_server* s, int64_t request_id);
/* Seconds on the server's clock (the clock of yc_request_info). */
double yc_serve_clock(const yc_server* s);
/* Frees every accumulator still held and the batch. */
int yc_serve_destroy(yc_server* s);

/* ---- options ---- */
enum {
  /* Interior hierarchy of uploaded scenes (applies to later yc_upload_scene calls):
   * 0 = the reference node tree as given; 1 (default) = the reference's leaves, each with
   * its triangles in vert_list order, under interior nodes rebuilt by a binned SAH over
   * the leaf boxes; 2 = the same hierarchy collapsed to four-child nodes (128 B, four
   * boxes tested per node visit). All give the reference's closest hit bit for bit; 1
   * and 2 test fewer boxes (the reference tree keeps the spatial boxes of empty children
   * in its parents' bounds and falls back to spatial-median splits below a node area of
   * about 1). */
  YC_OPT_TREE = 1,
  /* End of a unidirectional pass: once at most this many paths are left, one kernel
   * finishes them a thread per path (trace and shading in turn) instead of round by
   * round; the result is the same bits. -1 (default) = as many paths as one resident
   * launch of that kernel holds; 0 = off. */
  YC_OPT_TAIL = 2,
  /* Traversal launches of a round: 1 (default) = the closest-hit (extension) and the
   * any-hit (shadow, MIS) rays of a round share one launch; 0 = one launch each, the two
   * overlapping on two streams. Same results either way. Applies to later
   * yc_render_pass(es) calls and to batches created afterwards. */
  YC_OPT_MIXED_TRACE = 3,
  /* Order of a round's rays in the mixed traversal launch: a counting sort by the cell of
   * the ray origin in the scene box and the cell of its direction, so that neighbouring
   * lanes walk the same nodes. value = origin bits per axis * 10 + direction bits per axis
   * (each 0..3, sum <= 5); 0 = rays in queue order. Default 32. Same results either way. */
  YC_OPT_RAY_SORT = 4,
  /* Rounds (and batch slot groups) with fewer rays than this are not sorted. Default 65536.
   * yc_render_pass also leaves scenes of fewer than 4096 triangles unsorted (their walks are
   * too short for the sort to pay). */
  YC_OPT_RAY_SORT_MIN = 5,
  /* yc_render_pass (BDPT passes, and unidirectional passes in scenes with a mirror or
   * dielectric material, in frames of at least 524288 pixels): shade queues of at least
   * this many paths are sorted by path phase and material class before the shading
   * kernel, as the batch engine's sort_threshold does; 0 = never. Default 65536. Same
   * results either way. */
  YC_OPT_SHADE_SORT_MIN = 6,
  /* Rounds (trace + shade) one pass may take before yc_render_pass(es) and
   * yc_render_pass_noalloc give up with YC_E_TIMEOUT. Default 1,000,000 (the reference's
   * GI loop bound is 100000 bounces, udpt.cl:463, at most three rays each). */
  YC_OPT_MAX_ROUNDS = 7,
  /* Traversal stack entries a walk may use in yc_render_pass(es) and
   * yc_render_pass_noalloc; 0 (default) = as many as the scene's hierarchy needs (its
   * depth + 2). A smaller bound shrinks the kernels' shared memory; a walk that reaches it
   * fails the call with YC_E_OVERFLOW. Otherwise >= 3. */
  YC_OPT_STACK_LIMIT = 8,
  /* Walk-stack entries kept in shared memory by yc_render_pass(es)'s traversal (one launch
   * per round, YC_OPT_MIXED_TRACE); the deeper entries go to a spill area of the context in
   * global memory (allocated by the first pass that needs it). Fewer entries leave more of
   * each SM's L1 to the node and triangle fetches and more blocks per SM. 0 = 12 (the
   * default); a value at or above the scene's stack depth keeps the whole stack in shared
   * memory. yc_render_pass_noalloc keeps the whole stack there (it allocates nothing). The
   * batch engine has its own setting (yc_batch_cfg.stack_smem). */
  YC_OPT_STACK_SMEM = 9,
  /* Where yc_upload_scene repacks a scene for YC_OPT_TREE 1: 1 (default) on the device
   * (the caller's triangle and node arrays are copied over and the SAH hierarchy above the
   * reference leaves, the leaves' triangle stream and the shading records are built by
   * kernels), 0 on the host. Both give the same bytes (yc_scene_digest equals
   * yc_scene_layout's digest). The node checks and the list of reachable leaves stay on
   * the host; tree modes 0 and 2, and scenes with fewer than two reachable leaves, are
   * repacked on the host either way. */
  YC_OPT_REPACK = 10
};
int yc_set_option(yc_ctx* ctx, int option, int value);

/* ---- statistics and tuning ---- */
int yc_get_stats(yc_ctx* ctx, yc_stats* out);
int yc_reset_stats(yc_ctx* ctx);
/* Span timing on the context stream (the OpenCL event profiling RendererCore reads for
 * its ms/frame and ms/kernel figures, src/RendererCore.cpp:483-505): yc_event_record
 * records event `slot` (0..7) after the work queued so far; yc_event_elapsed_ms waits for
 * event `to` and gives the milliseconds between the two recorded events. */
int yc_event_record(yc_ctx* ctx, int slot);
int yc_event_elapsed_ms(yc_ctx* ctx, int from, int to, float* ms);
/* Device allocations (cudaMalloc) the library's contexts and batches have made in this
 * process so far. A caller that must not allocate while it renders can check that this
 * count does not change across its calls (yc_render_pass_noalloc never allocates). */
int yc_device_allocations(uint64_t* count);
/* Wall time of the device work of the last yc_render_pass(es) call, in ms (CUDA
 * events on the context stream). */
int yc_last_pass_ms(yc_ctx* ctx, float* ms);
/* Per-kernel event timing of yc_render_pass(es) (off by default). */
int yc_set_profiling(yc_ctx* ctx, int on);
int yc_get_kernel_times(yc_ctx* ctx, yc_kernel_times* out);
/* Writes `bytes` of scratch memory on the context stream (evicts L2 between timed
 * passes; benchmark hygiene). */
int yc_flush_l2(yc_ctx* ctx, size_t bytes);
/* Measured L2 read bandwidth in GB/s: `iters` sweeps of a `bytes` buffer (below the L2
 * size) with 128-bit loads; the roofline denominator of the traversal kernels. */
int yc_measure_l2_gbs(yc_ctx* ctx, size_t bytes, int iters, double* gbs);

#ifdef __cplusplus
}
#endif

#endif /* YUNE_CUDA_H */
