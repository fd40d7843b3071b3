// tune.cpp -- the batch engine's launch-shape tuner (yc_batch_tune), host code over the
// C-ABI of the engine.
//
// The engine's shape parameters change its speed but never its results: path slots in
// flight (the wavefront), rounds per graph launch, shading blocks per SM, the shade-queue
// size from which the queue is sorted by phase and material, slot groups whose rounds
// run concurrently, the ray sort before the traversal, and the traversal kernels' block
// (threads per block, which with the per-thread stack columns sets the shared memory per
// block, hence the blocks and the L1 left per SM). The best values depend on the job mix,
// so the tuner times candidate shapes on the mix itself (the ray sort: off, by origin and
// direction cell, or by job and cell): each candidate renders the
// jobs' calibration passes into scratch accumulators, timed with CUDA events on the
// context stream. It searches one parameter at a time from a starting shape, keeps the
// best value of each, and repeats the sweep while a sweep changed the shape (up to
// `sweeps` sweeps). The stack depth is not searched: every walk needs the deepest
// scene's levels + 2 entries (a shorter stack would fail the walks with YC_E_OVERFLOW).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "yune_cuda.h"

namespace yc {
int set_error(int code, const char* msg);   // api.cu: sets yc_last_error()
}

static_assert(sizeof(yc_tune_job) == 144, "yc_tune_job: cam, cfg, four ints, a pointer");
static_assert(sizeof(yc_tune_trial) == 52, "yc_tune_trial: yc_batch_cfg (12 ints) and a float");

namespace {

// one search dimension: one field, or fields searched together (each value a tuple)
struct Param {
  std::vector<int32_t yc_batch_cfg::*> fields;
  std::vector<std::vector<int32_t>> values;
};

bool same(const yc_batch_cfg& a, const yc_batch_cfg& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

// stack_smem of a whole stack in shared memory (above any scene's depth + 2)
constexpr int32_t kWholeStack = 64;

// device milliseconds of the calibration passes of every job under `cfg`
int calibrate(yc_ctx* ctx, const yc_tune_job* jobs, int n_jobs, const std::vector<int>& accs,
              const yc_batch_cfg& cfg, float* ms) {
  yc_batch* b = nullptr;
  yc_batch_cfg c = cfg;
  c.max_jobs = std::max(c.max_jobs, n_jobs);
  if (int r = yc_batch_create(ctx, &c, &b)) return r;
  int r = YC_OK;
  for (int i = 0; i < n_jobs && !r; ++i) {
    int job = -1;
    r = yc_batch_add_job(b, jobs[i].scene_id, accs[i], &jobs[i].cam, jobs[i].seeds_host, jobs[i].n_pass, 1,
                         &jobs[i].cfg, &job);
  }
  int left = 0;
  if (!r) r = yc_batch_run(b, 0, &left);
  if (!r) r = yc_last_pass_ms(ctx, ms);
  yc_batch_destroy(b);
  return r;
}

}  // namespace

namespace {

// the clock of yc_batch_tune: the calibration run of the mix
struct MixClock {
  yc_ctx* ctx;
  const yc_tune_job* jobs;
  int n_jobs;
  std::vector<int> accs;
  int err = YC_OK;
};

float mix_clock(const yc_batch_cfg* cfg, void* user) {
  MixClock* m = static_cast<MixClock*>(user);
  float ms = -1.0f;
  if (m->err) return -1.0f;
  m->err = calibrate(m->ctx, m->jobs, m->n_jobs, m->accs, *cfg, &ms);
  return m->err ? -1.0f : ms;
}

}  // namespace

extern "C" int yc_tune_search(const yc_batch_cfg* start, int64_t total_px, int sweeps, yc_tune_clock clock, void* user,
                              yc_batch_cfg* best_out, yc_tune_trial* trials, int trial_cap, int* n_trials) {
  if (!start || !clock || !best_out || sweeps < 1 || total_px <= 0 || (trial_cap > 0 && !trials))
    return yc::set_error(YC_E_INVALID, "yc_tune_search: bad argument");
  // more slots than the mix has pixels would stay idle
  int32_t pool_cap = 1 << 16;
  while (pool_cap < total_px && pool_cap < (1 << 22)) pool_cap <<= 1;
  // slot groups and the traversal's share of each SM are searched together: more groups
  // pay only when a group's traversal leaves room on the SMs for the others' kernels
  const std::vector<Param> params = {
      {{&yc_batch_cfg::pool_paths}, {{1 << 19}, {1 << 20}, {1 << 21}, {1 << 22}}},
      {{&yc_batch_cfg::rounds_per_launch}, {{4}, {8}, {16}, {32}}},
      {{&yc_batch_cfg::logic_blocks_per_sm}, {{2}, {4}, {8}}},
      {{&yc_batch_cfg::sort_threshold}, {{0}, {1 << 16}, {1 << 18}}},
      {{&yc_batch_cfg::groups, &yc_batch_cfg::trace_share},
       {{1, 100}, {2, 100}, {4, 100}, {2, 50}, {4, 50}, {8, 50}, {4, 25}, {8, 25}}},
      {{&yc_batch_cfg::ray_sort}, {{-1}, {32}, {322}}},
      {{&yc_batch_cfg::trace_block}, {{64}, {128}, {256}}},
      {{&yc_batch_cfg::stack_smem}, {{8}, {12}, {16}, {kWholeStack}}},
  };
  std::vector<std::pair<yc_batch_cfg, float>> timed;
  auto record = [&](const yc_batch_cfg& c, float ms) {
    timed.emplace_back(c, ms);
    if ((int)timed.size() <= trial_cap) trials[timed.size() - 1] = yc_tune_trial{c, ms};
  };
  yc_batch_cfg best = *start;
  if (best.pool_paths <= 0 || best.pool_paths > pool_cap) best.pool_paths = std::min(1 << 21, pool_cap);
  if (best.trace_block <= 0) best.trace_block = 128;
  if (best.stack_smem <= 0) best.stack_smem = 12;
  if (best.trace_share <= 0) best.trace_share = 100;
  if (best.groups <= 0) best.groups = 2;
  float best_ms = clock(&best, user);
  if (best_ms < 0.0f) return yc::set_error(YC_E_LAUNCH, "yc_tune_search: the clock failed");
  record(best, best_ms);
  for (int sw = 0; sw < sweeps; ++sw) {
    const yc_batch_cfg at_start = best;
    for (const Param& p : params) {
      for (const std::vector<int32_t>& v : p.values) {
        yc_batch_cfg cand = best;
        for (size_t f = 0; f < p.fields.size(); ++f) cand.*p.fields[f] = v[f];
        if (same(cand, best)) continue;
        if (p.fields[0] == &yc_batch_cfg::pool_paths && v[0] > pool_cap) continue;
        bool seen = false;
        for (const auto& t : timed) seen = seen || same(t.first, cand);
        if (seen) continue;
        const float ms = clock(&cand, user);
        if (ms < 0.0f) return yc::set_error(YC_E_LAUNCH, "yc_tune_search: the clock failed");
        record(cand, ms);
        if (ms < best_ms) {
          best = cand;
          best_ms = ms;
        }
      }
    }
    if (same(best, at_start)) break;
  }
  *best_out = best;
  if (n_trials) *n_trials = (int)timed.size();
  return YC_OK;
}

extern "C" int yc_batch_tune(yc_ctx* ctx, const yc_tune_job* jobs, int n_jobs, const yc_batch_cfg* start, int sweeps,
                             yc_batch_cfg* best_out, yc_tune_trial* trials, int trial_cap, int* n_trials) {
  if (!ctx || !jobs || n_jobs <= 0 || !start || !best_out || sweeps < 1 || (trial_cap > 0 && !trials))
    return yc::set_error(YC_E_INVALID, "yc_batch_tune: bad argument");
  int64_t total_px = 0;
  for (int i = 0; i < n_jobs; ++i) {
    if (jobs[i].width <= 0 || jobs[i].height <= 0 || jobs[i].n_pass <= 0 || !jobs[i].seeds_host)
      return yc::set_error(YC_E_INVALID, "yc_batch_tune: a job needs a frame, passes and their seeds");
    total_px += (int64_t)jobs[i].width * jobs[i].height;
  }
  MixClock m{ctx, jobs, n_jobs, std::vector<int>(n_jobs, -1)};
  int r = YC_OK;
  for (int i = 0; i < n_jobs && !r; ++i) r = yc_alloc_accum(ctx, jobs[i].width, jobs[i].height, &m.accs[i]);
  if (!r) r = yc_tune_search(start, total_px, sweeps, mix_clock, &m, best_out, trials, trial_cap, n_trials);
  if (m.err) r = m.err;
  for (int a : m.accs)
    if (a >= 0) yc_free_accum(ctx, a);
  return r;
}
