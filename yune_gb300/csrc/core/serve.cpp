// serve.cpp -- the request server of include/yune_cuda.h (yc_serve_*) and its admission
// rules (yc_admission_*), host code over the batch engine's C-ABI (yc_batch_*).
//
// The reference renders one frame at a time from its GUI loop (src/RendererCore.cpp:
// 248-469). A server instead keeps one long-lived batch whose path slots take pixels
// from every admitted request, so requests that arrive while others render join the same
// wavefront as soon as memory allows (continuous batching). Admission is by device
// bytes: a request holds its accumulator (width * height float4) and its seeds while it
// runs. The rules live in yc_admission, which needs no device.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <vector>

#include "yune_cuda.h"

namespace yc {
int set_error(int code, const char* msg);   // api.cu: sets yc_last_error()
}
using yc::set_error;

static_assert(sizeof(yc_request_desc) == 144, "yc_request_desc: cam, cfg, four ints, a pointer");
static_assert(sizeof(yc_serve_cfg) == 64, "yc_serve_cfg: 16 bytes, then yc_batch_cfg (12 ints)");
static_assert(sizeof(yc_request_info) == 48, "yc_request_info: two ints, two int64, three doubles");

// ---------------------------------------------------------------------------------------
// admission
struct yc_admission {
  struct Req {
    uint64_t bytes;
    int32_t state;
  };
  uint64_t budget = 0, in_use = 0;
  int32_t max_queue = -1;
  int32_t running = 0;          // requests holding bytes (running or cancelling)
  std::deque<int64_t> waiting;  // arrival order
  std::vector<Req> reqs;        // by ticket
};

namespace {

bool valid_ticket(const yc_admission* a, int64_t t) { return a && t >= 0 && t < (int64_t)a->reqs.size(); }

void admit(yc_admission* a, int64_t t) {
  a->reqs[t].state = YC_REQ_RUNNING;
  a->in_use += a->reqs[t].bytes;
  ++a->running;
}

}  // namespace

extern "C" {

int yc_admission_create(uint64_t budget_bytes, int32_t max_queue, yc_admission** out) {
  if (!out) return set_error(YC_E_INVALID, "out is NULL");
  *out = new (std::nothrow) yc_admission;
  if (!*out) return set_error(YC_E_NOMEM, "host allocation failed");
  (*out)->budget = budget_bytes;
  (*out)->max_queue = max_queue;
  return YC_OK;
}

int yc_admission_submit(yc_admission* a, uint64_t bytes, int64_t* ticket, int32_t* state) {
  if (!a || !ticket || !state) return set_error(YC_E_INVALID, "NULL argument");
  const int64_t t = (int64_t)a->reqs.size();
  int32_t st;
  if (bytes > a->budget) st = YC_REQ_REJECTED_BUDGET;
  else if (a->waiting.empty() && a->in_use + bytes <= a->budget) st = YC_REQ_RUNNING;
  else if (a->max_queue >= 0 && (int64_t)a->waiting.size() >= a->max_queue) st = YC_REQ_REJECTED_QUEUE;
  else st = YC_REQ_WAITING;
  a->reqs.push_back({bytes, st});
  if (st == YC_REQ_RUNNING) {
    a->reqs[t].state = YC_REQ_WAITING;
    admit(a, t);
  } else if (st == YC_REQ_WAITING) {
    a->waiting.push_back(t);
  }
  *ticket = t;
  *state = st;
  return YC_OK;
}

int yc_admission_next(yc_admission* a, int64_t* ticket) {
  if (!a || !ticket) return set_error(YC_E_INVALID, "NULL argument");
  *ticket = -1;
  if (a->waiting.empty()) return YC_OK;
  const int64_t t = a->waiting.front();
  if (a->in_use + a->reqs[t].bytes > a->budget) return YC_OK;   // the oldest waits; no one overtakes it
  a->waiting.pop_front();
  admit(a, t);
  *ticket = t;
  return YC_OK;
}

int yc_admission_cancel(yc_admission* a, int64_t t, int32_t* state) {
  if (!valid_ticket(a, t)) return set_error(YC_E_NOTFOUND, "unknown ticket");
  yc_admission::Req& r = a->reqs[t];
  if (r.state == YC_REQ_WAITING) {
    a->waiting.erase(std::find(a->waiting.begin(), a->waiting.end(), t));
    r.state = YC_REQ_CANCELLED;
  } else if (r.state == YC_REQ_RUNNING) {
    r.state = YC_REQ_CANCELLING;
  }
  if (state) *state = r.state;
  return YC_OK;
}

int yc_admission_finish(yc_admission* a, int64_t t, int32_t* state) {
  if (!valid_ticket(a, t)) return set_error(YC_E_NOTFOUND, "unknown ticket");
  yc_admission::Req& r = a->reqs[t];
  if (r.state != YC_REQ_RUNNING && r.state != YC_REQ_CANCELLING)
    return set_error(YC_E_INVALID, "only a running or cancelling request can finish");
  r.state = r.state == YC_REQ_RUNNING ? YC_REQ_DONE : YC_REQ_CANCELLED;
  a->in_use -= r.bytes;
  --a->running;
  if (state) *state = r.state;
  return YC_OK;
}

int yc_admission_state(const yc_admission* a, int64_t t, int32_t* state) {
  if (!valid_ticket(a, t)) return set_error(YC_E_NOTFOUND, "unknown ticket");
  if (!state) return set_error(YC_E_INVALID, "state is NULL");
  *state = a->reqs[t].state;
  return YC_OK;
}

int yc_admission_usage(const yc_admission* a, uint64_t* bytes, int32_t* waiting, int32_t* running) {
  if (!a) return set_error(YC_E_INVALID, "admission is NULL");
  if (bytes) *bytes = a->in_use;
  if (waiting) *waiting = (int32_t)a->waiting.size();
  if (running) *running = a->running;
  return YC_OK;
}

int yc_admission_destroy(yc_admission* a) {
  delete a;
  return YC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// server
namespace {

struct ServeReq {
  yc_request_desc desc{};
  std::vector<uint32_t> seeds;
  int32_t state = YC_REQ_WAITING;
  int32_t accum = -1;
  int32_t job = -1;
  int64_t pixels_total = 0, pixels_done = 0;
  bool holds_bytes = false;   // the admission counts its bytes
  double t_submit = -1.0, t_admit = -1.0, t_finish = -1.0;
};

uint64_t request_bytes(const yc_request_desc& d) {
  return (uint64_t)d.width * (uint64_t)d.height * 16u + (uint64_t)d.n_pass * 4u;
}

}  // namespace

struct yc_server {
  yc_ctx* ctx = nullptr;
  yc_serve_cfg cfg{};
  yc_admission* adm = nullptr;
  yc_batch* batch = nullptr;
  std::vector<ServeReq> reqs;     // by request id (= admission ticket)
  std::vector<int64_t> live;      // running or cancelling, in admission order
  bool started = false;           // the batch has run (its traversal stack is fixed)
  int32_t stack_cap = 0;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

// the job of an admitted request: its accumulator and its passes in the batch
int start_request(yc_server* s, int64_t id) {
  ServeReq& q = s->reqs[id];
  int aid = -1;
  if (int r = yc_alloc_accum(s->ctx, q.desc.width, q.desc.height, &aid)) return r;
  int job = -1;
  const int r = yc_batch_add_job(s->batch, q.desc.scene_id, aid, &q.desc.cam, q.seeds.data(), q.desc.n_pass, 1,
                                 &q.desc.cfg, &job);
  if (r) {
    yc_free_accum(s->ctx, aid);
    return r;
  }
  q.accum = aid;
  q.job = job;
  q.state = YC_REQ_RUNNING;
  q.holds_bytes = true;
  q.t_admit = s->now();
  s->live.push_back(id);
  return YC_OK;
}

int admit_waiting(yc_server* s) {
  for (;;) {
    int64_t t = -1;
    if (int r = yc_admission_next(s->adm, &t)) return r;
    if (t < 0) return YC_OK;
    if (int r = start_request(s, t)) return r;
  }
}

void release_bytes(yc_server* s, ServeReq& q, int64_t id) {
  if (q.accum >= 0) yc_free_accum(s->ctx, q.accum);
  q.accum = -1;
  if (q.holds_bytes) yc_admission_finish(s->adm, id, nullptr);
  q.holds_bytes = false;
}

}  // namespace

extern "C" {

int yc_serve_create(yc_ctx* ctx, const yc_serve_cfg* cfg, yc_server** out) {
  if (!ctx || !cfg || !out) return set_error(YC_E_INVALID, "NULL argument");
  *out = nullptr;
  yc_server* s = new (std::nothrow) yc_server;
  if (!s) return set_error(YC_E_NOMEM, "host allocation failed");
  s->ctx = ctx;
  s->cfg = *cfg;
  int r = yc_admission_create(cfg->budget_bytes, cfg->max_queue, &s->adm);
  if (!r) r = yc_batch_create(ctx, &s->cfg.batch, &s->batch);
  if (r) {
    yc_admission_destroy(s->adm);
    delete s;
    return r;
  }
  s->stack_cap = cfg->batch.stack_cap;
  *out = s;
  return YC_OK;
}

int yc_serve_submit(yc_server* s, const yc_request_desc* d, int64_t* id, int32_t* state) {
  if (!s || !d || !id || !state) return set_error(YC_E_INVALID, "NULL argument");
  if (d->width <= 0 || d->height <= 0 || d->n_pass <= 0 || !d->seeds_host)
    return set_error(YC_E_INVALID, "a request needs a positive frame size, passes and their seeds");
  if (d->cfg.integrator != YC_UDPT) return set_error(YC_E_INVALID, "the server renders with YC_UDPT");
  int depth = 0;
  if (int r = yc_scene_depth(s->ctx, d->scene_id, &depth)) return r;
  if (s->started && depth + 2 > s->stack_cap)
    return set_error(YC_E_INVALID, "scene BVH deeper than the running batch's traversal stack (set batch.stack_cap)");
  ServeReq q;
  q.desc = *d;
  q.seeds.assign(d->seeds_host, d->seeds_host + d->n_pass);
  q.desc.seeds_host = nullptr;
  q.pixels_total = (int64_t)d->width * d->height;
  q.t_submit = s->now();
  int64_t t = -1;
  int32_t st = 0;
  if (int r = yc_admission_submit(s->adm, request_bytes(*d), &t, &st)) return r;
  if (t != (int64_t)s->reqs.size()) return set_error(YC_E_INVALID, "admission ticket out of order");
  q.state = st;
  if (st == YC_REQ_REJECTED_BUDGET || st == YC_REQ_REJECTED_QUEUE) q.t_finish = q.t_submit;
  s->reqs.push_back(std::move(q));
  if (!s->started) s->stack_cap = std::max(s->stack_cap, depth + 2);
  if (st == YC_REQ_RUNNING) {
    s->reqs[t].state = YC_REQ_WAITING;
    if (int r = start_request(s, t)) {
      yc_admission_cancel(s->adm, t, nullptr);
      yc_admission_finish(s->adm, t, nullptr);
      s->reqs[t].state = YC_REQ_CANCELLED;
      s->reqs[t].t_finish = s->now();
      return r;
    }
  }
  *id = t;
  *state = s->reqs[t].state;
  return YC_OK;
}

int yc_serve_cancel(yc_server* s, int64_t id) {
  if (!s || id < 0 || id >= (int64_t)s->reqs.size()) return set_error(YC_E_NOTFOUND, "unknown request");
  ServeReq& q = s->reqs[id];
  if (q.state == YC_REQ_WAITING) {
    yc_admission_cancel(s->adm, id, nullptr);
    q.state = YC_REQ_CANCELLED;
    q.t_finish = s->now();
  } else if (q.state == YC_REQ_RUNNING) {
    if (int r = yc_batch_cancel_job(s->batch, q.job)) return r;
    yc_admission_cancel(s->adm, id, nullptr);
    q.state = YC_REQ_CANCELLING;
  }
  return YC_OK;
}

int yc_serve_step(yc_server* s, int max_launches, int32_t* running, int32_t* waiting) {
  if (!s || max_launches < 0) return set_error(YC_E_INVALID, "bad argument");
  if (int r = admit_waiting(s)) return r;
  if (!s->live.empty() && max_launches > 0) {
    int unfinished = 0;
    if (int r = yc_batch_run(s->batch, max_launches, &unfinished)) return r;
    s->started = true;
  }
  std::vector<int64_t> still;
  for (int64_t id : s->live) {
    ServeReq& q = s->reqs[id];
    int64_t done = 0, total = 0;
    if (int r = yc_batch_job_progress(s->batch, q.job, &done, &total)) return r;
    q.pixels_done = done;
    if (done < total) {
      still.push_back(id);
      continue;
    }
    q.state = q.state == YC_REQ_CANCELLING ? YC_REQ_CANCELLED : YC_REQ_DONE;
    q.t_finish = s->now();
    if (!s->cfg.keep_results || q.state == YC_REQ_CANCELLED) release_bytes(s, q, id);
  }
  s->live.swap(still);
  if (int r = admit_waiting(s)) return r;   // memory freed by the finished requests
  int32_t w = 0;
  yc_admission_usage(s->adm, nullptr, &w, nullptr);
  if (running) *running = (int32_t)s->live.size();
  if (waiting) *waiting = w;
  return YC_OK;
}

int yc_serve_info(yc_server* s, int64_t id, yc_request_info* out) {
  if (!s || !out) return set_error(YC_E_INVALID, "NULL argument");
  if (id < 0 || id >= (int64_t)s->reqs.size()) return set_error(YC_E_NOTFOUND, "unknown request");
  const ServeReq& q = s->reqs[id];
  out->state = q.state;
  out->accum_id = q.accum;
  out->pixels_done = q.state == YC_REQ_DONE ? q.pixels_total : q.pixels_done;
  out->pixels_total = q.pixels_total;
  out->submit_s = q.t_submit;
  out->admit_s = q.t_admit;
  out->finish_s = q.t_finish;
  return YC_OK;
}

int yc_serve_read(yc_server* s, int64_t id, float* rgba) {
  if (!s || !rgba) return set_error(YC_E_INVALID, "NULL argument");
  if (id < 0 || id >= (int64_t)s->reqs.size()) return set_error(YC_E_NOTFOUND, "unknown request");
  const ServeReq& q = s->reqs[id];
  if (q.state != YC_REQ_DONE || q.accum < 0)
    return set_error(YC_E_INVALID, "the request is not done or its result was not kept (keep_results)");
  return yc_read_accum(s->ctx, q.accum, rgba);
}

int yc_serve_release(yc_server* s, int64_t id) {
  if (!s) return set_error(YC_E_INVALID, "server is NULL");
  if (id < 0 || id >= (int64_t)s->reqs.size()) return set_error(YC_E_NOTFOUND, "unknown request");
  ServeReq& q = s->reqs[id];
  if (q.state != YC_REQ_DONE) return set_error(YC_E_INVALID, "only a done request is released");
  release_bytes(s, q, id);
  return YC_OK;
}

double yc_serve_clock(const yc_server* s) { return s ? s->now() : -1.0; }

int yc_serve_destroy(yc_server* s) {
  if (!s) return YC_OK;
  if (s->batch) yc_batch_destroy(s->batch);   // waits for the batch's work
  for (size_t i = 0; i < s->reqs.size(); ++i)
    if (s->reqs[i].accum >= 0) yc_free_accum(s->ctx, s->reqs[i].accum);
  yc_admission_destroy(s->adm);
  delete s;
  return YC_OK;
}

}  // extern "C"
