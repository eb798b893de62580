// Serving loop (include/rils_rols_serve.h): fit jobs admitted by
// device-memory footprint, each run as one search on the device context of
// its worker, on that context's streams.
//
// The workers are max_active threads.  A free worker takes the job at the
// head of the queue once its footprint fits what the jobs in flight leave of
// the budget.  When the head does not fit, one of the next kBypassWindow
// jobs that does fit may start instead, but the head is passed over at most
// kMaxBypass times: jobs start in arrival order within a window, and a large
// job waits for a bounded number of smaller ones.
//
// A worker keeps its context from job to job (its scratch buffers only grow,
// and come from the device's stream-ordered pool, so a job's start and end
// cost no device-wide wait).  It is charged the larger of the job's
// footprint and what its context already holds; a context holding more than
// twice a new job's footprint is released first, so that one large job does
// not pin its memory for every later small one.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../../include/rils_rols_gb300.h"
#include "../../../include/rils_rols_host.h"
#include "../../../include/rils_rols_serve.h"
#include "../common/error.h"
#include "search.h"

namespace {

using Clock = std::chrono::steady_clock;

double seconds(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

int64_t round_up64(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// Device memory of one job: the resident dataset (X and y in FP64 and as
// double-float pairs) plus the context's two scratch limits and a fixed
// allowance for the per-round buffers (programs, pair sums, results).  The
// limits also bound the job's column caches (factor columns kept across its
// rounds): 4096 double-float and 4096 FP64 columns where they fit the caps,
// enough for most of a search's rounds to read instead of evaluate.
struct Footprint {
  int64_t scratch, table, total;
};
Footprint job_footprint(int64_t n, int64_t d) {
  const int64_t n_pad = round_up64(std::max<int64_t>(n, 1), 4096);
  const int64_t col64 = n_pad * 8;
  Footprint f;
  // 8192 FP64 columns (half of them the FP64 column cache, half QR working
  // columns) and 4096 double-float factor columns, within [64 MiB, 16 GiB] /
  // [64 MiB, 8 GiB]
  f.scratch = std::min<int64_t>(std::max<int64_t>(8192 * col64, 64ll << 20), 16ll << 30);
  f.table = std::min<int64_t>(std::max<int64_t>(4096 * col64, 64ll << 20), 8ll << 30);
  const int64_t dataset = n_pad * (d + 1) * (8 + 4 + 4);
  f.total = dataset + f.scratch + f.table + (256ll << 20) + 64 * n_pad;
  return f;
}

constexpr int kBypassWindow = 16;  // queue positions a free worker looks at
constexpr int kMaxBypass = 8;      // times the head of the queue may be passed over

struct Job {
  int64_t id = 0;
  int32_t bypassed = 0;  // jobs admitted ahead of it while it headed the queue
  rrs_job_params p{};
  int32_t n = 0, d = 0;
  std::vector<double> X, y;
  Footprint fp{};
  int32_t state = RRS_QUEUED;
  Clock::time_point t_submit, t_start, t_end;
  std::string model, error;
  int32_t fit_calls = 0;
  double best_time = 0;
  int64_t rounds = 0, candidates = 0;
};

// Device backend of one job: its worker's context (created on the server's
// device when the worker has none), with the job's scratch limits.
struct JobDevice {
  int32_t device;
  Footprint fp;
  rrg_context** ctx;  // the worker's context slot
};
void* jd_dataset_create(void* self, const double* X, const double* y, int64_t n, int32_t d) {
  JobDevice* j = static_cast<JobDevice*>(self);
  if (!*j->ctx && rrg_context_create(j->device, j->ctx) != RRG_OK) return nullptr;
  if (rrg_context_set_limits(*j->ctx, j->fp.scratch, j->fp.table) != RRG_OK) return nullptr;
  rrg_dataset* ds = nullptr;
  if (rrg_dataset_create(*j->ctx, X, y, n, d, &ds) != RRG_OK) return nullptr;
  return ds;
}

// What a worker whose context holds `held` bytes is charged for a job of
// footprint `fp`: a context more than twice the job's size is released first.
int64_t charge_for(int64_t fp, int64_t held) { return held > 2 * fp ? fp : std::max(fp, held); }
int32_t jd_eval(void* ds, const rrg_batch* b, int32_t p, rrg_result* r, double* c) {
  return rrg_eval(static_cast<rrg_dataset*>(ds), b, p, r, c);
}
int32_t jd_predict(void* ds, const rrg_batch* b, double* v) { return rrg_predict(static_cast<rrg_dataset*>(ds), b, v); }
void jd_dataset_destroy(void* ds) { rrg_dataset_destroy(static_cast<rrg_dataset*>(ds)); }

}  // namespace

struct rrs_server {
  int32_t device = 0;
  int64_t budget = 0, used = 0;
  int32_t max_active = 1, running = 0, peak_running = 0;
  bool has_backend = false, stopping = false, started = false;
  rrh_backend backend{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> queue;
  std::map<int64_t, std::unique_ptr<Job>> jobs;
  int64_t next_id = 0;
  Clock::time_point t_first;
  Clock::time_point t_last;
  bool any_done = false;
  std::vector<std::thread> workers;

  void worker();
  void run(Job& j, rrg_context** ctx);
  // the queue position a worker whose context holds `held` bytes may
  // admit, or -1
  int pick(int64_t held);
};

int rrs_server::pick(int64_t held) {
  const int w = (int)std::min<size_t>(queue.size(), kBypassWindow);
  for (int i = 0; i < w; ++i) {
    const Job& j = *jobs[queue[i]];
    if (used + charge_for(j.fp.total, held) <= budget) return i;
    if (i == 0 && j.bypassed >= kMaxBypass) return -1;  // the head waits for no more jobs
  }
  return -1;
}

void rrs_server::run(Job& j, rrg_context** ctx) {
  rrh::Search search(j.p.classification != 0, j.p.max_fit_calls, j.p.max_seconds, j.p.complexity_penalty,
                     j.p.max_complexity, j.p.sample_size, false, j.p.random_state);
  search.set_precision(j.p.precision);
  JobDevice dev{device, j.fp, ctx};
  if (has_backend) {
    search.set_backend(backend);
  } else {
    rrh_backend be;
    be.self = &dev;
    be.dataset_create = jd_dataset_create;
    be.eval = jd_eval;
    be.predict = jd_predict;
    be.dataset_destroy = jd_dataset_destroy;
    search.set_backend(be);
  }
  try {
    search.fit(j.X.data(), j.y.data(), j.n, j.d);
    j.model = search.model_string();
    j.fit_calls = search.fit_calls();
    j.best_time = search.best_time();
    j.rounds = search.counter(2);
    j.candidates = search.counter(3);
    j.state = RRS_DONE;
  } catch (const std::exception& e) {
    j.error = e.what();
    j.state = RRS_FAILED;
  }
  // the search's dataset is gone with `search`; the context stays with the worker
}

void rrs_server::worker() {
  rrg_context* ctx = nullptr;  // kept from job to job
  int64_t held = 0;            // device bytes its scratch holds
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    int at = -1;
    cv_work.wait(lk, [&] {
      if (stopping) return true;
      if (queue.empty()) return false;
      at = pick(held);
      return at >= 0;
    });
    if (stopping) break;
    Job& j = *jobs[queue[at]];
    if (at > 0) jobs[queue.front()]->bypassed += 1;
    queue.erase(queue.begin() + at);
    if (ctx && held > 2 * j.fp.total) {
      // far larger than this job needs: its memory goes back first
      rrg_context_destroy(ctx);
      ctx = nullptr;
      held = 0;
    }
    const int64_t charge = charge_for(j.fp.total, held);
    used += charge;
    ++running;
    peak_running = std::max(peak_running, running);
    j.state = RRS_RUNNING;
    j.t_start = Clock::now();
    lk.unlock();
    run(j, &ctx);
    const int64_t now_held = ctx ? rrg_context_memory(ctx) : 0;
    lk.lock();
    j.t_end = Clock::now();
    j.X.clear();
    j.X.shrink_to_fit();
    j.y.clear();
    j.y.shrink_to_fit();
    used -= charge;
    held = std::max<int64_t>(now_held, 0);
    --running;
    t_last = j.t_end;
    any_done = true;
    cv_done.notify_all();
    cv_work.notify_all();
  }
  lk.unlock();
  if (ctx) rrg_context_destroy(ctx);
}

extern "C" {

rrs_server* rrs_create(int32_t device, int64_t memory_budget_bytes, int32_t max_active) {
  if (device < 0 || memory_budget_bytes < 0 || max_active < 1 || max_active > 256) {
    rrc::set_error("rrs_create: invalid arguments");
    return nullptr;
  }
  try {
    rrs_server* s = new rrs_server();
    s->device = device;
    s->budget = memory_budget_bytes;
    s->max_active = max_active;
    return s;
  } catch (const std::exception& e) {
    rrc::set_error(e.what());
    return nullptr;
  }
}

// The budget of 0 is resolved and the workers are started at the first
// submission, so that a CPU backend installed before it needs no device.
static bool start_locked(rrs_server* s) {
  if (s->started) return true;
  if (s->budget == 0) {
    if (s->has_backend) {
      s->budget = INT64_MAX;
    } else {
      int64_t free_b = 0, total_b = 0;
      if (rrg_device_memory(s->device, &free_b, &total_b) != RRG_OK) return false;
      s->budget = free_b / 10 * 8;
    }
  }
  for (int i = 0; i < s->max_active; ++i) s->workers.emplace_back([s] { s->worker(); });
  s->started = true;
  return true;
}

void rrs_destroy(rrs_server* s) {
  if (!s) return;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    // queued jobs are dropped; jobs in flight finish
    for (int64_t id : s->queue) {
      s->jobs[id]->state = RRS_FAILED;
      s->jobs[id]->error = "server destroyed before the job started";
    }
    s->queue.clear();
    s->stopping = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  delete s;
}

int32_t rrs_set_backend(rrs_server* s, const rrh_backend* be) {
  if (!s) return RRG_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->started) {
    rrc::set_error("rrs_set_backend: jobs were already submitted");
    return RRG_E_INVALID;
  }
  s->has_backend = be != nullptr;
  if (be) s->backend = *be;
  return RRG_OK;
}

int64_t rrs_submit(rrs_server* s, const double* X, const double* y, int32_t n, int32_t d, const rrs_job_params* p) {
  if (!s || !X || !y || !p || n <= 0 || d <= 0 ||
      (p->precision != RRG_PLAIN_FP64 && p->precision != RRG_MIXED && p->precision != RRG_MIXED_CERTIFIED)) {
    rrc::set_error("rrs_submit: invalid arguments");
    return -(int64_t)RRG_E_INVALID;
  }
  try {
    auto j = std::make_unique<Job>();
    j->p = *p;
    j->n = n;
    j->d = d;
    j->X.assign(X, X + (size_t)n * d);
    j->y.assign(y, y + n);
    j->fp = job_footprint(n, d);
    std::unique_lock<std::mutex> lk(s->mu);
    if (!start_locked(s)) return -(int64_t)RRG_E_NO_DEVICE;
    if (j->fp.total > s->budget) {
      rrc::set_error("rrs_submit: the job's device footprint exceeds the server's memory budget");
      return -(int64_t)RRG_E_OOM;
    }
    j->id = s->next_id++;
    j->t_submit = Clock::now();
    if (s->jobs.empty()) s->t_first = j->t_submit;
    const int64_t id = j->id;
    s->jobs[id] = std::move(j);
    s->queue.push_back(id);
    lk.unlock();
    s->cv_work.notify_one();
    return id;
  } catch (const std::exception& e) {
    rrc::set_error(e.what());
    return -(int64_t)RRG_E_OOM;
  }
}

int32_t rrs_wait(rrs_server* s, int64_t job, int32_t timeout_ms) {
  if (!s) return RRG_E_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job);
  if (it == s->jobs.end()) {
    rrc::set_error("rrs_wait: unknown job");
    return RRG_E_INVALID;
  }
  Job& j = *it->second;
  auto finished = [&] { return j.state == RRS_DONE || j.state == RRS_FAILED; };
  if (timeout_ms < 0) {
    s->cv_done.wait(lk, finished);
    return RRG_OK;
  }
  return s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished) ? RRG_OK : RRG_E_TIMEOUT;
}

int32_t rrs_result(rrs_server* s, int64_t job, char* model, int32_t cap, rrs_job_info* info) {
  if (!s) return RRG_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job);
  if (it == s->jobs.end()) {
    rrc::set_error("rrs_result: unknown job");
    return -1;
  }
  const Job& j = *it->second;
  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->state = j.state;
    info->fit_calls = j.fit_calls;
    info->footprint_bytes = j.fp.total;
    info->best_time = j.best_time;
    info->device_rounds = j.rounds;
    info->candidates = j.candidates;
    const auto now = Clock::now();
    if (j.state == RRS_QUEUED) {
      info->queued_s = seconds(j.t_submit, now);
    } else {
      info->queued_s = seconds(j.t_submit, j.t_start);
      const bool fin = j.state == RRS_DONE || j.state == RRS_FAILED;
      info->run_s = seconds(j.t_start, fin ? j.t_end : now);
      if (fin) info->time_to_model_s = seconds(j.t_submit, j.t_end);
    }
  }
  const std::string& out = j.state == RRS_FAILED ? j.error : j.model;
  if ((int64_t)out.size() + 1 > cap || !model) return -(int32_t)(out.size() + 1);
  std::memcpy(model, out.c_str(), out.size() + 1);
  return (int32_t)out.size();
}

int32_t rrs_stats_get(rrs_server* s, rrs_stats* out) {
  if (!s || !out) return RRG_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  std::vector<double> ttm;
  for (auto& kv : s->jobs) {
    const Job& j = *kv.second;
    ++out->submitted;
    switch (j.state) {
      case RRS_QUEUED: ++out->queued; break;
      case RRS_RUNNING: ++out->running; break;
      case RRS_DONE:
        ++out->done;
        out->candidates += j.candidates;
        ttm.push_back(seconds(j.t_submit, j.t_end));
        break;
      default:
        ++out->failed;
        if (j.t_end > j.t_submit) ttm.push_back(seconds(j.t_submit, j.t_end));
    }
  }
  if (!ttm.empty()) {
    std::sort(ttm.begin(), ttm.end());
    // nearest-rank percentiles
    auto pct = [&](double q) {
      size_t k = (size_t)std::ceil(q * ttm.size());
      return ttm[std::min(ttm.size() - 1, k == 0 ? 0 : k - 1)];
    };
    out->p50_time_to_model_s = pct(0.50);
    out->p99_time_to_model_s = pct(0.99);
    double sum = 0;
    for (double t : ttm) sum += t;
    out->mean_time_to_model_s = sum / ttm.size();
  }
  if (s->any_done) out->wall_s = seconds(s->t_first, s->t_last);
  out->peak_running = s->peak_running;
  return RRG_OK;
}

const char* rrs_last_error(void) { return rrc::get_error(); }

}  // extern "C"
