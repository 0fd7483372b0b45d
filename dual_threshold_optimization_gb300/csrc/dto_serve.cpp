// dto_serve.cpp -- request executor and batch entry point.
//
// The reference runs one permutation null per process invocation
// (src/main.rs:122-166: tasks over threads, src/run/single_node.rs:83-137).
// Serving many of them on one GPU is this file: a server owns `lanes` lanes
// (dto_host.h), each with its own two streams, scratch and table screens,
// and one worker thread per lane.  Requests queue in arrival order; the head
// of the queue is admitted as soon as a lane is free and its device working
// set fits under the memory budget next to the requests already running, so
// requests that arrive while others are on the GPU start as slots and memory
// free up, and their kernels overlap on the device.  A request computes
// exactly what dto_run_range computes for it alone: permutations are a
// function of (seed, stream id, permutation id), and every kernel's result is
// independent of what else runs.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dto_host.h"

using namespace dto;

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
  dto_job id = 0;
  dto_pair* pair = nullptr;
  uint32_t first = 1;
  int64_t n_perm = 0;
  uint64_t seed = 0;
  int precision = DTO_PRECISION_SCREEN;
  dto_result* out_unpermuted = nullptr;
  double* out_minp = nullptr;
  dto_summary* out_summary = nullptr;
  long long need = 0;  // device bytes reserved while it runs
  int status = DTO_OK;
  bool done = false;
  bool started = false;
  std::atomic<int> cancel{0};  // set by dto_serve_cancel; the run stops at its next batch
  std::string err;
  Clock::time_point t_submit, t_start, t_end;
};

}  // namespace

struct dto_server {
  dto_ctx* ctx = nullptr;
  long long budget = 0;  // 0: no budget
  long long reserved = 0;
  int running = 0;
  std::vector<Lane*> lanes;
  std::vector<std::string> lane_err;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::unordered_map<dto_job, Job*> jobs;
  dto_job next_id = 1;
  bool stop = false;
  std::string err;
  long long completed = 0;
};

namespace {

bool admissible(const dto_server* s, const Job* j) {
  if (s->budget <= 0) return true;
  return s->running == 0 || s->reserved + j->need <= s->budget;
}

// Labels of the requests a worker takes into one wave (continuous batching:
// short screen requests queued together share one multi-pair sweep).
constexpr long long kGroupLabelBytes = 4LL << 30;

void worker(dto_server* s, int w) {
  Lane* L = s->lanes[(size_t)w];
  cudaSetDevice(s->ctx->device);
  for (;;) {
    std::vector<Job*> group;
    bool wave = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_work.wait(lk, [&] { return s->stop || (!s->queue.empty() && admissible(s, s->queue.front())); });
      if (s->queue.empty() || !admissible(s, s->queue.front())) {
        if (s->stop) return;
        continue;
      }
      Job* j = s->queue.front();
      s->queue.pop_front();
      group.push_back(j);
      // a request that a wave takes brings the queued requests a wave also
      // takes, in arrival order, while their labels fit and memory admits them
      wave = wave_eligible(s->ctx, j->pair, j->n_perm, j->precision);
      if (wave) {
        long long bytes = wave_label_bytes(j->pair, j->n_perm);
        s->reserved += j->need;
        s->running += 1;
        for (auto it = s->queue.begin(); it != s->queue.end() && bytes < kGroupLabelBytes;) {
          Job* x = *it;
          const long long b = wave_label_bytes(x->pair, x->n_perm);
          if (bytes + b <= kGroupLabelBytes && admissible(s, x) &&
              wave_eligible(s->ctx, x->pair, x->n_perm, x->precision)) {
            group.push_back(x);
            bytes += b;
            s->reserved += x->need;
            s->running += 1;
            it = s->queue.erase(it);
          } else {
            ++it;
          }
        }
      } else {
        s->reserved += j->need;
        s->running += 1;
      }
      for (Job* x : group) {
        x->started = true;
        x->t_start = Clock::now();
      }
    }
    s->lane_err[(size_t)w].clear();
    int rc = DTO_OK;
    std::vector<dto_result> unperm(group.size());
    if (wave) {
      // the group's runs in waves (requests in a wave run to the end: a
      // cancel reaches only requests still queued)
      std::vector<WaveJob> wj(group.size());
      for (size_t q = 0; q < group.size(); ++q) {
        Job* x = group[q];
        wj[q].P = x->pair;
        wj[q].first = x->first;
        wj[q].n_perm = x->n_perm;
        wj[q].seed = x->seed;
        wj[q].out_unpermuted = x->out_unpermuted ? x->out_unpermuted : &unperm[q];
        wj[q].out_minp = x->out_minp;
        wj[q].out_summary = x->out_summary;
      }
      rc = lane_wave(L, wj);
    } else {
      Job* j = group[0];
      L->cancel = &j->cancel;
      rc = lane_run_range(L, j->pair, j->first, j->n_perm, j->seed, nullptr, j->precision,
                          j->out_unpermuted ? j->out_unpermuted : &unperm[0], j->out_minp, nullptr, j->out_summary);
      L->cancel = nullptr;
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (Job* x : group) {
        x->status = rc;
        if (rc) x->err = s->lane_err[(size_t)w];
        x->t_end = Clock::now();
        x->done = true;
        s->reserved -= x->need;
        s->running -= 1;
        s->completed += 1;
      }
    }
    s->cv_done.notify_all();
    s->cv_work.notify_all();  // memory freed: the head may now fit
  }
}

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

extern "C" {

int dto_serve_create(dto_ctx* ctx, int lanes, int64_t mem_budget, dto_server** out) {
  if (!ctx || !out || lanes <= 0 || lanes > 64 || mem_budget < 0) return set_err(ctx, DTO_ERR_INVALID, "dto_serve_create: invalid argument");
  *out = nullptr;
  CK(cudaSetDevice(ctx->device));
  dto_server* s = new dto_server();
  s->ctx = ctx;
  s->budget = mem_budget;
  s->lane_err.resize((size_t)lanes);
  for (int w = 0; w < lanes; ++w) {
    Lane* L = nullptr;
    const int rc = lane_create(ctx, &L, &s->lane_err[(size_t)w]);
    if (rc) {
      set_err(ctx, rc, "dto_serve_create: " + s->lane_err[(size_t)w]);
      for (Lane* x : s->lanes) lane_destroy(x);
      delete s;
      return rc;
    }
    L->coop_first = false;  // requests share the GPU: throughput first
    L->use_model = true;    // many pairs, each run once: start from similar pairs' ladders
    s->lanes.push_back(L);
  }
  for (int w = 0; w < lanes; ++w) s->workers.emplace_back(worker, s, w);
  *out = s;
  return DTO_OK;
}

int dto_serve_destroy(dto_server* s) {
  if (!s) return DTO_ERR_INVALID;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->queue.empty() && s->running == 0; });
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (std::thread& t : s->workers) t.join();
  cudaSetDevice(s->ctx->device);
  for (Lane* L : s->lanes) lane_destroy(L);
  for (auto& kv : s->jobs) delete kv.second;
  delete s;
  return DTO_OK;
}

int dto_serve_submit(dto_server* s, dto_pair* pair, uint32_t perm_first, int64_t n_perm, uint64_t seed,
                     int precision, dto_result* out_unpermuted, double* out_minp, dto_summary* out_summary,
                     dto_job* job) {
  if (!s || !pair || !job || pair->ctx != s->ctx) return DTO_ERR_INVALID;
  if (n_perm < 0 || n_perm > 0x7fffffffLL || (long long)perm_first + n_perm > 0xffffffffLL) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = "dto_serve_submit: n_perm out of range";
    return DTO_ERR_INVALID;
  }
  if (precision != DTO_PRECISION_FP64 && precision != DTO_PRECISION_SCREEN) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = "dto_serve_submit: unknown precision";
    return DTO_ERR_INVALID;
  }
  Job* j = new Job();
  j->pair = pair;
  j->first = perm_first;
  j->n_perm = n_perm;
  j->seed = seed;
  j->precision = precision;
  j->out_unpermuted = out_unpermuted;
  j->out_minp = out_minp;
  j->out_summary = out_summary;
  j->need = run_device_bytes(s->ctx, pair, n_perm, false);
  j->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    j->id = s->next_id++;
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    *job = j->id;
  }
  s->cv_work.notify_all();
  return DTO_OK;
}

int dto_serve_poll(dto_server* s, dto_job job, int* done) {
  if (!s || !done) return DTO_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job);
  if (it == s->jobs.end()) return DTO_ERR_NOT_FOUND;
  *done = it->second->done ? 1 : 0;
  return DTO_OK;
}

// Waits for a request (timeout_ms < 0: without limit).  A finished request
// returns its status and is forgotten; one still queued or running when the
// time runs out returns DTO_ERR_TIMEOUT and stays known.
static int serve_wait(dto_server* s, dto_job job, double timeout_ms, double* queue_ms, double* run_ms) {
  if (!s) return DTO_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(job);
  if (it == s->jobs.end()) {
    s->err = "dto_serve_wait: unknown request";
    return DTO_ERR_NOT_FOUND;
  }
  Job* j = it->second;
  if (timeout_ms < 0.0) {
    s->cv_done.wait(lk, [&] { return j->done; });
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms),
                                  [&] { return j->done; })) {
    s->err = j->started ? "dto_serve_wait: the request is still running" : "dto_serve_wait: the request is still queued";
    return DTO_ERR_TIMEOUT;
  }
  if (queue_ms) *queue_ms = j->started ? ms_between(j->t_submit, j->t_start) : ms_between(j->t_submit, j->t_end);
  if (run_ms) *run_ms = j->started ? ms_between(j->t_start, j->t_end) : 0.0;
  const int status = j->status;
  if (status) s->err = j->err;
  s->jobs.erase(it);
  delete j;
  return status;
}

int dto_serve_wait(dto_server* s, dto_job job, double* queue_ms, double* run_ms) {
  return serve_wait(s, job, -1.0, queue_ms, run_ms);
}

int dto_serve_wait_for(dto_server* s, dto_job job, double timeout_ms, double* queue_ms, double* run_ms) {
  if (!(timeout_ms >= 0.0)) return DTO_ERR_INVALID;
  return serve_wait(s, job, timeout_ms, queue_ms, run_ms);
}

int dto_serve_cancel(dto_server* s, dto_job job) {
  if (!s) return DTO_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) {
      s->err = "dto_serve_cancel: unknown request";
      return DTO_ERR_NOT_FOUND;
    }
    Job* j = it->second;
    if (j->done) return DTO_OK;  // finished already: its results stand
    if (!j->started) {
      for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
        if (*q == j) {
          s->queue.erase(q);
          break;
        }
      j->status = DTO_ERR_CANCELLED;
      j->err = "dto_serve_cancel: cancelled before it started";
      j->t_end = Clock::now();
      j->done = true;
    } else {
      j->cancel.store(1);  // the run stops at its next batch boundary
    }
  }
  s->cv_done.notify_all();
  s->cv_work.notify_all();  // the next request may now be the head
  return DTO_OK;
}

const char* dto_serve_last_error(dto_server* s) { return s ? s->err.c_str() : "null server"; }

int dto_serve_stats(dto_server* s, int64_t* queued, int64_t* running, int64_t* completed, int64_t* reserved_bytes) {
  if (!s) return DTO_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = (int64_t)s->queue.size();
  if (running) *running = s->running;
  if (completed) *completed = s->completed;
  if (reserved_bytes) *reserved_bytes = s->reserved;
  return DTO_OK;
}

int64_t dto_run_device_bytes(const dto_pair* pair, int64_t n_perm) {
  if (!pair || n_perm < 0) return -1;
  return run_device_bytes(pair->ctx, pair, n_perm, false);
}

int dto_batch_run(dto_ctx* ctx, int npairs, dto_pair* const* pairs, const int64_t* n_perm, const uint64_t* seeds,
                  int precision, int lanes, dto_result* out_unpermuted, double* const* out_minp,
                  dto_summary* out_summary) {
  if (!ctx || npairs < 0 || (npairs > 0 && (!pairs || !n_perm || !seeds || !out_unpermuted)))
    return set_err(ctx, DTO_ERR_INVALID, "dto_batch_run: null argument");
  if (npairs == 0) return DTO_OK;
  // Runs that a wave takes (dto_wave.cpp: short screen runs of pairs with a
  // ladder) go through waves on the context's own lane in this thread; the
  // others through a server's lanes meanwhile.
  std::vector<dto::WaveJob> wave;
  std::vector<char> in_wave((size_t)npairs, 0);
  for (int q = 0; q < npairs; ++q) {
    if (!dto::wave_eligible(ctx, pairs[q], n_perm[q], precision)) continue;
    dto::WaveJob j;
    j.P = pairs[q];
    j.n_perm = n_perm[q];
    j.seed = seeds[q];
    j.out_unpermuted = &out_unpermuted[q];
    j.out_minp = out_minp ? out_minp[q] : nullptr;
    j.out_summary = out_summary ? &out_summary[q] : nullptr;
    wave.push_back(j);
    in_wave[(size_t)q] = 1;
  }
  dto_server* s = nullptr;
  int rc = DTO_OK;
  if (wave.size() < (size_t)npairs) {
    rc = dto_serve_create(ctx, lanes > 0 ? lanes : 4, 0, &s);
    if (rc) return rc;
  }
  std::vector<dto_job> ids((size_t)npairs, 0);
  int first_bad = DTO_OK;
  for (int q = 0; q < npairs && s; ++q) {
    if (in_wave[(size_t)q]) continue;
    rc = dto_serve_submit(s, pairs[q], 1u, n_perm[q], seeds[q], precision, &out_unpermuted[q],
                          out_minp ? out_minp[q] : nullptr, out_summary ? &out_summary[q] : nullptr, &ids[(size_t)q]);
    if (rc) {
      set_err(ctx, rc, "dto_batch_run: pair " + std::to_string(q) + ": " + dto_serve_last_error(s));
      first_bad = rc;
      break;
    }
  }
  if (!wave.empty() && !first_bad) {
    std::lock_guard<std::mutex> g(ctx->mu);
    dto::Lane* L = ctx->lane0;
    std::string err;
    std::string* prev = L->err;
    L->err = &err;
    rc = dto::lane_wave(L, wave);
    L->err = prev;
    if (rc) {
      ctx->err = "dto_batch_run: " + err;
      first_bad = rc;
    }
  }
  for (int q = 0; q < npairs && s; ++q) {
    if (!ids[(size_t)q]) continue;
    rc = dto_serve_wait(s, ids[(size_t)q], nullptr, nullptr);
    if (rc && !first_bad) {
      set_err(ctx, rc, "dto_batch_run: pair " + std::to_string(q) + ": " + dto_serve_last_error(s));
      first_bad = rc;
    }
  }
  if (s) dto_serve_destroy(s);
  return first_bad;
}

}  // extern "C"
