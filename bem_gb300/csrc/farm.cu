// Request farm: the in-process counterpart of the reference's MPI task farm
// (src/transfer-mpi.cpp:25-190).  There, a Master thread queues
// (a, gap, f, T1, T2) jobs and hands each to an idle Servant process, which
// runs CalcHeatTransfer and sends back one double.  Here the servants are
// lanes: each lane is a context (its own CUDA stream and workspace) driven by
// one host thread, so the solves of several requests overlap on one GPU (the
// latency-bound LU panels and fill tails of one lane run beside the
// tensor-core products of another).  Requests wait in a FIFO; results are
// collected by ticket.  No kernels live here: this file is host C++.
//
// Admission by HBM footprint: a lane starts a request only when the
// request's footprint (bemgpu_solve_footprint) plus what the other lanes hold
// or have reserved fits the farm's budget (by default 90 % of the device
// memory free when the farm was created).  A lane that must wait first gives
// back its own workspace if it holds more than the request needs, then the
// workspaces of idle lanes; requests wait in ticket order, and a request
// larger than the whole budget fails with BEMGPU_ERR_OOM at once.
#include "bemgpu_internal.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

struct FarmJob {
  int64_t ticket = 0;
  bemgpu_tree_t top = nullptr, s = nullptr, t = nullptr;
  bemgpu_solve_req_t req{};
  bemgpu_options_t opt{};
  int precision = 0;
};

enum JobState { QUEUED, RUNNING, DONE };
enum LaneState { IDLE, WAITING, BUSY, TRIMMING };

typedef std::chrono::steady_clock Clock;

struct FarmResult {
  JobState state = QUEUED;
  int status = BEMGPU_OK;
  double P = 0.0;
  bemgpu_solve_info_t info{};
  std::string error;
  Clock::time_point t_submit, t_start;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct bemgpu_farm_s {
  int device = 0;
  std::vector<bemgpu_ctx_t> lanes;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_job, cv_done;
  std::deque<FarmJob> queue;
  std::unordered_map<int64_t, FarmResult> results;  // every ticket not yet collected
  int64_t next_ticket = 1;
  bool stop = false;
  std::string last_error;
  // admission
  size_t budget = 0;
  std::vector<LaneState> state;
  std::vector<size_t> held, reserved;  // workspace held; reserved while running
  std::deque<int64_t> waiters;         // tickets waiting for memory, in order
  std::condition_variable cv_mem;
  int batch = 1;                       // requests a lane solves together at most
};

namespace {

// Gives back lane l's workspace; called with f->mu held, which it releases
// while the context synchronises and frees.
void trim_lane(bemgpu_farm_s *f, int l, std::unique_lock<std::mutex> &lk) {
  const LaneState was = f->state[l];
  f->state[l] = TRIMMING;
  lk.unlock();
  bemgpu_ctx_trim(f->lanes[l]);
  lk.lock();
  f->held[l] = f->reserved[l] = 0;
  f->state[l] = was;
  f->cv_mem.notify_all();
  f->cv_job.notify_all();
}

// Waits until lane `me` may run a request needing `need` bytes.  Called with
// f->mu held and the lane in state WAITING.  Returns false if it can never fit.
bool admit(bemgpu_farm_s *f, int me, int64_t ticket, size_t need, std::unique_lock<std::mutex> &lk) {
  if (need > f->budget) return false;
  f->waiters.push_back(ticket);
  for (;;) {
    if (f->waiters.front() == ticket) {
      size_t others = 0;
      bool running = false;
      for (int l = 0; l < (int)f->lanes.size(); l++)
        if (l != me) {
          others += std::max(f->held[l], f->reserved[l]);
          running |= f->state[l] == BUSY || f->state[l] == TRIMMING;
        }
      if (others + std::max(f->held[me], need) <= f->budget) break;
      if (f->held[me] > need) {
        trim_lane(f, me, lk);
        continue;
      }
      int victim = -1;
      for (int l = 0; l < (int)f->lanes.size(); l++)
        if (l != me && (f->state[l] == IDLE || f->state[l] == WAITING) && f->held[l] > 0) victim = l;
      if (victim >= 0) {
        trim_lane(f, victim, lk);
        continue;
      }
      if (!running) break;  // nothing else holds memory: run (and fail with OOM if it does not fit)
    }
    f->cv_mem.wait(lk);
  }
  f->waiters.pop_front();
  f->reserved[me] = std::max(f->held[me], need);
  f->cv_mem.notify_all();
  return true;
}

bool same_kind(const FarmJob &a, const FarmJob &b) {
  return a.precision == b.precision && a.s->nrwg == b.s->nrwg && a.t->nrwg == b.t->nrwg &&
         memcmp(&a.opt, &b.opt, sizeof a.opt) == 0;
}

void lane_main(bemgpu_farm_s *f, int lane) {
  bemgpu_ctx_t ctx = f->lanes[lane];
  for (;;) {
    std::vector<FarmJob> jobs;
    bool ok;
    {
      std::unique_lock<std::mutex> lk(f->mu);
      f->cv_job.wait(lk, [f, lane] { return (f->stop || !f->queue.empty()) && f->state[lane] != TRIMMING; });
      if (f->queue.empty()) return;  // stopping, nothing left
      jobs.push_back(f->queue.front());
      f->queue.pop_front();
      // continuous batching: queued requests of the same sizes, precision and
      // options join this one (in queue order), up to the farm's batch size
      for (auto it = f->queue.begin(); it != f->queue.end() && (int)jobs.size() < f->batch;) {
        if (same_kind(*it, jobs[0])) {
          jobs.push_back(*it);
          it = f->queue.erase(it);
        } else {
          ++it;
        }
      }
      const FarmJob &job = jobs[0];
      f->state[lane] = WAITING;
      int64_t need = jobs.size() == 1 ? bemgpu_ctx_solve_footprint(ctx, job.s->nrwg, job.t->nrwg, job.precision)
                                      : bemgpu_batch_footprint((int)jobs.size(), job.s->nrwg, job.t->nrwg,
                                                               job.precision);
      if (jobs.size() > 1 && (size_t)need > f->budget) {
        // the batch does not fit the budget: the others go back to the front
        for (size_t k = jobs.size() - 1; k >= 1; k--) f->queue.push_front(jobs[k]);
        jobs.resize(1);
        need = bemgpu_ctx_solve_footprint(ctx, job.s->nrwg, job.t->nrwg, job.precision);
      }
      ok = admit(f, lane, job.ticket, (size_t)need, lk);
      f->state[lane] = ok ? BUSY : IDLE;
      const Clock::time_point now = Clock::now();
      for (const FarmJob &j : jobs) {
        FarmResult &r = f->results[j.ticket];
        r.state = RUNNING;
        r.t_start = now;
        if (!ok) {
          r.state = DONE;
          r.status = BEMGPU_ERR_OOM;
          char buf[160];
          snprintf(buf, sizeof buf, "farm: the request needs %.2f GB, more than the farm's budget of %.2f GB",
                   need / 1e9, f->budget / 1e9);
          r.error = buf;
        }
      }
    }
    if (!ok) {
      f->cv_done.notify_all();
      continue;
    }
    const int nb = (int)jobs.size();
    std::vector<double> P(nb, 0.0);
    std::vector<bemgpu_solve_info_t> info(nb);
    std::vector<int> rcs(nb, BEMGPU_OK);
    if (nb == 1) {
      const FarmJob &job = jobs[0];
      rcs[0] = bemgpu_heat_transfer(ctx, job.top, job.s, job.t, &job.req, &job.opt, job.precision, &P[0], &info[0]);
    } else {
      std::vector<bemgpu_tree_t> tops(nb), ss(nb), ts(nb);
      std::vector<bemgpu_solve_req_t> reqs(nb);
      for (int k = 0; k < nb; k++) {
        tops[k] = jobs[k].top;
        ss[k] = jobs[k].s;
        ts[k] = jobs[k].t;
        reqs[k] = jobs[k].req;
      }
      bemgpu_heat_transfer_batch(ctx, nb, tops.data(), ss.data(), ts.data(), reqs.data(), &jobs[0].opt,
                                 jobs[0].precision, P.data(), info.data(), rcs.data());
    }
    const size_t held = (size_t)std::max<int64_t>(0, bemgpu_ctx_workspace_bytes(ctx));
    {
      std::unique_lock<std::mutex> lk(f->mu);
      const Clock::time_point now = Clock::now();
      for (int k = 0; k < nb; k++) {
        FarmResult &r = f->results[jobs[k].ticket];
        r.state = DONE;
        r.status = rcs[k];
        r.P = P[k];
        r.info = info[k];
        r.info.ms_queued = ms_between(r.t_submit, r.t_start);
        r.info.ms_latency = ms_between(r.t_submit, now);
        if (rcs[k] != BEMGPU_OK) r.error = bemgpu_ctx_last_error(ctx);
      }
      f->held[lane] = held;
      f->reserved[lane] = 0;
      f->state[lane] = IDLE;
      // a request waiting for memory gets this lane's workspace
      if (!f->waiters.empty() && held > 0) trim_lane(f, lane, lk);
      f->cv_mem.notify_all();
    }
    f->cv_done.notify_all();
  }
}

}  // namespace

extern "C" {

int bemgpu_farm_create(int device, int lanes, bemgpu_farm_t *out) {
  if (!out || lanes < 1 || lanes > 16) return BEMGPU_ERR_ARG;
  *out = nullptr;
  bemgpu_farm_s *f = new bemgpu_farm_s();
  f->device = device;
  for (int i = 0; i < lanes; i++) {
    bemgpu_ctx_t c = nullptr;
    const int rc = bemgpu_ctx_create(device, &c);
    if (rc != BEMGPU_OK) {
      for (bemgpu_ctx_t l : f->lanes) bemgpu_ctx_destroy(l);
      delete f;
      return rc;
    }
    f->lanes.push_back(c);
  }
  size_t fr = 0, tot = 0;
  cudaSetDevice(device);
  cudaMemGetInfo(&fr, &tot);
  f->budget = (size_t)(0.9 * (double)fr);
  f->state.assign(lanes, IDLE);
  f->held.assign(lanes, 0);
  f->reserved.assign(lanes, 0);
  for (int i = 0; i < lanes; i++) f->threads.emplace_back(lane_main, f, i);
  *out = f;
  return BEMGPU_OK;
}

int bemgpu_farm_destroy(bemgpu_farm_t f) {
  if (!f) return BEMGPU_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(f->mu);
    // queued requests are dropped (as cancelled); running ones finish
    for (const FarmJob &j : f->queue) {
      FarmResult &r = f->results[j.ticket];
      r.state = DONE;
      r.status = BEMGPU_ERR_CANCELLED;
    }
    f->queue.clear();
    f->stop = true;
  }
  f->cv_job.notify_all();
  for (std::thread &t : f->threads) t.join();
  for (bemgpu_ctx_t c : f->lanes) bemgpu_ctx_destroy(c);
  delete f;
  return BEMGPU_OK;
}

int bemgpu_farm_lanes(bemgpu_farm_t f) { return f ? (int)f->lanes.size() : BEMGPU_ERR_ARG; }

int bemgpu_farm_set_batch(bemgpu_farm_t f, int max_requests) {
  if (!f || max_requests < 1 || max_requests > BEM_MAX_BATCH) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(f->mu);
  f->batch = max_requests;
  return BEMGPU_OK;
}

int bemgpu_farm_set_budget(bemgpu_farm_t f, int64_t bytes) {
  if (!f || bytes <= 0) return BEMGPU_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(f->mu);
    f->budget = (size_t)bytes;
  }
  f->cv_mem.notify_all();
  return BEMGPU_OK;
}

int64_t bemgpu_farm_budget(bemgpu_farm_t f) {
  if (!f) return BEMGPU_ERR_ARG;
  std::lock_guard<std::mutex> lk(f->mu);
  return (int64_t)f->budget;
}

int bemgpu_farm_lane_ctx(bemgpu_farm_t f, int lane, bemgpu_ctx_t *ctx) {
  if (!f || !ctx || lane < 0 || lane >= (int)f->lanes.size()) return BEMGPU_ERR_ARG;
  *ctx = f->lanes[lane];
  return BEMGPU_OK;
}

int bemgpu_farm_submit(bemgpu_farm_t f, bemgpu_tree_t top, bemgpu_tree_t s, bemgpu_tree_t t,
                       const bemgpu_solve_req_t *req, const bemgpu_options_t *opt, int precision, int64_t *ticket) {
  if (!f || !top || !s || !t || !req || !ticket) return BEMGPU_ERR_ARG;
  if (top->geom != s->geom || top->geom != t->geom || top->nrwg != s->nrwg + t->nrwg) {
    std::lock_guard<std::mutex> lk(f->mu);
    f->last_error = "farm_submit: top, s, t must share one geometry and size(top) = size(s) + size(t)";
    return BEMGPU_ERR_ARG;
  }
  if (top->geom->ctx->device != f->device) {
    std::lock_guard<std::mutex> lk(f->mu);
    f->last_error = "farm_submit: the trees live on another device than the farm";
    return BEMGPU_ERR_ARG;
  }
  if (precision != BEMGPU_PREC_FP64 && precision != BEMGPU_PREC_MIXED && precision != BEMGPU_PREC_MIXED_LA) {
    std::lock_guard<std::mutex> lk(f->mu);
    f->last_error = "farm_submit: unknown precision";
    return BEMGPU_ERR_ARG;
  }
  FarmJob j;
  j.top = top;
  j.s = s;
  j.t = t;
  j.req = *req;
  if (opt) j.opt = *opt; else bemgpu_options_default(&j.opt);
  j.precision = precision;
  {
    std::lock_guard<std::mutex> lk(f->mu);
    if (f->stop) return BEMGPU_ERR_ARG;
    j.ticket = f->next_ticket++;
    f->results[j.ticket] = FarmResult();
    f->results[j.ticket].t_submit = Clock::now();
    f->queue.push_back(j);
    *ticket = j.ticket;
  }
  f->cv_job.notify_one();
  return BEMGPU_OK;
}

int bemgpu_farm_poll(bemgpu_farm_t f, int64_t ticket, double timeout_ms, double *P_out, bemgpu_solve_info_t *info) {
  if (!f) return BEMGPU_ERR_ARG;
  std::unique_lock<std::mutex> lk(f->mu);
  auto it = f->results.find(ticket);
  if (it == f->results.end()) {
    f->last_error = "farm_poll: unknown or already collected ticket";
    return BEMGPU_ERR_ARG;
  }
  auto done = [f, ticket] {
    auto i = f->results.find(ticket);
    return i == f->results.end() || i->second.state == DONE;
  };
  if (timeout_ms < 0) {
    f->cv_done.wait(lk, done);
  } else if (timeout_ms > 0) {
    f->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), done);
  }
  it = f->results.find(ticket);
  if (it == f->results.end()) {  // collected meanwhile by another thread
    f->last_error = "farm_poll: ticket collected by another caller";
    return BEMGPU_ERR_ARG;
  }
  if (it->second.state != DONE) return BEMGPU_PENDING;
  const FarmResult r = it->second;
  f->results.erase(it);
  if (P_out) *P_out = r.P;
  if (info) *info = r.info;
  if (r.status != BEMGPU_OK) f->last_error = r.error.empty() ? "farm: request cancelled" : r.error;
  return r.status;
}

int bemgpu_farm_cancel(bemgpu_farm_t f, int64_t ticket) {
  if (!f) return BEMGPU_ERR_ARG;
  bool found = false;
  {
    std::lock_guard<std::mutex> lk(f->mu);
    if (f->results.find(ticket) == f->results.end()) {
      f->last_error = "farm_cancel: unknown or already collected ticket";
      return BEMGPU_ERR_ARG;
    }
    for (auto it = f->queue.begin(); it != f->queue.end(); ++it)
      if (it->ticket == ticket) {
        f->queue.erase(it);
        FarmResult &r = f->results[ticket];
        r.state = DONE;
        r.status = BEMGPU_ERR_CANCELLED;
        found = true;
        break;
      }
  }
  if (found) f->cv_done.notify_all();
  return found ? BEMGPU_OK : BEMGPU_PENDING;
}

const char *bemgpu_farm_last_error(bemgpu_farm_t f) { return f ? f->last_error.c_str() : "null farm"; }

}  // extern "C"
