// Serving loop: flow solves of different meshes and freestream conditions
// arrive at any time and run concurrently on one GPU.
//
// A worker thread owns all GPU work.  Requests wait in a FIFO until a slot
// (a CUDA stream) is free and the HBM budget admits their estimated footprint;
// admission builds the request's device solver on its slot's stream.  Every
// active request then advances one V-cycle at a time: the cycle (a CUDA graph
// launch), an asynchronous copy of the solver's device status block to pinned
// host memory and an event.  When the event has completed the worker reads the
// level-0 density residual and decides: stop (converged, failed, or the cycle
// limit reached: fetch the result, free the solver, release slot and budget)
// or enqueue the next cycle.  Requests therefore join and leave at V-cycle
// boundaries and their kernels overlap on the device (continuous batching at
// V-cycle granularity).  Each request's arithmetic is exactly that of a solver
// running alone, so with the deterministic gather increment a result is
// bit-identical alone and in any mix.
#include <algorithm>
#include <chrono>
#include <memory>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "common.h"
#include "solver_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  int64_t id = 0;
  std::vector<mgcfd_level_view> levels;
  double mach = 0, aoa = 0;
  double* out = nullptr;  // level-0 variables [N0][5] on completion, may be NULL
  int64_t estimate = 0;
  double t_submit = 0, t_admit = -1, t_finish = -1;
  mgcfd_solver* solver = nullptr;
  int slot = -1;
  int cycles = 0;
  bool inflight = false;
  double rho_first = -1, rho_last = -1;
  int status = MGCFD_OK;
};

}  // namespace

struct mgcfd_server {
  mgcfd_server_options opt{};
  int device = 0;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request*> pending;
  std::vector<Request*> active;
  std::vector<mgcfd_request_result> done;
  bool stop = false;
  int64_t next_id = 1;
  int64_t used = 0;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  std::vector<int> slot_free;
  DevStatus* pinned = nullptr;  // one status block per slot
  Clock::time_point t0;
  mgcfd_server_stats stats{};
  std::string worker_error;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Device bytes a request may need at its peak (setup scratch included).
int64_t estimate_bytes(const std::vector<mgcfd_level_view>& lv, int precision, int increment) {
  int64_t b = 1 << 20;
  for (const auto& v : lv) {
    const int64_t n = v.nnodes, e = v.nedges, nb = v.nbnd;
    int64_t node = 8 * 8 + 5 * 8 * 3 + 8 * 3 + 4 * 4 + 32;   // rec, old/res/flux, vol constants, maps, dvec
    int64_t edge = 8 + 32;                                    // e2n, w4
    if (precision == MGCFD_PRECISION_MIXED) { node += 32; edge += 16; }
    if (increment == MGCFD_INCREMENT_GATHER || (increment == MGCFD_INCREMENT_AUTO && precision == MGCFD_PRECISION_MIXED))
      edge += 40 + 4;
    b += n * node + e * edge + nb * 96;
    b += n * 80 + e * 120 + nb * 64;                          // setup scratch (uploads, sort buffers)
  }
  return b;
}

void finish(mgcfd_server* S, Request* r) {
  if (r->solver) {
    if (r->out && r->status == MGCFD_OK) {
      int st = mgcfd_solver_fetch(r->solver, 0, MGCFD_Q_VARIABLES, r->out);
      if (st) r->status = st;
    }
    mgcfd_solver_destroy(r->solver);
    r->solver = nullptr;
  }
  r->t_finish = S->now();
  mgcfd_request_result res;
  std::memset(&res, 0, sizeof(res));
  res.id = r->id;
  res.status = r->status;
  res.cycles = r->cycles;
  res.submit_s = r->t_submit;
  res.admit_s = r->t_admit;
  res.finish_s = r->t_finish;
  res.rho_rms_first = r->rho_first;
  res.rho_rms_last = r->rho_last;
  std::lock_guard<std::mutex> lock(S->mu);
  if (r->slot >= 0) S->slot_free[(size_t)r->slot] = 1;
  S->used -= r->t_admit >= 0 ? r->estimate : 0;
  S->done.push_back(res);
  S->stats.completed++;
  if (r->status != MGCFD_OK) S->stats.failed++;
  S->cv.notify_all();
  delete r;
}

int enqueue_cycle(mgcfd_server* S, Request* r) {
  int st = mgcfd_solver_run(r->solver, 1);
  if (st) return st;
  const cudaStream_t s = S->streams[(size_t)r->slot];
  cudaError_t e = cudaMemcpyAsync(&S->pinned[r->slot], r->solver->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaEventRecord(S->events[(size_t)r->slot], s);
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("server: ") + cudaGetErrorString(e));
  r->inflight = true;
  return MGCFD_OK;
}

void worker_main(mgcfd_server* S) {
  cudaSetDevice(S->device);
  mgcfd_solver_options so;
  mgcfd_solver_default_options(&so);
  so.precision = S->opt.precision;
  so.increment = S->opt.increment;
  for (;;) {
    // Admission.
    for (;;) {
      Request* r = nullptr;
      {
        std::unique_lock<std::mutex> lock(S->mu);
        if (S->stop && S->pending.empty() && S->active.empty()) return;
        if (S->pending.empty()) {
          if (S->active.empty()) S->cv.wait_for(lock, std::chrono::milliseconds(2));
          break;
        }
        Request* f = S->pending.front();
        if (f->estimate > S->opt.hbm_budget_bytes) {  // can never fit
          S->pending.pop_front();
          f->status = MGCFD_ERR_BUDGET;
          lock.unlock();
          finish(S, f);
          continue;
        }
        int slot = -1;
        for (size_t k = 0; k < S->slot_free.size(); k++)
          if (S->slot_free[k]) { slot = (int)k; break; }
        if (slot < 0 || S->used + f->estimate > S->opt.hbm_budget_bytes) break;
        S->pending.pop_front();
        S->slot_free[(size_t)slot] = 0;
        S->used += f->estimate;
        S->stats.peak_bytes = std::max(S->stats.peak_bytes, S->used);
        f->slot = slot;
        f->t_admit = S->now();
        S->active.push_back(f);
        S->stats.peak_active = std::max<int64_t>(S->stats.peak_active, (int64_t)S->active.size());
        r = f;
      }
      int st = mgcfd_solver_create((int32_t)r->levels.size(), r->levels.data(), r->mach, r->aoa, &so,
                                   S->streams[(size_t)r->slot], &r->solver);
      if (st == MGCFD_OK) st = enqueue_cycle(S, r);
      if (st) {
        r->status = st;
        std::lock_guard<std::mutex> lock(S->mu);
        S->active.erase(std::find(S->active.begin(), S->active.end(), r));
      }
      if (st) finish(S, r);
    }
    // Progress.
    std::vector<Request*> act;
    {
      std::lock_guard<std::mutex> lock(S->mu);
      act = S->active;
    }
    bool progressed = false;
    for (Request* r : act) {
      if (!r->inflight) continue;
      cudaError_t q = cudaEventQuery(S->events[(size_t)r->slot]);
      if (q == cudaErrorNotReady) continue;
      progressed = true;
      r->inflight = false;
      r->cycles++;
      bool stop = false;
      if (q != cudaSuccess) {
        r->status = mgcfd::set_error(MGCFD_ERR_CUDA, std::string("server: ") + cudaGetErrorString(q));
        stop = true;
      } else {
        const DevStatus& h = S->pinned[r->slot];
        const double n0 = (double)r->levels[0].nnodes;
        const double rho = std::sqrt(h.rho_acc / n0);
        if (r->rho_first < 0) r->rho_first = rho;
        r->rho_last = rho;
        if (h.halt) {
          r->status = h.neg_dt ? MGCFD_ERR_NEGATIVE_DT : MGCFD_ERR_BAD_VALUES;
          stop = true;
        } else if (r->cycles >= S->opt.max_cycles ||
                   (S->opt.residual_drop > 0 && r->cycles > 1 && rho <= S->opt.residual_drop * r->rho_first)) {
          stop = true;
        }
      }
      if (!stop) {
        int st = enqueue_cycle(S, r);
        if (st) { r->status = st; stop = true; }
      }
      if (stop) {
        {
          std::lock_guard<std::mutex> lock(S->mu);
          S->active.erase(std::find(S->active.begin(), S->active.end(), r));
        }
        finish(S, r);
      }
    }
    if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

}  // namespace

extern "C" void mgcfd_server_default_options(mgcfd_server_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->hbm_budget_bytes = 150ll << 30;
  o->max_active = 16;
  o->precision = MGCFD_PRECISION_FP64;
  o->increment = MGCFD_INCREMENT_AUTO;
  o->max_cycles = 50;
  o->residual_drop = 1e-6;
}

extern "C" int mgcfd_server_create(const mgcfd_server_options* opt, mgcfd_server** out) {
  if (!out) return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_create: null output");
  *out = nullptr;
  std::unique_ptr<mgcfd_server> S(new (std::nothrow) mgcfd_server());
  if (!S) return mgcfd::set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  if (opt) S->opt = *opt; else mgcfd_server_default_options(&S->opt);
  if (S->opt.max_active < 1 || S->opt.max_active > 1024 || S->opt.max_cycles < 1 || S->opt.hbm_budget_bytes <= 0)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_create: bad options");
  CK(cudaGetDevice(&S->device));
  const int k = S->opt.max_active;
  S->streams.resize((size_t)k);
  S->events.resize((size_t)k);
  S->slot_free.assign((size_t)k, 1);
  for (int i = 0; i < k; i++) {
    CK(cudaStreamCreateWithFlags(&S->streams[(size_t)i], cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&S->events[(size_t)i], cudaEventDisableTiming));
  }
  CK(cudaMallocHost(reinterpret_cast<void**>(&S->pinned), sizeof(DevStatus) * (size_t)k));
  S->t0 = Clock::now();
  mgcfd_server* raw = S.get();
  S->worker = std::thread(worker_main, raw);
  *out = S.release();
  return MGCFD_OK;
}

extern "C" int mgcfd_server_submit(mgcfd_server* S, int32_t nlevels, const mgcfd_level_view* levels, double mach,
                                   double aoa_deg, double* out_variables_l0, int64_t* id) {
  if (!S || !levels || nlevels < 1 || nlevels > kMaxLevels)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_submit: bad arguments");
  Request* r = new (std::nothrow) Request();
  if (!r) return mgcfd::set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  r->levels.assign(levels, levels + nlevels);
  r->mach = mach;
  r->aoa = aoa_deg;
  r->out = out_variables_l0;
  r->estimate = estimate_bytes(r->levels, S->opt.precision, S->opt.increment);
  std::lock_guard<std::mutex> lock(S->mu);
  r->id = S->next_id++;
  r->t_submit = S->now();
  if (id) *id = r->id;
  S->pending.push_back(r);
  S->stats.submitted++;
  S->cv.notify_all();
  return MGCFD_OK;
}

extern "C" int mgcfd_request_estimate_bytes(int32_t nlevels, const mgcfd_level_view* levels, int32_t precision,
                                            int32_t increment, int64_t* bytes) {
  if (nlevels < 1 || !levels || !bytes) return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_request_estimate_bytes: bad arguments");
  *bytes = estimate_bytes(std::vector<mgcfd_level_view>(levels, levels + nlevels), precision, increment);
  return MGCFD_OK;
}

extern "C" int mgcfd_server_poll(mgcfd_server* S, mgcfd_request_result* out, int32_t capacity, int32_t* count) {
  if (!S || !count || (capacity > 0 && !out)) return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_poll: bad arguments");
  std::lock_guard<std::mutex> lock(S->mu);
  int32_t n = (int32_t)std::min<size_t>((size_t)std::max(capacity, 0), S->done.size());
  for (int32_t i = 0; i < n; i++) out[i] = S->done[(size_t)i];
  S->done.erase(S->done.begin(), S->done.begin() + n);
  *count = n;
  return MGCFD_OK;
}

extern "C" int mgcfd_server_drain(mgcfd_server* S, double timeout_s) {
  if (!S) return mgcfd::set_error(MGCFD_ERR_INVALID, "null server");
  std::unique_lock<std::mutex> lock(S->mu);
  const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s);
  while (!(S->pending.empty() && S->active.empty())) {
    if (S->cv.wait_until(lock, deadline) == std::cv_status::timeout && Clock::now() >= deadline)
      return mgcfd::set_error(MGCFD_ERR_TIMEOUT, "mgcfd_server_drain: requests still running");
  }
  return MGCFD_OK;
}

extern "C" int mgcfd_server_get_stats(mgcfd_server* S, mgcfd_server_stats* out) {
  if (!S || !out) return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_get_stats: null argument");
  std::lock_guard<std::mutex> lock(S->mu);
  *out = S->stats;
  out->used_bytes = S->used;
  out->active = (int64_t)S->active.size();
  out->pending = (int64_t)S->pending.size();
  return MGCFD_OK;
}

extern "C" void mgcfd_server_destroy(mgcfd_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  for (auto st : S->streams) cudaStreamDestroy(st);
  for (auto ev : S->events) cudaEventDestroy(ev);
  if (S->pinned) cudaFreeHost(S->pinned);
  delete S;
}
