// Serving loop: flow solves of different meshes and freestream conditions
// arrive at any time and run concurrently on one GPU.
//
// Two host threads share the work:
//   * the host-work thread admits requests and retires them.  Requests wait
//     in a FIFO until a slot (a CUDA stream) is free and the HBM budget covers
//     their estimated footprint; admission builds the request's device solver
//     on its slot's stream (upload, device setup), installs the device-side
//     stop rule and enqueues the first V-cycles.  Retirement copies the final
//     level-0 state out, frees the solver and releases slot and budget.
//   * the progress thread keeps every active job's stream fed (a job is one
//     request's solver, or a cohort's batched solver).  Cycles are enqueued in
//     chunks of kChunk V-cycles (CUDA graph launches), each followed by an
//     asynchronous copy of the solver's status (per mesh for a cohort) to
//     pinned memory and an event; up to kDepth chunks are in flight per job,
//     so the stream never waits for the host between chunks.
// The stop rule runs on the device at the end of every V-cycle (k_cycle_end):
// it counts cycles, records the level-0 density residual norm and, once the
// norm has dropped to residual_drop times the first cycle's or max_cycles is
// reached, stops the solver's kernels, so cycles enqueued beyond that point
// do no work and the solve ends exactly where a host-driven loop would have
// stopped it.  min_dt < 0 and NaN/Inf stop it the same way with an error.
//
// Meshes stay resident: a request submitted with a nonzero mesh key leaves its
// solver (mesh tables and state buffers) in an idle cache when it retires,
// charged to the budget, and the next request with that key reuses it after
// re-initialising state and far-field terms for its own freestream
// (solver_retarget): no upload and no setup.  Idle solvers are evicted, least
// recently used first, when a new mesh needs their budget.
//
// Cohorts: with batch_max_meshes > 1, small requests (at most batch_max_nodes
// level-0 nodes) that wait next to each other at the front of the queue with
// the same number of levels are admitted together into one slot as one
// batched solver (mgcfd_batch_create): every V-cycle stage is one launch over
// all of their meshes, which matters for meshes too small to fill the GPU on
// their own.  The batched solver carries the stop rule per mesh
// (k_cycle_end_seg): a request that meets it, or fails, stops changing while
// the others go on, and its cycle count and residual norms are its own.  The
// cohort retires when its last request has stopped; each request's record and
// level-0 state are then published.
//
// Requests therefore join and leave at V-cycle boundaries and their kernels
// overlap on the device (continuous batching at V-cycle granularity).  Each
// request's arithmetic is exactly that of a solver running alone -- batched
// kernels included -- so with a deterministic increment (gather or the fused
// stage) a result is bit-identical alone, in the mix and in a cohort.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "common.h"
#include "solver_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kChunk = 4;       // V-cycles per enqueued chunk
constexpr int kDepth = 2;       // chunks in flight per job
constexpr int kMaxCohort = 64;  // requests per cohort at most

struct Request {
  int64_t id = 0;
  int64_t key = 0;        // mesh key (0: no reuse)
  std::vector<mgcfd_level_view> levels;
  double mach = 0, aoa = 0;
  double* out = nullptr;  // level-0 variables [N0][5] on completion, may be NULL
  int64_t estimate = 0;
  double t_submit = 0, t_admit = -1, t_finish = -1;
  int cycles = 0;
  double rho_first = -1, rho_last = -1;
  int status = MGCFD_OK;
};

// What one slot runs: one request's own solver, or a cohort of requests in
// one batched solver (request m is the batch's mesh m).
struct Job {
  std::vector<Request*> reqs;
  mgcfd_solver* solver = nullptr;
  bool cohort = false;
  int slot = -1;
  int64_t charged = 0;   // budget charged for this job (0: never admitted)
  int enqueued = 0;      // V-cycles enqueued so far
  int inflight = 0;      // chunks not yet seen complete
  int next_buf = 0;      // status buffer of the next chunk
  int oldest_buf = 0;    // status buffer of the oldest chunk in flight
  bool ending = false;   // no more chunks: waiting for the ones in flight
  int status = MGCFD_OK; // failure of the job itself (set-up, CUDA)
  // GPU timestamps: recorded before the first chunk, and again after every
  // chunk, so at retirement ev_end holds the end of the last one.
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
};

// Copied to page-locked memory after every chunk: the solver's status block
// and, for a cohort, every mesh's stop rule and failure flags.
struct ChunkStatus {
  DevStatus st;
  SegStop seg[kMaxCohort];
  int neg[kMaxCohort];
  int bad[kMaxCohort];
};

}  // namespace

struct mgcfd_server {
  mgcfd_server_options opt{};
  int device = 0;
  std::thread host_worker, progress_worker;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Request*> pending;
  std::vector<Job*> active;
  std::deque<Job*> retiring;
  std::vector<mgcfd_request_result> done;
  struct Idle {
    int64_t key;
    mgcfd_solver* solver;
    int64_t estimate;
  };
  std::list<Idle> idle_cache;  // front = most recently used
  bool stop = false;
  int admitting = 0;     // jobs between pending and active
  int retiring_now = 0;  // jobs taken for retirement whose records are not yet published
  int64_t active_requests = 0;
  int64_t next_id = 1;
  int64_t used = 0;
  std::vector<cudaEvent_t> events;  // [slot][kDepth]
  std::vector<int> slot_free;
  ChunkStatus* pinned = nullptr;    // [slot][kDepth]
  cudaEvent_t t0_ev = nullptr;      // GPU time zero of the device timestamps
  Clock::time_point t0;
  mgcfd_server_stats stats{};

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  bool idle() const {
    return pending.empty() && active.empty() && retiring.empty() && admitting == 0 && retiring_now == 0;
  }
  bool batchable(const Request* r) const {
    return opt.batch_max_meshes > 1 && r->levels[0].nnodes <= opt.batch_max_nodes;
  }
};

namespace {

// Device bytes a request may need at its peak (setup scratch included).
int64_t estimate_bytes(const std::vector<mgcfd_level_view>& lv, int precision, int increment) {
  const bool mixed = precision == MGCFD_PRECISION_MIXED, dw = precision == MGCFD_PRECISION_DW;
  const bool fused = increment == MGCFD_INCREMENT_FUSED || (increment == MGCFD_INCREMENT_AUTO && (mixed || dw));
  const bool gather = fused || increment == MGCFD_INCREMENT_GATHER;
  int64_t b = 1 << 20;
  for (const auto& v : lv) {
    const int64_t n = v.nnodes, e = v.nedges, nb = v.nbnd;
    int64_t node = 8 * 8 + 5 * 8 * 3 + 8 * 3 + 4 * 4 + 32;   // rec, old/res/flux, vol constants, maps, dvec
    int64_t edge = 8 + 32;                                    // e2n, w4
    if (mixed) { node += fused ? 64 : 32; edge += 16; }
    if (dw) {  // rec2, w4dw; fused: rec2b, off2, ent2
      node += 64 + (fused ? 68 : 0);
      edge += 32 + (fused ? 16 : 0);
    }
    if (fused) edge += 4 + 4 + 16;                 // b_list, b_nbr, b_w4f
    else if (gather) edge += (mixed ? 20 : 40) + 4;  // per-edge fluxes, b_list
    b += n * node + e * edge + nb * 96;
    b += n * 80 + e * 120 + nb * 64;                          // setup scratch (uploads, sort buffers)
  }
  return b;
}

// Host-work thread: copy the results out, free or cache the solver, publish
// one record per request.
void retire(mgcfd_server* S, Job* job) {
  bool cached = false;
  if (job->solver) {
    if (job->status == MGCFD_OK) {
      for (size_t m = 0; m < job->reqs.size(); m++) {
        Request* r = job->reqs[m];
        if (!r->out || r->status != MGCFD_OK) continue;
        const int st = job->cohort ? mgcfd_solver_fetch_mesh(job->solver, (int32_t)m, 0, MGCFD_Q_VARIABLES, r->out)
                                   : mgcfd_solver_fetch(job->solver, 0, MGCFD_Q_VARIABLES, r->out);
        if (st) r->status = st;
      }
    }
    Request* r0 = job->reqs[0];
    if (!job->cohort && r0->key != 0 && job->status == MGCFD_OK && r0->status == MGCFD_OK) {
      std::lock_guard<std::mutex> lock(S->mu);
      S->idle_cache.push_front({r0->key, job->solver, job->charged});
      cached = true;
    } else {
      mgcfd_solver_destroy(job->solver);
    }
    job->solver = nullptr;
  }
  double dev_begin = -1.0, dev_end = -1.0;
  if (job->ev_begin && job->ev_end) {  // the stream is idle: every chunk has completed
    float b = 0.f, e = 0.f;
    if (cudaEventElapsedTime(&b, S->t0_ev, job->ev_begin) == cudaSuccess &&
        cudaEventElapsedTime(&e, S->t0_ev, job->ev_end) == cudaSuccess) {
      dev_begin = 1e-3 * b;
      dev_end = 1e-3 * e;
    }
    cudaGetLastError();
  }
  if (job->ev_begin) cudaEventDestroy(job->ev_begin);
  if (job->ev_end) cudaEventDestroy(job->ev_end);
  const double t = S->now();
  std::lock_guard<std::mutex> lock(S->mu);
  for (Request* r : job->reqs) {
    if (job->status != MGCFD_OK && r->status == MGCFD_OK) r->status = job->status;
    r->t_finish = t;
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
    res.device_begin_s = dev_begin;
    res.device_end_s = dev_end;
    S->done.push_back(res);
    S->stats.completed++;
    if (r->status != MGCFD_OK) S->stats.failed++;
    delete r;
  }
  if (job->slot >= 0) {
    S->slot_free[(size_t)job->slot] = 1;
    S->active_requests -= (int64_t)job->reqs.size();
  }
  if (!cached) S->used -= job->charged;
  S->retiring_now--;
  S->cv.notify_all();
  delete job;
}

// Enqueue the next chunk of V-cycles, then the status copies and their event.
int enqueue_chunk(mgcfd_server* S, Job* job) {
  const int n = std::min(kChunk, S->opt.max_cycles - job->enqueued);
  mgcfd_solver* sv = job->solver;
  const cudaStream_t s = sv->stream;
  cudaError_t e = cudaSuccess;
  if (!job->ev_begin) {
    e = cudaEventCreate(&job->ev_begin);
    if (e == cudaSuccess) e = cudaEventCreate(&job->ev_end);
    if (e == cudaSuccess) e = cudaEventRecord(job->ev_begin, s);
    if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("server: ") + cudaGetErrorString(e));
  }
  int st = mgcfd_solver_run(sv, n);
  if (st) return st;
  job->enqueued += n;
  const size_t k = (size_t)job->slot * kDepth + (size_t)job->next_buf;
  ChunkStatus* c = &S->pinned[k];
  e = cudaEventRecord(job->ev_end, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&c->st, sv->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  if (job->cohort) {
    const size_t m = job->reqs.size();
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->seg, sv->seg_stop, sizeof(SegStop) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->neg, sv->seg_neg, sizeof(int) * m, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->bad, sv->seg_bad, sizeof(int) * m, cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaEventRecord(S->events[k], s);
  if (e != cudaSuccess) return mgcfd::set_error(MGCFD_ERR_CUDA, std::string("server: ") + cudaGetErrorString(e));
  job->next_buf = (job->next_buf + 1) % kDepth;
  job->inflight++;
  return MGCFD_OK;
}

// Builds the job's solver: a cached solver retargeted, a new solver, or one
// batched solver for a cohort; every one with the server's stop rule.
int start_job(mgcfd_server* S, Job* job, mgcfd_solver* reuse, const mgcfd_solver_options& so) {
  Request* r0 = job->reqs[0];
  int st;
  if (reuse) {
    job->solver = reuse;
    return mgcfd::solver_retarget(reuse, r0->mach, r0->aoa);
  }
  if (job->cohort) {
    const size_t m = job->reqs.size();
    std::vector<const mgcfd_level_view*> lv(m);
    std::vector<double> mach(m), aoa(m);
    for (size_t i = 0; i < m; i++) {
      lv[i] = job->reqs[i]->levels.data();
      mach[i] = job->reqs[i]->mach;
      aoa[i] = job->reqs[i]->aoa;
    }
    st = mgcfd_batch_create((int32_t)m, (int32_t)r0->levels.size(), lv.data(), mach.data(), aoa.data(), &so, nullptr,
                            &job->solver);
  } else {
    st = mgcfd_solver_create((int32_t)r0->levels.size(), r0->levels.data(), r0->mach, r0->aoa, &so, nullptr,
                             &job->solver);
  }
  if (st == MGCFD_OK) st = mgcfd::solver_set_stop_rule(job->solver, S->opt.max_cycles, S->opt.residual_drop);
  (void)S;
  return st;
}

// Host-work thread: admission and retirement.
void host_main(mgcfd_server* S) {
  cudaSetDevice(S->device);
  mgcfd_solver_options so;
  mgcfd_solver_default_options(&so);
  so.precision = S->opt.precision;
  so.increment = S->opt.increment;
  so.accumulation = S->opt.accumulation;
  for (;;) {
    Job* job = nullptr;
    bool admit = false;
    mgcfd_solver* reuse = nullptr;        // an idle solver of this request's mesh
    std::vector<mgcfd_solver*> victims;  // idle solvers evicted to make room
    {
      std::unique_lock<std::mutex> lock(S->mu);
      for (;;) {
        if (!S->retiring.empty()) {
          job = S->retiring.front();
          S->retiring.pop_front();
          S->retiring_now++;
          break;
        }
        if (!S->pending.empty()) {
          Request* f = S->pending.front();
          if (f->estimate > S->opt.hbm_budget_bytes) {  // can never fit
            S->pending.pop_front();
            f->status = MGCFD_ERR_BUDGET;
            job = new Job();
            job->reqs.push_back(f);
            S->retiring_now++;
            break;
          }
          int slot = -1;
          for (size_t k = 0; k < S->slot_free.size(); k++)
            if (S->slot_free[k]) { slot = (int)k; break; }
          if (slot >= 0) {
            // A cohort: the run of batchable requests at the front of the
            // queue with the first one's number of levels.
            std::vector<Request*> co;
            int64_t co_bytes = 0;
            if (S->batchable(f)) {
              for (Request* r : S->pending) {
                if ((int)co.size() >= std::min(S->opt.batch_max_meshes, kMaxCohort) || !S->batchable(r) ||
                    r->levels.size() != f->levels.size())
                  break;
                co.push_back(r);
                co_bytes += r->estimate;
              }
            }
            if (co.size() >= 2) {
              while (S->used + co_bytes > S->opt.hbm_budget_bytes && !S->idle_cache.empty()) {
                victims.push_back(S->idle_cache.back().solver);
                S->used -= S->idle_cache.back().estimate;
                S->idle_cache.pop_back();
              }
              while (co.size() > 1 && S->used + co_bytes > S->opt.hbm_budget_bytes) {
                co_bytes -= co.back()->estimate;
                co.pop_back();
              }
            }
            if (co.size() >= 2) {
              job = new Job();
              job->cohort = true;
              job->reqs = co;
              job->charged = co_bytes;
              S->used += co_bytes;
              for (size_t k = 0; k < co.size(); k++) S->pending.pop_front();
              S->stats.cohorts++;
              S->stats.cohort_requests += (int64_t)co.size();
              admit = true;
            } else {
              auto hit = S->idle_cache.end();
              if (f->key != 0)
                for (auto it = S->idle_cache.begin(); it != S->idle_cache.end(); ++it)
                  if (it->key == f->key) { hit = it; break; }
              bool fits = hit != S->idle_cache.end();
              int64_t charged = f->estimate;
              if (fits) {  // already charged to the budget
                reuse = hit->solver;
                charged = hit->estimate;
                S->idle_cache.erase(hit);
                S->stats.cache_hits++;
              } else {
                // Evict least recently used idle solvers until the new mesh fits.
                while (S->used + f->estimate > S->opt.hbm_budget_bytes && !S->idle_cache.empty()) {
                  victims.push_back(S->idle_cache.back().solver);
                  S->used -= S->idle_cache.back().estimate;
                  S->idle_cache.pop_back();
                }
                fits = S->used + f->estimate <= S->opt.hbm_budget_bytes;
                if (fits) S->used += f->estimate;
              }
              if (fits) {
                S->pending.pop_front();
                job = new Job();
                job->reqs.push_back(f);
                job->charged = charged;
                admit = true;
              }
            }
            if (admit) {
              S->slot_free[(size_t)slot] = 0;
              S->stats.peak_bytes = std::max(S->stats.peak_bytes, S->used);
              job->slot = slot;
              const double t = S->now();
              for (Request* r : job->reqs) r->t_admit = t;
              S->active_requests += (int64_t)job->reqs.size();
              S->stats.peak_active = std::max(S->stats.peak_active, S->active_requests);
              S->admitting++;
              break;
            }
          }
        }
        if (!victims.empty()) break;  // free them, then look again
        if (S->stop && S->idle()) {
          for (auto& c : S->idle_cache) mgcfd_solver_destroy(c.solver);
          S->idle_cache.clear();
          return;
        }
        S->cv.wait(lock);
      }
    }
    for (mgcfd_solver* v : victims) mgcfd_solver_destroy(v);
    if (!job) continue;
    if (!admit) {
      retire(S, job);
      continue;
    }
    int st = start_job(S, job, reuse, so);
    for (int c = 0; st == MGCFD_OK && c < kDepth && job->enqueued < S->opt.max_cycles; c++) st = enqueue_chunk(S, job);
    {
      std::lock_guard<std::mutex> lock(S->mu);
      S->admitting--;
      if (st == MGCFD_OK) {
        S->active.push_back(job);
        S->cv.notify_all();
        continue;
      }
      S->retiring_now++;
    }
    if (job->solver) cudaStreamSynchronize(job->solver->stream);
    job->status = st;
    retire(S, job);
  }
}

// Reads one completed chunk's status into the job's requests; true when
// every request of the job has stopped.
bool read_chunk(Job* job, const ChunkStatus& c) {
  if (!job->cohort) {
    Request* r = job->reqs[0];
    const DevStatus& h = c.st;
    r->cycles = h.cycles_done;
    if (h.cycles_done > 0) { r->rho_first = h.rho_first; r->rho_last = h.rho_last; }
    if (h.halt && !h.stopped && r->status == MGCFD_OK) r->status = h.neg_dt ? MGCFD_ERR_NEGATIVE_DT : MGCFD_ERR_BAD_VALUES;
    return h.halt != 0;
  }
  bool all = true;
  for (size_t m = 0; m < job->reqs.size(); m++) {
    Request* r = job->reqs[m];
    const SegStop& g = c.seg[m];
    r->cycles = g.cycles_done;
    if (g.cycles_done > 0) { r->rho_first = g.rho_first; r->rho_last = g.rho_last; }
    if (r->status == MGCFD_OK && (c.neg[m] || c.bad[m]))
      r->status = c.neg[m] ? MGCFD_ERR_NEGATIVE_DT : MGCFD_ERR_BAD_VALUES;
    all = all && g.halt != 0;
  }
  return all;
}

// Progress thread: completes chunks and enqueues the next ones.
void progress_main(mgcfd_server* S) {
  cudaSetDevice(S->device);
  std::vector<Job*> act;
  for (;;) {
    {
      std::unique_lock<std::mutex> lock(S->mu);
      if (S->active.empty()) {
        if (S->stop && S->idle()) return;
        S->cv.wait_for(lock, std::chrono::milliseconds(2));
        continue;
      }
      act = S->active;
    }
    bool progressed = false;
    for (Job* job : act) {
      const size_t k = (size_t)job->slot * kDepth + (size_t)job->oldest_buf;
      const cudaError_t q = cudaEventQuery(S->events[k]);
      if (q == cudaErrorNotReady) continue;
      progressed = true;
      job->inflight--;
      job->oldest_buf = (job->oldest_buf + 1) % kDepth;
      if (q != cudaSuccess) {
        job->status = mgcfd::set_error(MGCFD_ERR_CUDA, std::string("server: ") + cudaGetErrorString(q));
        job->ending = true;
      } else if (read_chunk(job, S->pinned[k])) {
        job->ending = true;
      }
      if (!job->ending && job->enqueued < S->opt.max_cycles) {
        const int st = enqueue_chunk(S, job);
        if (st) { job->status = st; job->ending = true; }
      }
      if (job->inflight == 0) {  // nothing left on the device for this job
        std::lock_guard<std::mutex> lock(S->mu);
        S->active.erase(std::find(S->active.begin(), S->active.end(), job));
        S->retiring.push_back(job);
        S->cv.notify_all();
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
  if (S->opt.max_active < 1 || S->opt.max_active > 1024 || S->opt.max_cycles < 1 || S->opt.hbm_budget_bytes <= 0 ||
      S->opt.precision < MGCFD_PRECISION_FP64 || S->opt.precision > MGCFD_PRECISION_DW ||
      S->opt.batch_max_meshes < 0 || S->opt.batch_max_meshes > kMaxCohort || S->opt.batch_max_nodes < 0)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_create: bad options");
  CK(cudaGetDevice(&S->device));
  const int k = S->opt.max_active;
  S->events.resize((size_t)k * kDepth);
  S->slot_free.assign((size_t)k, 1);
  for (auto& ev : S->events) CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  CK(cudaEventCreate(&S->t0_ev));
  CK(cudaEventRecord(S->t0_ev, nullptr));
  CK(cudaEventSynchronize(S->t0_ev));
  CK(cudaMallocHost(reinterpret_cast<void**>(&S->pinned), sizeof(ChunkStatus) * (size_t)k * kDepth));
  S->t0 = Clock::now();
  mgcfd_server* raw = S.get();
  S->host_worker = std::thread(host_main, raw);
  S->progress_worker = std::thread(progress_main, raw);
  *out = S.release();
  return MGCFD_OK;
}

extern "C" int mgcfd_server_submit(mgcfd_server* S, int32_t nlevels, const mgcfd_level_view* levels, double mach,
                                   double aoa_deg, int64_t mesh_key, double* out_variables_l0, int64_t* id) {
  if (!S || !levels || nlevels < 1 || nlevels > kMaxLevels)
    return mgcfd::set_error(MGCFD_ERR_INVALID, "mgcfd_server_submit: bad arguments");
  Request* r = new (std::nothrow) Request();
  if (!r) return mgcfd::set_error(MGCFD_ERR_NOMEM, "host allocation failed");
  r->levels.assign(levels, levels + nlevels);
  r->mach = mach;
  r->aoa = aoa_deg;
  r->out = out_variables_l0;
  r->key = mesh_key;
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
  while (!S->idle()) {
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
  out->active = S->active_requests;
  out->pending = (int64_t)S->pending.size();
  out->cached_solvers = (int64_t)S->idle_cache.size();
  return MGCFD_OK;
}

extern "C" void mgcfd_server_destroy(mgcfd_server* S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lock(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->host_worker.joinable()) S->host_worker.join();
  if (S->progress_worker.joinable()) S->progress_worker.join();
  for (auto ev : S->events) cudaEventDestroy(ev);
  if (S->t0_ev) cudaEventDestroy(S->t0_ev);
  if (S->pinned) cudaFreeHost(S->pinned);
  delete S;
}
