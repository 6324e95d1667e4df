// afar_server_*: a queue of solve requests served on one GPU under a device-memory budget.
//
// One worker thread owns every solver and the batch, so all CUDA work of a server stays on one
// host thread (the solvers' threading rule); submit, wait and stats only touch the queue under a
// mutex.  Each round the worker admits queued requests in arrival order while the estimated device
// memory of the running solves plus the next one fits the budget (the first always runs), steps
// the batch by one chunk, and retires the solves that reached their end time or step count.
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "afar_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  afar_request req;
  long long id;
  Clock::time_point t_submit;
  Clock::time_point t_done;
  int status = AFAR_OK;
  std::string message;
  bool done = false;
  afar_solver* solver = nullptr;
  size_t bytes = 0;
  long long steps0 = 0;
  long long steps_done = 0;
  bool cancel = false;  // set by afar_server_cancel while running: retired at the next chunk boundary
};

// Device memory of a solve before it is built: a per-cell, per-face model of the allocations
// (state, intermediates, slot-major operator rows, the state snapshot, the residual dump and, for
// mixed, the transfer staging), by policy.  The worker also scales it by the largest ratio of
// built to estimated bytes seen so far, so admission never trusts a model that fell short.
size_t estimate_bytes(const afar_fieldSizes& z, int policy) {
  const double nc = z.cellsNum, nf = z.facesNum, nb = z.totalBoundaryFacesNum;
  const double s = z.maxStencilSize, m = z.maxCompactStencilSize;
  const double w = policy == AFAR_POLICY_FP64 ? 8.0 : 4.0;  // operator word
  const double g = policy == AFAR_POLICY_MIXED ? 4.0 : 8.0; // state / intermediate word
  const double snapshot = 4 * g + 64, res_dump = 32, staging = policy == AFAR_POLICY_MIXED ? 32 : 0;
  const double per_cell = 4 * g + 64 + 8 * g + 4 * w + 2 + 4 * s + 4 * m + 8 * m * w + 2 * m * w + m * (s + 1) * w + 48 +
                          snapshot + res_dump + staging;
  const double per_face = 8 * g + 4 * g + 48 + 16 + 8;
  return (size_t)(nc * per_cell + (nf + nb) * per_face + nb * 48 + (64u << 20));
}

}  // namespace

struct afar_server {
  int policy = AFAR_POLICY_MIXED;
  int device = 0;
  size_t budget = 0;
  double est_scale = 1.0;  // largest built / estimated bytes so far (worker thread only)
  int chunk = 50;
  afar_batch* batch = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::vector<Request*> running;
  std::map<long long, Request*> all;
  long long next_id = 1;
  bool stop = false;
  afar_server_stats st{};
  std::thread worker;

  void fail(Request* r, int status, const char* what) {
    r->status = status;
    r->message = std::string(what) + ": " + afar_last_error();
  }

  // Builds the request's solver (worker thread).  Returns false (request failed) on error.
  bool build(Request* r) {
    const afar_request& q = r->req;
    const afar_fieldSizes& z = q.sizes;
    afar_solver* s = nullptr;
    int e;
    if ((e = afar_solver_create(&s, policy, device))) return fail(r, e, "solver"), false;
    r->solver = s;
    if ((e = afar_setDeviceFieldData(s, q.host, z.cellsNum, z.facesNum, z.totalBoundaryFacesNum)))
      return fail(r, e, "upload"), false;
    if (policy == AFAR_POLICY_FP64 && q.RBFbasis64 && (e = afar_set_rbf_basis64(s, q.RBFbasis64, q.RBFbasis64Count)))
      return fail(r, e, "FP64 weights"), false;
    if ((e = afar_setDeviceFieldDataStencil(s, q.host, z.cellsNum, z.facesNum, z.patchesNum, z.totalBoundaryFacesNum,
                                            z.maxStencilSize, z.maxCompactStencilSize, z.maxLocalBlockStencilSize,
                                            z.maxCompactLocalBlockStencilSize)))
      return fail(r, e, "stencil upload"), false;
    if ((e = afar_set_gas(s, q.R, q.Cv))) return fail(r, e, "gas"), false;
    if ((e = afar_set_step_params(s, 0.0, q.CFL, q.tEnd > 0.0 ? q.tEnd : 0.0))) return fail(r, e, "step"), false;
    if ((e = afar_device_bytes(s, &r->bytes))) return fail(r, e, "bytes"), false;
    double t, dt;
    if ((e = afar_get_time(s, &t, &dt, &r->steps0))) return fail(r, e, "time"), false;
    if ((e = afar_batch_add(batch, s))) return fail(r, e, "batch"), false;
    return true;
  }

  void release(Request* r) {
    if (r->solver) {
      afar_freeFieldData(r->solver);  // also leaves the batch
      r->solver = nullptr;
    }
  }

  void finish(Request* r) {
    std::lock_guard<std::mutex> lock(mu);
    finish_locked(r);
  }
  void finish_locked(Request* r) {
    r->done = true;
    r->t_done = Clock::now();
    if (r->status == AFAR_OK) st.completed++;
    else st.failed++;
    if (r->status == AFAR_ERR_CANCELLED) st.cancelled++;
    cv_done.notify_all();
  }

  void loop() {
    for (;;) {
      std::vector<Request*> admit;
      {
        std::unique_lock<std::mutex> lock(mu);
        cv_work.wait(lock, [&] { return stop || !queue.empty() || !running.empty(); });
        if (stop && queue.empty() && running.empty()) return;
        size_t used = st.bytesInUse;
        while (!queue.empty()) {
          Request* r = queue.front();
          const size_t est = (size_t)(est_scale * (double)estimate_bytes(r->req.sizes, policy));
          if (!(running.empty() && admit.empty()) && used + est > budget) break;
          queue.pop_front();
          used += est;
          admit.push_back(r);
        }
      }
      for (Request* r : admit) {
        if (build(r)) {
          const double est = (double)estimate_bytes(r->req.sizes, policy);
          if (est > 0.0 && (double)r->bytes > est_scale * est) est_scale = (double)r->bytes / est;
          std::lock_guard<std::mutex> lock(mu);
          running.push_back(r);
          st.bytesInUse += r->bytes;
          if (st.bytesInUse > st.peakBytes) st.peakBytes = st.bytesInUse;
          if ((long long)running.size() > st.peakRunning) st.peakRunning = (long long)running.size();
        } else {
          release(r);
          finish(r);
        }
      }
      std::vector<Request*> run;
      {
        std::lock_guard<std::mutex> lock(mu);
        run = running;
      }
      if (run.empty()) continue;
      int n = chunk;
      for (Request* r : run) {
        if (r->req.nSteps <= 0) continue;
        long long steps;
        double t, dt;
        afar_get_time(r->solver, &t, &dt, &steps);
        const long long left = r->steps0 + r->req.nSteps - steps;
        if (left > 0 && left < n) n = (int)left;
      }
      float ms = 0.f;
      int e = afar_batch_run(batch, n, &ms);
      {
        std::lock_guard<std::mutex> lock(mu);
        st.batchSteps += n;
      }
      std::vector<Request*> keep;
      for (Request* r : run) {
        double t = 0.0, dt = 0.0;
        long long steps = 0;
        bool fin = false;
        bool cancelled;
        {
          std::lock_guard<std::mutex> lock(mu);
          cancelled = r->cancel;
        }
        if (cancelled) {
          r->status = AFAR_ERR_CANCELLED;
          r->message = "the request was cancelled";
          fin = true;
        } else if (e) {
          fail(r, e, "batch run");
          fin = true;
        } else if ((e = afar_get_time(r->solver, &t, &dt, &steps))) {
          fail(r, e, "time");
          fin = true;
        } else {
          const bool by_steps = r->req.nSteps > 0 && steps - r->steps0 >= r->req.nSteps;
          const bool by_time = r->req.tEnd > 0.0 && t >= r->req.tEnd * (1.0 - 1e-12);
          fin = by_steps || by_time;
          if (!fin && steps - r->steps0 == 0 && !(dt > 0.0) && n > 0) {  // no progress: a broken state
            r->status = AFAR_ERR_NOT_FINITE;
            r->message = "the solve stopped advancing (non-finite or non-positive step)";
            fin = true;
          }
        }
        if (fin) {
          r->steps_done = steps - r->steps0;
          if (r->status == AFAR_OK &&
              (e = afar_download_state(r->solver, r->req.outFD, nullptr, r->req.outShockIndicator)))
            fail(r, e, "download");
          if (r->status == AFAR_OK) {  // a state that broke down still advanced: report it
            const size_t n = 4 * (size_t)(r->req.sizes.cellsNum + r->req.sizes.totalBoundaryFacesNum);
            const double* v = reinterpret_cast<const double*>(r->req.outFD);
            for (size_t i = 0; i < n; ++i)
              if (!std::isfinite(v[i])) {
                r->status = AFAR_ERR_NOT_FINITE;
                r->message = "the solve's state is not finite";
                break;
              }
          }
          {
            std::lock_guard<std::mutex> lock(mu);
            st.bytesInUse -= r->bytes;
          }
          release(r);
          finish(r);
        } else {
          keep.push_back(r);
        }
        e = AFAR_OK;
      }
      std::lock_guard<std::mutex> lock(mu);
      running = keep;
    }
  }
};

extern "C" afar_status afar_server_create(afar_server** out, int policy, int device, size_t budget, int chunkSteps) {
  using afar::set_error;
  if (!out || (policy != AFAR_POLICY_MIXED && policy != AFAR_POLICY_FP64) || chunkSteps < 1) {
    set_error("afar_server_create: null output, policy other than fp64/mixed, or chunkSteps < 1");
    return AFAR_ERR_ARGUMENT;
  }
  *out = nullptr;
  afar_server* s = new afar_server();
  s->policy = policy;
  s->device = device;
  s->budget = budget;
  s->chunk = chunkSteps;
  s->st.budgetBytes = budget;
  afar_status e = afar_batch_create(&s->batch, policy, device);
  if (e) {
    delete s;
    return e;
  }
  s->worker = std::thread([s] { s->loop(); });
  *out = s;
  return AFAR_OK;
}

extern "C" afar_status afar_server_submit(afar_server* s, const afar_request* q, long long* id) {
  using afar::set_error;
  if (!s || !q || !id || !q->host || !q->outFD || !(q->R > 0.0) || !(q->Cv > 0.0) || !(q->CFL > 0.0) ||
      (!(q->tEnd > 0.0) && q->nSteps <= 0) || q->sizes.cellsNum <= 0) {
    set_error("afar_server_submit: null argument, non-positive R/Cv/CFL, no end (tEnd or nSteps) or no cells");
    return AFAR_ERR_ARGUMENT;
  }
  Request* r = new Request();
  r->req = *q;
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) {
      delete r;
      set_error("afar_server_submit: the server is shutting down");
      return AFAR_ERR_STATE;
    }
    r->id = s->next_id++;
    s->all[r->id] = r;
    s->queue.push_back(r);
    s->st.submitted++;
  }
  s->cv_work.notify_one();
  *id = r->id;
  return AFAR_OK;
}

extern "C" afar_status afar_server_wait(afar_server* s, long long id, double timeout, int* done, int* status,
                                        double* latency_ms, long long* steps) {
  using afar::set_error;
  if (!s || !done) return (set_error("afar_server_wait: null argument"), AFAR_ERR_ARGUMENT);
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return (set_error("afar_server_wait: unknown request id"), AFAR_ERR_ARGUMENT);
  Request* r = it->second;
  auto ready = [&] { return r->done; };
  if (timeout < 0.0)
    s->cv_done.wait(lock, ready);
  else
    s->cv_done.wait_for(lock, std::chrono::duration<double>(timeout), ready);
  *done = r->done ? 1 : 0;
  if (r->done) {
    if (status) *status = r->status;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (steps) *steps = r->steps_done;
    if (r->status != AFAR_OK) set_error("%s", r->message.c_str());
  }
  return AFAR_OK;
}

extern "C" afar_status afar_server_cancel(afar_server* s, long long id) {
  using afar::set_error;
  if (!s) return (set_error("afar_server_cancel: null server"), AFAR_ERR_ARGUMENT);
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return (set_error("afar_server_cancel: unknown request id"), AFAR_ERR_ARGUMENT);
  Request* r = it->second;
  if (r->done) return (set_error("afar_server_cancel: the request has finished"), AFAR_ERR_STATE);
  for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
    if (*q == r) {  // not admitted yet: it never touches the GPU
      s->queue.erase(q);
      r->status = AFAR_ERR_CANCELLED;
      r->message = "the request was cancelled";
      s->finish_locked(r);
      return AFAR_OK;
    }
  r->cancel = true;  // being built or running: the worker retires it after its current chunk
  return AFAR_OK;
}

extern "C" afar_status afar_server_get_stats(afar_server* s, afar_server_stats* out) {
  using afar::set_error;
  if (!s || !out) return (set_error("afar_server_get_stats: null argument"), AFAR_ERR_ARGUMENT);
  std::lock_guard<std::mutex> lock(s->mu);
  *out = s->st;
  out->queued = (long long)s->queue.size();
  out->running = (long long)s->running.size();
  return AFAR_OK;
}

extern "C" afar_status afar_server_destroy(afar_server* s) {
  if (!s) return AFAR_OK;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  afar_batch_destroy(s->batch);
  for (auto& kv : s->all) delete kv.second;
  delete s;
  return AFAR_OK;
}
