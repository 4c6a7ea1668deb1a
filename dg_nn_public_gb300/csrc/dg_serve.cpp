// Native request queue of the serving form: dg_server_create, dg_enqueue,
// dg_poll, dg_wait, dg_server_destroy.
//
// nworkers host threads, each with its own non-blocking CUDA stream, take
// queued requests in arrival order and run them through the public entry
// points of the library: an optional operator rebuild for new diffusivities
// (dg_set_kappa + dg_build_operator) and the solve (dg_solve_mixed or
// dg_gmres), then synchronise their stream.  A context serves one request
// at a time: a request whose context is busy stays queued, and later
// requests on free contexts may start before it (requests on one context
// keep their order).  Requests on different contexts run concurrently on
// the workers' streams; the per-context calls are the ones a single-threaded
// caller would make, so their results are those of the same calls made
// directly.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "dg_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  dg_ctx* ctx = nullptr;
  double* x = nullptr;
  const double* b = nullptr;
  double tol = 0.0, inner_rtol = 1e-3;
  int32_t mode = 0, m = 30, max_its = 1000;
  bool has_kappa = false;
  std::vector<double> kappa;
  int32_t state = DG_REQ_QUEUED;
  int32_t status = DG_OK, its = 0;
  double res = 0.0;
  Clock::time_point t_enq, t_start, t_end;
};

double secs(Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); }

}  // namespace

struct dg_server {
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<int64_t> queue;
  std::unordered_map<int64_t, Request> reqs;   // queued, running and finished-but-unreported requests
  std::unordered_set<dg_ctx*> busy;
  std::vector<std::thread> workers;
  bool stop = false;
  int64_t next_id = 1;
  int dev = 0;
};

namespace {

void run_request(Request& r, cudaStream_t st) {
  int rc = DG_OK;
  int32_t its = 0;
  double res = 0.0;
  if (!st) {
    rc = dg::set_thread_error(DG_ERR_CUDA, "dg_enqueue: the worker has no CUDA stream");
  } else {
    if (r.has_kappa) {
      rc = dg_set_kappa(r.ctx, r.kappa.data());
      if (!rc) rc = dg_build_operator(r.ctx, st);
    }
    if (!rc) {
      if (r.mode == 0) {
        int32_t outer = 0;
        rc = dg_solve_mixed(r.ctx, r.x, r.b, r.tol, r.m, r.max_its, r.inner_rtol, &its, &res, &outer, st);
      } else {
        rc = dg_gmres(r.ctx, r.x, r.b, r.tol, r.m, r.max_its, &its, &res, st);
      }
    }
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess && !rc) rc = DG_ERR_CUDA;
  }
  r.status = rc;
  r.its = its;
  r.res = res;
}

void worker_main(dg_server* s) {
  cudaSetDevice(s->dev);
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) st = nullptr;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    auto it = s->queue.begin();
    while (it != s->queue.end() && s->busy.count(s->reqs[*it].ctx)) ++it;
    if (it == s->queue.end()) {
      if (s->stop && s->queue.empty()) break;
      s->work_cv.wait(lk);
      continue;
    }
    const int64_t id = *it;
    s->queue.erase(it);
    // references into the map stay valid: only finished requests are erased
    Request& r = s->reqs[id];
    s->busy.insert(r.ctx);
    r.state = DG_REQ_RUNNING;
    r.t_start = Clock::now();
    lk.unlock();
    run_request(r, st);
    lk.lock();
    r.t_end = Clock::now();
    r.state = DG_REQ_DONE;
    s->busy.erase(r.ctx);
    s->done_cv.notify_all();
    s->work_cv.notify_all();
  }
  lk.unlock();
  if (st) cudaStreamDestroy(st);
}

// outputs of a finished request; the record is dropped (reported once)
void report(dg_server* s, std::unordered_map<int64_t, Request>::iterator it, int32_t* state, int32_t* status,
            int32_t* its, double* res, double* seconds) {
  const Request& r = it->second;
  if (state) *state = r.state;
  if (r.state != DG_REQ_DONE) return;
  if (status) *status = r.status;
  if (its) *its = r.its;
  if (res) *res = r.res;
  if (seconds) {
    seconds[0] = secs(r.t_enq, r.t_start);
    seconds[1] = secs(r.t_start, r.t_end);
  }
  s->reqs.erase(it);
}

}  // namespace

extern "C" int dg_server_create(int32_t device, int32_t nworkers, dg_server** out) {
  if (!out) return dg::set_thread_error(DG_ERR_ARG, "dg_server_create: null argument");
  *out = nullptr;
  if (nworkers < 1 || nworkers > 64) return dg::set_thread_error(DG_ERR_ARG, "dg_server_create: 1 <= nworkers <= 64");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return dg::set_thread_error(DG_ERR_CUDA, "dg_server_create: no such CUDA device");
  }
  dg_server* s = new dg_server();
  s->dev = device;
  try {
    for (int i = 0; i < nworkers; ++i) s->workers.emplace_back(worker_main, s);
  } catch (...) {
    dg_server_destroy(s);
    return dg::set_thread_error(DG_ERR_ALLOC, "dg_server_create: could not start the worker threads");
  }
  *out = s;
  return DG_OK;
}

extern "C" int dg_server_destroy(dg_server* s) {
  if (!s) return DG_OK;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->work_cv.notify_all();
  for (auto& t : s->workers)
    if (t.joinable()) t.join();
  delete s;
  return DG_OK;
}

extern "C" int dg_enqueue(dg_server* s, dg_ctx* ctx, double* x, const double* b, double tol, int32_t mode, int32_t m,
                          int32_t max_its, double inner_rtol, const double* kappa, int64_t* id) {
  if (!s || !ctx || !x || !b || !id) return dg::set_thread_error(DG_ERR_ARG, "dg_enqueue: null argument");
  if (mode != 0 && mode != 1) return dg::set_thread_error(DG_ERR_ARG, "dg_enqueue: mode 0 (mixed) or 1 (FP64)");
  Request r;
  r.ctx = ctx;
  r.x = x;
  r.b = b;
  r.tol = tol;
  r.mode = mode;
  r.m = m;
  r.max_its = max_its;
  r.inner_rtol = inner_rtol;
  if (kappa) {
    int64_t info[3] = {0, 0, 0};
    if (dg_info(ctx, info, 3)) return DG_ERR_ARG;
    r.has_kappa = true;
    r.kappa.assign(kappa, kappa + info[2]);
  }
  r.t_enq = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return dg::set_thread_error(DG_ERR_STATE, "dg_enqueue: the server is shutting down");
    *id = s->next_id++;
    s->reqs.emplace(*id, std::move(r));
    s->queue.push_back(*id);
  }
  s->work_cv.notify_all();
  return DG_OK;
}

extern "C" int dg_poll(dg_server* s, int64_t id, int32_t* state, int32_t* status, int32_t* its, double* res_norm,
                       double* seconds) {
  if (!s) return dg::set_thread_error(DG_ERR_ARG, "dg_poll: null server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return dg::set_thread_error(DG_ERR_ARG, "dg_poll: unknown or already reported request");
  report(s, it, state, status, its, res_norm, seconds);
  return DG_OK;
}

extern "C" int dg_wait(dg_server* s, int64_t id, double timeout_s, int32_t* state, int32_t* status, int32_t* its,
                       double* res_norm, double* seconds) {
  if (!s) return dg::set_thread_error(DG_ERR_ARG, "dg_wait: null server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto done = [&] {
    auto it = s->reqs.find(id);
    return it == s->reqs.end() || it->second.state == DG_REQ_DONE;
  };
  if (timeout_s < 0.0) {
    s->done_cv.wait(lk, done);
  } else {
    s->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
  }
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return dg::set_thread_error(DG_ERR_ARG, "dg_wait: unknown or already reported request");
  report(s, it, state, status, its, res_norm, seconds);
  return DG_OK;
}
