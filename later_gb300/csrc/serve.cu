// Least-squares serving loop (no reference counterpart).
//
// A server owns one device, `slots` worker threads (each with its own CUDA
// stream) and an HBM budget carved out of one device allocation by a
// first-fit free-list pool (HbmPool). Requests (host A, B; host X out) enter
// a FIFO queue; a free worker admits the head request as soon as the pool can
// hold everything the request needs (A, B, X, the solver's work and hwork),
// so requests that arrive while others run are admitted as slots and memory
// free up, and their kernels overlap on the device (continuous batching; no
// request waits for a "batch" to fill). Each request runs later::ls_solve:
// tensor-core rgsqrf, QR factors kept in HBM for the whole solve, FP64-residual
// refinement to the requested backward error. Latency is measured per request
// from submit to completion on the host's steady clock.
//
// Each request has its own device status word (carved with its buffers): the
// worker thread directs the status reports of the kernels it launches for the
// request to that word, so a timeout, range or pivot flag raised by one
// request is seen by that request alone. Each request's arithmetic does not
// depend on the others.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/later_c.h"
#include "qr.cuh"
#include "solve.cuh"

namespace later {
namespace {

using Clock = std::chrono::steady_clock;

// First-fit free list with coalescing over [0, size).
class HbmPool {
 public:
  explicit HbmPool(size_t size) : size_(size) { free_[0] = size; }
  // Returns the offset or SIZE_MAX when nothing fits.
  size_t alloc(size_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        const size_t off = it->first, rest = it->second - bytes;
        free_.erase(it);
        if (rest) free_[off + bytes] = rest;
        used_ += bytes;
        if (used_ > peak_) peak_ = used_;
        return off;
      }
    }
    return SIZE_MAX;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }
  size_t peak() const { return peak_; }
  size_t size() const { return size_; }

 private:
  size_t size_;
  size_t used_ = 0;
  size_t peak_ = 0;
  std::map<size_t, size_t> free_;
};

struct Job {
  later_ls_request_t req{};
  int64_t ticket = 0;
  Clock::time_point t_submit, t_start, t_done;
  later_ls_result_t res{};
  bool done = false;
  size_t bytes = 0;
};

struct Layout {
  size_t status, a, b, x, work, hwork, total;
  int64_t lwork, lhwork;
};

Layout layout_for(const later_ls_request_t& r, const Options& o) {
  Layout L{};
  const SolveNeed need = ls_solve_need(r.m, r.n, r.nrhs, o);
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  size_t off = 0;
  L.status = off;
  off += 256;
  L.a = off;
  off += up(sizeof(float) * r.m * static_cast<size_t>(r.n));
  L.b = off;
  off += up(sizeof(float) * r.m * static_cast<size_t>(r.nrhs));
  L.x = off;
  off += up(sizeof(double) * r.n * static_cast<size_t>(r.nrhs));
  L.work = off;
  L.lwork = need.work;
  off += up(sizeof(float) * static_cast<size_t>(need.work));
  L.hwork = off;
  L.lhwork = need.hwork;
  off += up(2 * static_cast<size_t>(need.hwork));
  L.total = off;
  return L;
}

}  // namespace
}  // namespace later

struct later_server {
  int device = 0;
  int slots = 1;
  later::Options opt;
  int max_iter = 30;
  double tol = 1e-6;
  char* base = nullptr;
  std::unique_ptr<later::HbmPool> pool;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<later::Job>> pending;
  std::unordered_map<int64_t, std::shared_ptr<later::Job>> jobs;
  int64_t next_ticket = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  later::Clock::time_point t0 = later::Clock::now();
};

namespace later {
namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

void run_job(later_server* s, Job& j, size_t off, const Layout& L, cudaStream_t st, int slot) {
  const auto& r = j.req;
  char* base = s->base + off;
  float* dA = reinterpret_cast<float*>(base + L.a);
  float* dB = reinterpret_cast<float*>(base + L.b);
  double* dX = reinterpret_cast<double*>(base + L.x);
  float* dW = reinterpret_cast<float*>(base + L.work);
  void* dH = base + L.hwork;
  int* status = reinterpret_cast<int*>(base + L.status);
  ThreadStatusWord own_status(status);  // this request's kernels report here
  later_status_t st_ = LATER_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && st_ == LATER_OK) st_ = LATER_ERR_CUDA;
  };
  ck(cudaMemsetAsync(status, 0, sizeof(int), st));
  ck(cudaMemcpy2DAsync(dA, sizeof(float) * r.m, r.A, sizeof(float) * r.lda, sizeof(float) * r.m, r.n,
                       cudaMemcpyHostToDevice, st));
  ck(cudaMemcpy2DAsync(dB, sizeof(float) * r.m, r.B, sizeof(float) * r.ldb, sizeof(float) * r.m, r.nrhs,
                       cudaMemcpyHostToDevice, st));
  SolveInfo info;
  if (st_ == LATER_OK)
    st_ = ls_solve(st, r.m, r.n, r.nrhs, dA, r.m, dB, r.m, dX, r.n, dW, L.lwork, dH, L.lhwork, s->opt, s->max_iter,
                   s->tol, &info);
  if (st_ == LATER_OK)
    ck(cudaMemcpy2DAsync(r.X, sizeof(double) * r.ldx, dX, sizeof(double) * r.n, sizeof(double) * r.n, r.nrhs,
                         cudaMemcpyDeviceToHost, st));
  ck(cudaStreamSynchronize(st));
  j.res.status = st_;
  j.res.iterations = info.iterations;
  j.res.backward_error = info.backward_error;
  j.res.slot = slot;
}

void worker(later_server* s, int slot) {
  cudaSetDevice(s->device);
  cudaStream_t st;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  while (true) {
    std::shared_ptr<Job> j;
    size_t off = 0;
    Layout L{};
    {
      std::unique_lock<std::mutex> lk(s->mu);
      while (true) {
        if (s->stop && s->pending.empty()) {
          lk.unlock();
          cudaStreamDestroy(st);
          return;
        }
        if (!s->pending.empty()) {
          L = layout_for(s->pending.front()->req, s->opt);
          off = s->pool->alloc(L.total);
          if (off != SIZE_MAX) break;  // head request admitted
        }
        s->cv_work.wait(lk);
      }
      j = s->pending.front();
      s->pending.pop_front();
      j->bytes = L.total;
      j->t_start = Clock::now();
    }
    s->cv_work.notify_all();  // the next request may fit as well
    run_job(s, *j, off, L, st, slot);
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->pool->release(off, L.total);
      j->t_done = Clock::now();
      j->res.queue_ms = ms_between(j->t_submit, j->t_start);
      j->res.service_ms = ms_between(j->t_start, j->t_done);
      j->res.latency_ms = ms_between(j->t_submit, j->t_done);
      j->res.submit_ms = ms_between(s->t0, j->t_submit);
      j->done = true;
    }
    s->cv_work.notify_all();
    s->cv_done.notify_all();
  }
}

}  // namespace
}  // namespace later

using namespace later;

extern "C" {

later_server_t* later_c_ls_server_create(int device, int slots, int64_t hbm_budget_bytes, const later_options_t* opt,
                                         int max_iter, double tol) {
  if (slots < 1 || hbm_budget_bytes < (1 << 20)) return nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  auto* s = new later_server;
  s->device = device;
  s->slots = slots;
  s->opt = options_from(opt);
  s->max_iter = max_iter;
  s->tol = tol;
  if (cudaMalloc(&s->base, static_cast<size_t>(hbm_budget_bytes)) != cudaSuccess) {
    delete s;
    return nullptr;
  }
  s->pool = std::make_unique<HbmPool>(static_cast<size_t>(hbm_budget_bytes));
  for (int i = 0; i < slots; ++i) s->workers.emplace_back(worker, s, i);
  return s;
}

int64_t later_c_ls_server_submit(later_server_t* s, const later_ls_request_t* r) {
  if (!s || !r || !r->A || !r->B || !r->X || r->m < r->n || r->n < 1 || r->nrhs < 1 || r->nrhs > 16 ||
      r->lda < r->m || r->ldb < r->m || r->ldx < r->n)
    return -static_cast<int64_t>(LATER_ERR_INVALID_ARG);
  const Layout L = layout_for(*r, s->opt);
  if (L.total > s->pool->size()) return -static_cast<int64_t>(LATER_ERR_WORKSPACE);
  auto j = std::make_shared<Job>();
  j->req = *r;
  j->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  j->ticket = s->next_ticket++;
  s->jobs[j->ticket] = j;
  s->pending.push_back(j);
  s->cv_work.notify_all();
  return j->ticket;
}

later_status_t later_c_ls_server_wait(later_server_t* s, int64_t ticket, later_ls_result_t* out) {
  if (!s) return LATER_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return LATER_ERR_INVALID_ARG;
  auto j = it->second;
  s->cv_done.wait(lk, [&] { return j->done; });
  if (out) *out = j->res;
  s->jobs.erase(it);
  return LATER_OK;
}

int64_t later_c_ls_server_hbm_in_use(later_server_t* s) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  return static_cast<int64_t>(s->pool->used());
}

int64_t later_c_ls_server_hbm_peak(later_server_t* s) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  return static_cast<int64_t>(s->pool->peak());
}

void later_c_ls_server_destroy(later_server_t* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto& t : s->workers) t.join();
  cudaFree(s->base);
  delete s;
}

}  // extern "C"
