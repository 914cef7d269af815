// Serving loop: continuous batching of factor + PCG requests on one GPU.
//
// A request names a matrix id, carries the matrix (CSC, full symmetric, as
// for rschol_factor_create) and 1..64 right-hand sides.  Each matrix id has
// at most one factor on the device and one PCG session on it
// (rschol_session_*): the columns of every request for that matrix join the
// session's block at an iteration boundary, so requests that arrive while
// others are iterating are admitted as soon as columns free up, and share
// one preconditioner pass per iteration.  The unit of scheduling is one
// session step (one PCG iteration of every active column of one matrix):
// worker threads take the matrices with work in turn, each step on that
// factor's own stream, so the steps of different matrices overlap on the
// device while one matrix is only ever stepped by one thread at a time.
//
// Admission by HBM footprint: a factor's bytes are its live device bytes
// (factor arrays, solve work vectors and session blocks), re-read after every
// step.  A new factor is admitted while the cached bytes stay within the
// budget, evicting idle factors (no queued or active columns) least recently
// used first; a factor that does not fit next to busy ones is dropped and
// built again once bytes free up, and one larger than the whole budget fails
// its requests with RSCHOL_E_OOM.  The budget bounds the admitted factors; a
// factor being built is on the device before it is admitted.
//
// A request's result does not depend on the mix: a factor is a deterministic
// function of its matrix and parameters, and a column's PCG iterates do not
// depend on the other columns of the block.
//
// No counterpart in the reference (its pcg_solver driver solves one system
// per process).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../../include/rschol_gpu.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

constexpr int kSessionColumns = 64;

struct Request {
  int id = 0, matrixId = 0, n = 0, nrhs = 1, maxit = 0;
  double eps = 1e-8;
  std::vector<int> colptr, rowind;
  std::vector<double> vals, xyz, b, x;
  std::vector<rschol_pcg_info> info;
  double submitted = 0, started = 0, finished = 0, factorSeconds = 0;
  int status = RSCHOL_OK;
  bool done = false, cacheHit = false;
};

struct Matrix {
  rschol_ctx* ctx = nullptr;
  rschol_factor* f = nullptr;
  rschol_session* ses = nullptr;
  double bytes = 0, lastUse = 0;
  bool built = false;     // factor and session exist and are admitted
  bool busy = false;      // a worker holds it (building or stepping)
  bool queued = false;    // in the ready queue
  bool blocked = false;   // did not fit next to busy factors: waits for bytes to free up
  std::deque<std::shared_ptr<Request>> waiting;            // not yet in the session
  std::map<long long, std::shared_ptr<Request>> running;   // columns in the session
  bool idle() const { return built && !busy && !queued && waiting.empty() && running.empty(); }
};

void release(Matrix& m) {
  if (m.ses) rschol_session_destroy(m.ses);
  if (m.f) rschol_factor_free(m.f);
  if (m.ctx) rschol_destroy(m.ctx);
  m.ses = nullptr;
  m.f = nullptr;
  m.ctx = nullptr;
}

}  // namespace

struct rschol_server {
  rschol_params params{};
  double budget = 0;
  std::mutex mu;
  std::condition_variable cvWork, cvDone;
  std::map<int, std::shared_ptr<Request>> requests;
  std::map<int, Matrix> mats;
  std::deque<int> ready;   // matrix ids with work and no worker
  double cachedBytes = 0, peakBytes = 0;
  long long hits = 0, misses = 0, evictions = 0, completed = 0;
  int nextId = 1;
  bool stopping = false;
  std::vector<std::thread> workers;

  // Caller holds mu.
  void enqueue(int id) {
    Matrix& m = mats[id];
    if (m.queued || m.busy || m.blocked) return;
    m.queued = true;
    ready.push_back(id);
    cvWork.notify_one();
  }

  // Caller holds mu.  Evict idle factors, least recently used first, until
  // `need` more bytes fit the budget; false if they cannot.
  bool make_room(double need) {
    while (cachedBytes + need > budget) {
      int victim = -1;
      double oldest = 0;
      for (auto& kv : mats)
        if (kv.second.idle() && (victim < 0 || kv.second.lastUse < oldest)) {
          victim = kv.first;
          oldest = kv.second.lastUse;
        }
      if (victim < 0) return false;
      Matrix& m = mats[victim];
      release(m);
      cachedBytes -= m.bytes;
      mats.erase(victim);
      ++evictions;
    }
    return true;
  }

  // Caller holds mu.  Bytes were freed: blocked matrices try again.
  void unblock() {
    for (auto& kv : mats)
      if (kv.second.blocked) {
        kv.second.blocked = false;
        enqueue(kv.first);
      }
  }

  // Caller holds mu.
  void finish(Request& r, int status) {
    r.status = status;
    r.finished = now_s();
    r.done = true;
    ++completed;
  }

  // Caller holds mu.
  void fail_all(Matrix& m, int status) {
    for (auto& r : m.waiting) finish(*r, status);
    for (auto& kv : m.running) finish(*kv.second, status);
    m.waiting.clear();
    m.running.clear();
  }

  // Build the factor and session of matrix `id` from request r (no lock held).
  void build(int id, const Request& r) {
    const double t0 = now_s();
    rschol_ctx* ctx = rschol_create(&params);
    rschol_factor* f = nullptr;
    rschol_session* ses = nullptr;
    int st = ctx ? rschol_factor_create(ctx, r.n, r.colptr.data(), r.rowind.data(), r.vals.data(),
                                        r.xyz.empty() ? nullptr : r.xyz.data(), &f)
                 : RSCHOL_E_NO_DEVICE;
    if (st == RSCHOL_OK) {
      ses = rschol_session_create(f, kSessionColumns);
      if (!ses) st = RSCHOL_E_CUDA;
    }
    const double bytes = st == RSCHOL_OK ? rschol_factor_device_bytes(f) : 0.0;
    const double dt = now_s() - t0;
    std::lock_guard<std::mutex> lock(mu);
    Matrix& m = mats[id];
    m.busy = false;
    if (st != RSCHOL_OK || bytes > budget) {
      if (ses) rschol_session_destroy(ses);
      if (f) rschol_factor_free(f);
      if (ctx) rschol_destroy(ctx);
      fail_all(m, st != RSCHOL_OK ? st : RSCHOL_E_OOM);
      mats.erase(id);
      cvDone.notify_all();
      return;
    }
    if (!make_room(bytes)) {   // wait for busy factors to go idle
      rschol_session_destroy(ses);
      rschol_factor_free(f);
      rschol_destroy(ctx);
      m.blocked = true;
      return;
    }
    m.ctx = ctx;
    m.f = f;
    m.ses = ses;
    m.bytes = bytes;
    m.built = true;
    m.lastUse = now_s();
    cachedBytes += bytes;
    peakBytes = std::max(peakBytes, cachedBytes);
    for (auto& q : m.waiting) q->factorSeconds = dt;
    enqueue(id);
  }

  // One step of matrix `id`'s session (no lock held on entry).
  void step(int id) {
    std::vector<std::shared_ptr<Request>> joining;
    rschol_session* ses;
    int n;
    {
      std::lock_guard<std::mutex> lock(mu);
      Matrix& m = mats[id];
      ses = m.ses;
      n = rschol_factor_n(m.f);
      const double t = now_s();
      while (!m.waiting.empty()) {
        auto r = m.waiting.front();
        m.waiting.pop_front();
        if (r->n != n) {   // a matrix id names one matrix
          finish(*r, RSCHOL_E_BAD_INPUT);
          continue;
        }
        r->started = t;
        m.running[r->id] = r;
        joining.push_back(r);
      }
    }
    for (auto& r : joining) {
      r->x.assign((size_t)n * r->nrhs, 0.0);
      r->info.assign(r->nrhs, rschol_pcg_info{});
      rschol_session_add(ses, r->id, r->nrhs, r->b.data(), r->x.data(), r->eps, r->maxit);
    }
    std::vector<long long> doneTags(kSessionColumns);
    int nd = 0;
    const int st = rschol_session_step(ses, doneTags.data(), &nd);
    int active = 0, queuedCols = 0;
    rschol_session_counts(ses, &active, &queuedCols);
    std::lock_guard<std::mutex> lock(mu);
    Matrix& m = mats[id];
    m.busy = false;
    if (st != RSCHOL_OK) {   // the session's state is lost: fail its requests, drop the factor
      fail_all(m, st);
      release(m);
      cachedBytes -= m.bytes;
      mats.erase(id);
      unblock();
      cvDone.notify_all();
      return;
    }
    for (int i = 0; i < nd; ++i) {
      auto it = m.running.find(doneTags[i]);
      if (it == m.running.end()) continue;
      Request& r = *it->second;
      finish(r, rschol_session_result(ses, doneTags[i], r.info.data()));
      m.running.erase(it);
    }
    const double now = rschol_factor_device_bytes(m.f);
    cachedBytes += now - m.bytes;
    m.bytes = now;
    peakBytes = std::max(peakBytes, cachedBytes);
    m.lastUse = now_s();
    if (active > 0 || queuedCols > 0 || !m.waiting.empty()) {
      enqueue(id);
    } else {
      if (cachedBytes > budget) make_room(0);
      unblock();
    }
    if (nd > 0) cvDone.notify_all();
  }

  void run_worker() {
    cudaSetDevice(params.device);   // every worker thread works on the server's device
    for (;;) {
      int id;
      std::shared_ptr<Request> first;
      bool needBuild;
      {
        std::unique_lock<std::mutex> lock(mu);
        cvWork.wait(lock, [&] { return stopping || !ready.empty(); });
        if (ready.empty()) return;   // stopping, nothing left to do
        id = ready.front();
        ready.pop_front();
        Matrix& m = mats[id];
        m.queued = false;
        m.busy = true;
        needBuild = !m.built;
        if (needBuild) {
          if (m.waiting.empty()) {   // nothing to build for
            mats.erase(id);
            continue;
          }
          first = m.waiting.front();
        }
      }
      if (needBuild) build(id, *first);
      else step(id);
    }
  }
};

extern "C" {

rschol_server* rschol_server_create(const rschol_params* p, int workers, double hbm_budget_bytes) {
  if (!p || workers < 1 || hbm_budget_bytes <= 0) return nullptr;
  rschol_server* s = new rschol_server();
  s->params = *p;
  s->budget = hbm_budget_bytes;
  for (int w = 0; w < workers; ++w) s->workers.emplace_back([s] { s->run_worker(); });
  return s;
}

int rschol_server_submit(rschol_server* s, int matrix_id, int n, const int* colptr, const int* rowind,
                         const double* vals, const double* xyz, int nrhs, const double* b, double eps, int maxit) {
  if (!s || n <= 0 || !colptr || !rowind || !vals || !b || nrhs < 1 || nrhs > 64 || maxit < 1)
    return -RSCHOL_E_BAD_INPUT;
  auto r = std::make_shared<Request>();
  r->matrixId = matrix_id;
  r->n = n;
  r->nrhs = nrhs;
  r->eps = eps;
  r->maxit = maxit;
  r->b.assign(b, b + (size_t)n * nrhs);
  r->submitted = now_s();
  std::lock_guard<std::mutex> lock(s->mu);
  Matrix& m = s->mats[matrix_id];
  const bool first = !m.built && !m.busy && !m.blocked && m.waiting.empty();
  if (first) {   // the request that builds the factor carries the matrix
    r->colptr.assign(colptr, colptr + n + 1);
    r->rowind.assign(rowind, rowind + colptr[n]);
    r->vals.assign(vals, vals + colptr[n]);
    if (xyz) r->xyz.assign(xyz, xyz + 3 * (size_t)n);
    ++s->misses;
  } else {
    ++s->hits;   // cached, or being built for an earlier request
  }
  r->cacheHit = m.built;
  r->id = s->nextId++;
  s->requests[r->id] = r;
  m.waiting.push_back(r);
  s->enqueue(matrix_id);
  return r->id;
}

int rschol_server_wait(rschol_server* s, int request_id, double* x, rschol_pcg_info* info, double* times) {
  if (!s) return RSCHOL_E_BAD_INPUT;
  std::shared_ptr<Request> r;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return RSCHOL_E_BAD_INPUT;
    r = it->second;
    s->cvDone.wait(lock, [&] { return r->done; });
    s->requests.erase(request_id);
  }
  if (x && !r->x.empty()) std::memcpy(x, r->x.data(), sizeof(double) * r->x.size());
  if (info)
    for (int k = 0; k < r->nrhs && k < (int)r->info.size(); ++k) info[k] = r->info[k];
  if (times) {
    const double started = r->started > 0 ? r->started : r->finished;
    times[0] = started - r->submitted;      // queued (includes building its factor)
    times[1] = r->factorSeconds;            // the factorisation it waited for (0 on a cache hit)
    times[2] = r->finished - started;       // PCG
    times[3] = r->finished - r->submitted;  // latency
    times[4] = r->cacheHit ? 1.0 : 0.0;
  }
  return r->status;
}

int rschol_server_stats(rschol_server* s, double* out) {
  if (!s || !out) return RSCHOL_E_BAD_INPUT;
  std::lock_guard<std::mutex> lock(s->mu);
  int cached = 0, waiting = 0;
  for (auto& kv : s->mats) {
    if (kv.second.built) ++cached;
    waiting += (int)kv.second.waiting.size();
  }
  out[0] = (double)s->completed;
  out[1] = (double)s->hits;
  out[2] = (double)s->misses;
  out[3] = (double)s->evictions;
  out[4] = s->cachedBytes;
  out[5] = s->peakBytes;
  out[6] = (double)cached;
  out[7] = (double)waiting;
  return RSCHOL_OK;
}

void rschol_server_destroy(rschol_server* s) {
  if (!s) return;
  {
    // finish what was submitted, then stop
    std::unique_lock<std::mutex> lock(s->mu);
    s->cvDone.wait(lock, [&] {
      for (auto& kv : s->requests)
        if (!kv.second->done) return false;
      return true;
    });
    s->stopping = true;
  }
  s->cvWork.notify_all();
  for (auto& t : s->workers) t.join();
  for (auto& kv : s->mats) release(kv.second);
  delete s;
}

}  // extern "C"
