// C ABI (include/rschol_gpu.h): FactorPreconditioner / PCG_SOLVER /
// pcg_pysolve replacements on one GB300.
#include <algorithm>
#include <climits>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "../../../include/rschol_gpu.h"
#include "../host/ordering.h"
#include "../host/parallel.h"
#include "../host/symbolic.h"
#include "factor.cuh"
#include "pcg.cuh"
#include "solve.cuh"

using namespace rschol;

struct rschol_ctx {
  rschol_params prm;
  cudaStream_t stream = nullptr;
  std::string err;
  int device = 0;
  double* noallocWork = nullptr;   // device address of the static work vector of this device
};

// Looks up (once per device, that device current) the device address of the
// static work vector of rschol_precond_apply_device_noalloc.
static cudaError_t noalloc_lookup(int device, double** addr);

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

Params to_params(const rschol_params& p) {
  Params q;
  q.max_dense_block = p.max_dense_block;
  q.max_diag_block = p.max_diag_block;
  q.explicit_threshold = p.explicit_threshold;
  q.nd_leaf = p.nd_leaf;
  q.oversampling = p.oversampling;
  q.rank_cap = p.rank_cap;
  q.power_iters = p.power_iters;
  q.reorder_separators = p.reorder_separators;
  q.rank_constant = p.rank_constant;
  q.diag_rank_constant = p.diag_rank_constant;
  q.max_factor_attempts = p.max_factor_attempts;
  q.rank_alpha = p.rank_alpha;
  q.seed = p.seed;
  q.root_fp64 = p.root_fp64;
  q.schur_bf16 = p.schur_bf16;
  return q;
}

struct Impl {
  virtual ~Impl() = default;
  unsigned long long planGen = 0;   // bumped by every plan(): the solve's buffers may have moved
  virtual void plan() = 0;
  virtual int run() = 0;
  virtual void apply(double* d_w, cudaStream_t s) = 0;
  virtual int apply_error(cudaStream_t s) = 0;   // nonzero: a row-block wait of the solve gave up
  virtual void step_timing(bool on, double* out) = 0;
  virtual void apply_batch(double* W, int k, cudaStream_t s) = 0;   // W: n x k row-major, permuted
  virtual int batch_capacity() const = 0;
  virtual int apply_batch_error(cudaStream_t s) = 0;
  virtual long long batch_generation() const = 0;
  virtual void set_values(const double* lower) = 0;
  virtual double* device_values() = 0;
  virtual long long launches() const = 0;
  virtual long long apply_launches() const = 0;
  virtual double flops() const = 0;
  // fused Cholesky steps: algorithmic bytes of each launch (in launch order), total flops
  virtual void chol_work(std::vector<double>* bytes, double* flops) const = 0;
  virtual double apply_bytes() const = 0;
  virtual size_t bytes() const = 0;
  virtual std::vector<std::array<double, 6>> batch_tuning() const = 0;
  virtual void autotune_batch(int kmax, cudaStream_t s) = 0;
  virtual void set_schedule(int tcMinK, bool fused) = 0;
  virtual int tc_min_k() const = 0;
  virtual bool fused_chol() const = 0;
  virtual void node_l11(int j, double* out) = 0;
  virtual void node_l21(int j, double* out) = 0;
};

template <class T>
struct ImplT : Impl {
  FactorEngine<T> fe;
  SolveEngine<T> se;
  ImplT(const Symbolic& S, const CSC& A, const Params& p, cudaStream_t s) : fe(S, A, p, s), se(fe) {
    fe.post = [this]() { return se.prepare(fe.stream); };
  }
  void plan() override {
    fe.plan();
    se.plan();
    ++planGen;
  }
  void set_schedule(int tcMinK, bool fused) override { fe.set_schedule(tcMinK, fused); }
  int tc_min_k() const override { return fe.tc_min_k(); }
  bool fused_chol() const override { return fe.fused_chol(); }
  int run() override { return fe.run(); }
  void apply(double* w, cudaStream_t s) override { se.apply_inplace(w, s); }
  int apply_error(cudaStream_t s) override { return se.take_error(s); }
  void apply_batch(double* W, int k, cudaStream_t s) override { se.apply_batch(W, k, s); }
  int batch_capacity() const override { return se.batch_capacity(); }
  int apply_batch_error(cudaStream_t s) override { return se.take_error_batch(s); }
  long long batch_generation() const override { return se.batch_generation(); }
  void step_timing(bool on, double* out) override {
    if (out)
      for (int k = 0; k < 8; ++k) {
        out[3 * k] = fe.stepMs[k];
        out[3 * k + 1] = fe.stepCount[k];
        out[3 * k + 2] = fe.stepFlops[k];
      }
    if (on && !fe.timeSteps)
      for (int k = 0; k < 8; ++k) fe.stepMs[k] = fe.stepCount[k] = fe.stepFlops[k] = 0;
    fe.timeSteps = on;
  }
  void set_values(const double* lower) override { fe.set_values(lower); }
  double* device_values() override { return fe.dAvals.template as<double>(); }
  long long launches() const override { return fe.launches; }
  long long apply_launches() const override { return se.launches_per_apply(); }
  double flops() const override { return fe.flops; }
  void chol_work(std::vector<double>* bytes, double* flops) const override {
    bytes->clear();
    *flops = 0;
    for (const Step& st : fe.steps_)
      if (st.kind == ST_CHOL) {
        bytes->push_back(st.bytes);
        *flops += st.flops;
      }
  }
  double apply_bytes() const override { return se.bytes_per_apply(); }
  size_t bytes() const override { return fe.deviceBytes; }
  std::vector<std::array<double, 6>> batch_tuning() const override { return se.batch_tuning(); }
  void autotune_batch(int kmax, cudaStream_t s) override { se.autotune_batch(kmax, s); }
  std::vector<T> fetch(const T* d, size_t count) {
    std::vector<T> h(count);
    if (count) RSCHOL_CUDA(cudaMemcpy(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost));
    return h;
  }
  void node_l11(int j, double* out) override {
    const Node& nd = fe.S.nodes[j];
    const int n = nd.n, ld = fe.ld[j];
    const T* base = nd.compressed ? fe.compressed() + fe.frontOff[j] : fe.interior() + fe.frontOff[j];
    std::vector<T> h = fetch(base, (size_t)(n - 1) * ld + n);
    for (int a = 0; a < n; ++a)
      for (int b = 0; b < n; ++b) out[(size_t)a * n + b] = b <= a ? (double)h[(size_t)a * ld + b] : 0.0;
  }
  void node_l21(int j, double* out) override {
    const Node& nd = fe.S.nodes[j];
    const int n = nd.n, ld = fe.ld[j];
    if (!nd.compressed) {
      if (nd.nStored == 0) return;
      std::vector<T> h = fetch(fe.interior() + fe.frontOff[j] + (size_t)n * ld, (size_t)(nd.nStored - 1) * ld + n);
      for (int a = 0; a < nd.nStored; ++a)
        for (int b = 0; b < n; ++b) out[(size_t)a * n + b] = (double)h[(size_t)a * ld + b];
      return;
    }
    const int r = fe.rank[j], m = nd.m();
    if (r == 0) return;
    std::vector<T> V = fetch(fe.vu() + fe.vOff[j], (size_t)m * r);
    std::vector<T> U = fetch(fe.vu() + fe.uOff[j], (size_t)n * r);
    for (int a = 0; a < m; ++a)
      for (int b = 0; b < n; ++b) {
        double s = 0;
        for (int k = 0; k < r; ++k) s += (double)V[(size_t)a * r + k] * (double)U[(size_t)b * r + k];
        out[(size_t)a * n + b] = s;
      }
  }
};

}  // namespace

namespace rschol {
thread_local std::atomic<long long>* g_devAccount = nullptr;
bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("RSCHOL_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}
}

struct rschol_factor {
  std::atomic<long long> devBytes{0};   // live device bytes of this factor (first member: destroyed last)
  rschol_ctx* ctx = nullptr;
  Params prm;
  int precision = RSCHOL_FP64;
  CSC Afull;
  OrderingResult ord;
  CSC A;                      // tril(P A P^T)
  std::vector<int> lowerSrc;  // A.x[k] = Afull.x[lowerSrc[k]]
  Symbolic S;
  std::unique_ptr<Impl> impl;
  std::unique_ptr<PcgEngine> pcg;
  std::vector<int> permCsrSrc;  // permuted CSR value k = Afull.x[permCsrSrc[k]]
  DevBuf dPerm, dB, dX, dBp, dXp, dLowerSrc, dCsrSrc;
  DevBuf dBk, dXk;   // batched right-hand sides / solutions, n x k row-major, permuted
  DevBuf dVals;      // rschol_refactor: the caller's values, staged on the device
  int kCap = 0;
  int nrhsCap = 0;
  double tSymbolic = 0, tNumeric = 0;
  double tPlan = 0;     // device plan: schedule, arenas, Gaussian stream, PCG engine
  int attempts = 0;
  double diagRankConstant = 0.5;
  double tunedMs = 0;   // rschol_factor_tune_schedule: the chosen schedule's factorisation time
  std::string desc;
};

static const char* const kSolveWaitMsg =
    "preconditioner solve: a wait between thread blocks exceeded its limit (result discarded)";

static int fail(rschol_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return code;
}

extern "C" {

void rschol_default_params(rschol_params* p) {
  p->max_dense_block = 200;
  p->max_diag_block = 400;
  p->explicit_threshold = 4000;
  p->nd_leaf = 64;
  p->oversampling = 5;
  p->rank_cap = 0;
  p->power_iters = 1;
  p->reorder_separators = 1;
  p->rank_constant = 0.4;
  p->diag_rank_constant = 0.5;
  p->max_factor_attempts = 10;
  p->rank_alpha = 1.25;
  p->seed = 152;
  p->precision = RSCHOL_FP64;
  p->device = 0;
  p->root_fp64 = 0;
  p->schur_bf16 = 0;
}

rschol_ctx* rschol_create(const rschol_params* p) {
  rschol_ctx* c = new rschol_ctx();
  if (p) c->prm = *p;
  else rschol_default_params(&c->prm);
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    c->err = "no CUDA device available";
    cudaGetLastError();
    return c;
  }
  c->device = c->prm.device;
  if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    c->err = "CUDA device initialisation failed";
    c->stream = nullptr;
    return c;
  }
  // the allocation-free apply's static work vector: its device address is
  // looked up here, with the device current, so that the apply only reads it
  const cudaError_t e = noalloc_lookup(c->device, &c->noallocWork);
  if (e != cudaSuccess) {
    c->err = std::string("cudaGetSymbolAddress of the static work vector: ") + cudaGetErrorString(e);
    cudaGetLastError();
    c->noallocWork = nullptr;
  }
  return c;
}

void rschol_destroy(rschol_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* rschol_last_error(const rschol_ctx* c) { return c ? c->err.c_str() : "null context"; }

// SparseSolver::factorNumeric (SparseSolver.cpp:174-214): retries only the
// IndefiniteDiagonalError of a compressed supernode's diagonal (its
// DiagonalBlock, DiagonalBlock.cpp:372-376 and 429-435) with a larger
// diagonal rank constant.  A non-positive pivot in an uncompressed
// supernode's exact Cholesky is where the reference aborts
// (Supernode.cpp:3681-3689): returned at once as RSCHOL_E_NOT_PD.
static int numeric_with_retry(rschol_factor* f) {
  rschol_ctx* ctx = f->ctx;
  double t0 = now_s();
  double dc = f->prm.diag_rank_constant;
  int status = 0;
  f->attempts = 0;
  for (int attempt = 0; attempt < f->prm.max_factor_attempts; ++attempt) {
    f->attempts++;
    if (attempt > 0) {
      // SparseSolver::factorNumeric: bump the diagonal rank constant, redo
      // the symbolic ranks without reordering, refactor from a reseeded stream
      assign_ranks(f->S, f->prm, f->prm.rank_constant, dc);
      f->impl->plan();
    }
    status = f->impl->run();   // 0, or 1 + the first supernode with a non-positive pivot
    if (status == 0) break;
    const int node = status - 1;
    if (node >= 0 && node < (int)f->S.nodes.size() && !f->S.nodes[node].compressed) {
      f->diagRankConstant = dc;
      f->tNumeric = now_s() - t0;
      return fail(ctx, RSCHOL_E_NOT_PD,
                  "matrix not positive definite: non-positive pivot in the diagonal of uncompressed supernode " +
                      std::to_string(node));
    }
    dc *= f->prm.rank_alpha;
  }
  f->diagRankConstant = dc;
  f->tNumeric = now_s() - t0;
  if (status != 0)
    return fail(ctx, RSCHOL_E_NOT_PD_AFTER_RETRY,
                "indefinite diagonal block of compressed supernode " + std::to_string(status - 1) + " after " +
                    std::to_string(f->attempts) + " attempts");
  return RSCHOL_OK;
}

// The pattern checks of rschol_factor_create; "" when the CSC arrays are valid.
static std::string csc_problem(int n, const int* colptr, const int* rowind) {
  if (n <= 0 || !colptr || !rowind) return "empty or null matrix";
  if (colptr[0] != 0) return "colptr[0] must be 0";
  for (int j = 0; j < n; ++j)
    if (colptr[j + 1] < colptr[j]) return "colptr must be non-decreasing";
  const int nnz = colptr[n];
  for (int k = 0; k < nnz; ++k)
    if (rowind[k] < 0 || rowind[k] >= n) return "row index out of range";
  return std::string();
}

// Host ordering and symbolic analysis only (no CUDA call): whether
// rschol_factor_create can take this structure with these parameters.
int rschol_check_structure(int n, const int* colptr, const int* rowind, const double* xyz,
                           const rschol_params* params, char* msg, int msg_len) {
  auto report = [&](int code, const std::string& why) {
    if (msg && msg_len > 0) {
      const size_t k = std::min(why.size(), (size_t)msg_len - 1);
      std::memcpy(msg, why.data(), k);
      msg[k] = 0;
    }
    return code;
  };
  const std::string bad = csc_problem(n, colptr, rowind);
  if (!bad.empty()) return report(RSCHOL_E_BAD_INPUT, bad);
  try {
    rschol_params c;
    if (params) c = *params;
    else rschol_default_params(&c);
    const Params prm = to_params(c);
    CSC A;
    A.n = n;
    A.p.assign(colptr, colptr + n + 1);
    A.i.assign(rowind, rowind + colptr[n]);
    const OrderingResult ord = build_ordering(A, xyz, prm);
    const Symbolic S = build_symbolic(permute_lower(A, ord.perm, ord.iperm), ord, prm);
    const std::string why = unsupported_reason(S, prm);
    return why.empty() ? report(RSCHOL_OK, "") : report(RSCHOL_E_UNSUPPORTED, why);
  } catch (const std::exception& e) {
    return report(RSCHOL_E_UNSUPPORTED, e.what());
  }
}

int rschol_factor_create(rschol_ctx* ctx, int n, const int* colptr, const int* rowind, const double* vals,
                         const double* xyz, rschol_factor** out) {
  if (!ctx || !out) return RSCHOL_E_BAD_INPUT;
  *out = nullptr;
  if (!ctx->stream) return fail(ctx, RSCHOL_E_NO_DEVICE, ctx->err.empty() ? "no device" : ctx->err);
  if (!vals) return fail(ctx, RSCHOL_E_BAD_INPUT, "empty or null matrix");
  {
    const std::string bad = csc_problem(n, colptr, rowind);
    if (!bad.empty()) return fail(ctx, RSCHOL_E_BAD_INPUT, bad);
  }
  const int nnz = colptr[n];
  std::unique_ptr<rschol_factor> f(new rschol_factor());
  AccountScope acct(&f->devBytes);
  f->ctx = ctx;
  f->prm = to_params(ctx->prm);
  f->precision = ctx->prm.precision;
  try {
    RSCHOL_CUDA(cudaSetDevice(ctx->device));
    double t0 = now_s();
    f->Afull.n = n;
    f->Afull.p.assign(colptr, colptr + n + 1);
    f->Afull.i.assign(rowind, rowind + nnz);
    f->Afull.x.assign(vals, vals + nnz);
    f->ord = build_ordering(f->Afull, xyz, f->prm);
    // permuted lower part, remembering where every value comes from
    {
      CSC idx = f->Afull;
      for (int k = 0; k < nnz; ++k) idx.x[k] = (double)k;
      CSC L = permute_lower(idx, f->ord.perm, f->ord.iperm);
      f->lowerSrc.resize(L.x.size());
      for (size_t k = 0; k < L.x.size(); ++k) f->lowerSrc[k] = (int)L.x[k];
      for (size_t k = 0; k < L.x.size(); ++k) L.x[k] = vals[f->lowerSrc[k]];
      f->A = std::move(L);
    }
    f->S = build_symbolic(f->A, f->ord, f->prm);
    {
      const std::string why = unsupported_reason(f->S, f->prm);
      if (!why.empty()) return fail(ctx, RSCHOL_E_UNSUPPORTED, why);
    }
    // permuted full CSR for the PCG SpMV (symmetric: CSC columns = CSR rows)
    std::vector<int> rp(n + 1, 0), ci(nnz);
    std::vector<double> cv(nnz);
    f->permCsrSrc.resize(nnz);
    for (int j = 0; j < n; ++j) rp[f->ord.iperm[j] + 1] = colptr[j + 1] - colptr[j];
    for (int i = 0; i < n; ++i) rp[i + 1] += rp[i];
    parallel_chunks(n, 16384, [&](long long b, long long e) {
      std::vector<std::pair<int, int>> tmp;
      for (long long i = b; i < e; ++i) {
        const int j = f->ord.perm[i];
        tmp.clear();
        for (int p = colptr[j]; p < colptr[j + 1]; ++p) tmp.push_back({f->ord.iperm[rowind[p]], p});
        std::sort(tmp.begin(), tmp.end());
        for (size_t k = 0; k < tmp.size(); ++k) {
          ci[rp[i] + k] = tmp[k].first;
          f->permCsrSrc[rp[i] + k] = tmp[k].second;
          cv[rp[i] + k] = vals[tmp[k].second];
        }
      }
    });
    f->tSymbolic = now_s() - t0;
    const double t1 = now_s();
    {
      PlanClock clk("create");
      if (f->precision == RSCHOL_MIXED) f->impl.reset(new ImplT<float>(f->S, f->A, f->prm, ctx->stream));
      else f->impl.reset(new ImplT<double>(f->S, f->A, f->prm, ctx->stream));
      clk.mark("engines");
      f->impl->plan();
      clk.mark("plan");
      f->pcg.reset(new PcgEngine(n, rp, ci, cv, ctx->stream));
      clk.mark("pcg");
    }
    f->tPlan = now_s() - t1;
    f->dPerm.alloc(sizeof(int) * n);
    RSCHOL_CUDA(cudaMemcpy(f->dPerm.p, f->ord.perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    f->dLowerSrc.alloc(sizeof(int) * std::max<size_t>(1, f->lowerSrc.size()));
    RSCHOL_CUDA(cudaMemcpy(f->dLowerSrc.p, f->lowerSrc.data(), sizeof(int) * f->lowerSrc.size(),
                           cudaMemcpyHostToDevice));
    f->dCsrSrc.alloc(sizeof(int) * std::max<size_t>(1, f->permCsrSrc.size()));
    RSCHOL_CUDA(cudaMemcpy(f->dCsrSrc.p, f->permCsrSrc.data(), sizeof(int) * f->permCsrSrc.size(),
                           cudaMemcpyHostToDevice));
    int st = numeric_with_retry(f.get());
    if (st != RSCHOL_OK) return st;
  } catch (const FactorWaitTimeout& e) {
    cudaGetLastError();
    return fail(ctx, RSCHOL_E_TIMEOUT, e.what());
  } catch (const CudaError& e) {
    cudaGetLastError();
    std::string m = e.what();
    return fail(ctx, m.find("out of memory") != std::string::npos ? RSCHOL_E_OOM : RSCHOL_E_CUDA, m);
  } catch (const std::exception& e) {
    return fail(ctx, RSCHOL_E_UNSUPPORTED, e.what());
  }
  *out = f.release();
  return RSCHOL_OK;
}

int rschol_refactor(rschol_factor* f, const double* vals) {
  if (!f || !vals) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    // one copy of the caller's values, then the device path's gathers into
    // the factor's lower triangle and the PCG's permuted CSR
    const size_t nnz = (size_t)f->Afull.p[f->Afull.n];
    f->dVals.alloc(sizeof(double) * std::max<size_t>(1, nnz));
    RSCHOL_CUDA(cudaMemcpyAsync(f->dVals.p, vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, f->ctx->stream));
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return rschol_refactor_device(f, f->dVals.as<double>());
}

static void ensure_vecs(rschol_factor* f, int nrhs);
static void ensure_batch(rschol_factor* f, int k);

int rschol_refactor_device(rschol_factor* f, const double* d_vals) {
  if (!f || !d_vals) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    cudaStream_t s = f->ctx->stream;
    launch_index_gather(d_vals, f->dLowerSrc.as<int>(), f->impl->device_values(), (long long)f->lowerSrc.size(), s);
    launch_index_gather(d_vals, f->dCsrSrc.as<int>(), f->pcg->values(), (long long)f->permCsrSrc.size(), s);
    if (f->attempts > 1) {
      assign_ranks(f->S, f->prm, f->prm.rank_constant, f->prm.diag_rank_constant);
      f->impl->plan();
    }
    return numeric_with_retry(f);
  } catch (const FactorWaitTimeout& e) {
    return fail(f->ctx, RSCHOL_E_TIMEOUT, e.what());
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
}

void* rschol_stream(rschol_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int rschol_profile(rschol_factor* f, const double* d_b, double* out) {
  if (!f || !d_b || !out) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    cudaStream_t s = f->ctx->stream;
    ensure_vecs(f, 1);
    cudaEvent_t e[8];
    for (auto& x : e) RSCHOL_CUDA(cudaEventCreate(&x));
    const int n = f->Afull.n;
    RSCHOL_CUDA(cudaEventRecord(e[0], s));
    int st = f->impl->run();
    RSCHOL_CUDA(cudaEventRecord(e[1], s));
    launch_gather(d_b, f->dPerm.as<int>(), f->dBp.as<double>(), n, s);
    RSCHOL_CUDA(cudaEventRecord(e[2], s));
    f->impl->apply(f->dBp.as<double>(), s);
    RSCHOL_CUDA(cudaEventRecord(e[3], s));
    f->pcg->spmv(f->dBp.as<double>(), f->dXp.as<double>());
    RSCHOL_CUDA(cudaEventRecord(e[4], s));
    launch_gather(d_b, f->dPerm.as<int>(), f->dBp.as<double>(), n, s);
    Impl* impl = f->impl.get();
    RSCHOL_CUDA(cudaEventRecord(e[5], s));
    PcgResult r = f->pcg->solve_graph(f->dBp.as<double>(), f->dXp.as<double>(), 1e-8, 10000,
                                      [impl, s](double* w) { impl->apply(w, s); }, impl->planGen);
    RSCHOL_CUDA(cudaEventRecord(e[6], s));
    RSCHOL_CUDA(cudaEventSynchronize(e[6]));
    float ms[6];
    RSCHOL_CUDA(cudaEventElapsedTime(&ms[0], e[0], e[1]));
    RSCHOL_CUDA(cudaEventElapsedTime(&ms[1], e[2], e[3]));
    RSCHOL_CUDA(cudaEventElapsedTime(&ms[2], e[3], e[4]));
    RSCHOL_CUDA(cudaEventElapsedTime(&ms[3], e[5], e[6]));
    for (auto& x : e) cudaEventDestroy(x);
    if (f->impl->apply_error(s)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
    out[0] = ms[0];
    out[1] = ms[1];
    out[2] = ms[2];
    out[3] = ms[3];
    out[4] = f->impl->apply_bytes();
    out[5] = f->pcg->spmvBytes;
    out[6] = (double)f->impl->launches();
    out[7] = (double)f->pcg->launches + (double)r.iterations * f->impl->apply_launches() +
             f->impl->apply_launches() + 2;
    out[8] = ms[1];
    out[9] = f->impl->apply_bytes();
    out[10] = r.iterations;
    out[11] = r.trueResidual;
    if (st != 0) return fail(f->ctx, RSCHOL_E_NOT_PD_AFTER_RETRY, "profile factorisation failed");
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

void rschol_factor_free(rschol_factor* f) { delete f; }

static void ensure_batch(rschol_factor* f, int k) {
  if (k <= f->kCap) return;
  const size_t bytes = sizeof(double) * (size_t)f->Afull.n * k;
  f->dBk.alloc(bytes);
  f->dXk.alloc(bytes);
  f->kCap = k;
}

static void ensure_vecs(rschol_factor* f, int nrhs) {
  if (nrhs <= f->nrhsCap) return;
  const size_t bytes = sizeof(double) * (size_t)f->Afull.n * nrhs;
  f->dB.alloc(bytes);
  f->dX.alloc(bytes);
  f->dBp.alloc(sizeof(double) * f->Afull.n);
  f->dXp.alloc(sizeof(double) * f->Afull.n);
  f->nrhsCap = nrhs;
}

int rschol_precond_apply_device(rschol_factor* f, const double* d_b, double* d_x, int nrhs) {
  if (!f || !d_b || !d_x || nrhs <= 0) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    ensure_vecs(f, 1);
    const int n = f->Afull.n;
    cudaStream_t s = f->ctx->stream;
    if (nrhs == 1) {
      launch_gather(d_b, f->dPerm.as<int>(), f->dBp.as<double>(), n, s);
      f->impl->apply(f->dBp.as<double>(), s);
      launch_scatter_perm(f->dBp.as<double>(), f->dPerm.as<int>(), d_x, n, s);
      RSCHOL_CUDA(cudaStreamSynchronize(s));
      if (f->impl->apply_error(s)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
    } else {   // batches of right-hand sides share one pass over the factor
      const int cap = std::max(1, std::min(64, f->impl->batch_capacity()));
      for (int k0 = 0; k0 < nrhs; k0 += cap) {
        const int k = std::min(cap, nrhs - k0);
        ensure_batch(f, k);
        launch_gather_k(d_b + (size_t)k0 * n, f->dPerm.as<int>(), f->dBk.as<double>(), n, k, s);
        f->impl->apply_batch(f->dBk.as<double>(), k, s);
        launch_scatter_k(f->dBk.as<double>(), f->dPerm.as<int>(), d_x + (size_t)k0 * n, n, k, s);
      }
      RSCHOL_CUDA(cudaStreamSynchronize(s));
      if (f->impl->apply_batch_error(s)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
    }
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

int rschol_precond_apply(rschol_factor* f, const double* b, double* x, int nrhs) {
  if (!f || !b || !x || nrhs <= 0) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    ensure_vecs(f, nrhs);
    const size_t bytes = sizeof(double) * (size_t)f->Afull.n * nrhs;
    RSCHOL_CUDA(cudaMemcpyAsync(f->dB.p, b, bytes, cudaMemcpyHostToDevice, f->ctx->stream));
    int st = rschol_precond_apply_device(f, f->dB.as<double>(), f->dX.as<double>(), nrhs);
    if (st != RSCHOL_OK) return st;
    RSCHOL_CUDA(cudaMemcpyAsync(x, f->dX.p, bytes, cudaMemcpyDeviceToHost, f->ctx->stream));
    RSCHOL_CUDA(cudaStreamSynchronize(f->ctx->stream));
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

int rschol_pcg_device(rschol_factor* f, const double* d_b, double* d_x, int nrhs, double eps, int maxit,
                      rschol_pcg_info* info) {
  if (!f || !d_b || !d_x || nrhs <= 0 || maxit < 0) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  int status = RSCHOL_OK;
  try {
    ensure_vecs(f, 1);
    const int n = f->Afull.n;
    cudaStream_t s = f->ctx->stream;
    Impl* impl = f->impl.get();
    if (nrhs == 1) {
      auto apply = [impl, s](double* w) { impl->apply(w, s); };
      double t0 = now_s();
      launch_gather(d_b, f->dPerm.as<int>(), f->dBp.as<double>(), n, s);
      PcgResult r = f->pcg->solve_graph(f->dBp.as<double>(), f->dXp.as<double>(), eps, maxit, apply, impl->planGen);
      launch_scatter_perm(f->dXp.as<double>(), f->dPerm.as<int>(), d_x, n, s);
      RSCHOL_CUDA(cudaStreamSynchronize(s));
      if (f->impl->apply_error(s)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
      if (info) {
        info[0].iterations = r.iterations;
        info[0].residual = r.residual;
        info[0].true_residual = r.trueResidual;
        info[0].seconds = now_s() - t0;
      }
      if (r.breakdown) status = RSCHOL_E_BREAKDOWN;
    } else {   // batched PCG: up to 64 right-hand sides in lockstep, one factor pass per apply
      const int cap = std::max(1, std::min(64, impl->batch_capacity()));
      for (int k0 = 0; k0 < nrhs; k0 += cap) {
        const int k = std::min(cap, nrhs - k0);
        ensure_batch(f, k);
        double t0 = now_s();
        auto apply = [impl, s, k](double* w) { impl->apply_batch(w, k, s); };
        launch_gather_k(d_b + (size_t)k0 * n, f->dPerm.as<int>(), f->dBk.as<double>(), n, k, s);
        std::vector<PcgResult> rs = f->pcg->solve_batch(f->dBk.as<double>(), f->dXk.as<double>(), k, eps, maxit, apply);
        launch_scatter_k(f->dXk.as<double>(), f->dPerm.as<int>(), d_x + (size_t)k0 * n, n, k, s);
        RSCHOL_CUDA(cudaStreamSynchronize(s));
        if (impl->apply_batch_error(s)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
        const double dt = now_s() - t0;
        for (int c = 0; c < k; ++c) {
          if (info) {
            info[k0 + c].iterations = rs[c].iterations;
            info[k0 + c].residual = rs[c].residual;
            info[k0 + c].true_residual = rs[c].trueResidual;
            info[k0 + c].seconds = dt;
          }
          if (rs[c].breakdown) status = RSCHOL_E_BREAKDOWN;
        }
      }
    }
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  if (status == RSCHOL_E_BREAKDOWN) fail(f->ctx, status, "PCG breakdown: d' A d == 0");
  return status;
}

int rschol_pcg(rschol_factor* f, const double* b, double* x, int nrhs, double eps, int maxit,
               rschol_pcg_info* info) {
  if (!f || !b || !x || nrhs <= 0) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    ensure_vecs(f, nrhs);
    const size_t bytes = sizeof(double) * (size_t)f->Afull.n * nrhs;
    RSCHOL_CUDA(cudaMemcpyAsync(f->dB.p, b, bytes, cudaMemcpyHostToDevice, f->ctx->stream));
    int st = rschol_pcg_device(f, f->dB.as<double>(), f->dX.as<double>(), nrhs, eps, maxit, info);
    RSCHOL_CUDA(cudaMemcpyAsync(x, f->dX.p, bytes, cudaMemcpyDeviceToHost, f->ctx->stream));
    RSCHOL_CUDA(cudaStreamSynchronize(f->ctx->stream));
    return st;
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
}

void rschol_pcg_pysolve(int nrow, const int* jc, const int* ir, const double* pr, const double* rhs,
                        double* solution) {
  rschol_params p;
  rschol_default_params(&p);
  p.reorder_separators = 0;
  rschol_ctx* ctx = rschol_create(&p);
  rschol_factor* f = nullptr;
  int st = rschol_factor_create(ctx, nrow, jc, ir, pr, nullptr, &f);
  if (st == RSCHOL_OK) {
    rschol_pcg_info info;
    st = rschol_pcg(f, rhs, solution, 1, 1e-6, 10000, &info);
    std::printf(" total iterations: %d\n residual: %g\n", info.iterations, info.true_residual);
  }
  if (st != RSCHOL_OK) {
    std::fprintf(stderr, "rschol_pcg_pysolve: %s\n", rschol_last_error(ctx));
    for (int i = 0; i < nrow; ++i) solution[i] = 0.0;
  }
  rschol_factor_free(f);
  rschol_destroy(ctx);
}

int rschol_factor_n(const rschol_factor* f) { return f ? f->Afull.n : 0; }
double rschol_factor_device_bytes(const rschol_factor* f) { return f ? (double)f->devBytes.load() : 0.0; }
int rschol_factor_num_nodes(const rschol_factor* f) { return f ? (int)f->S.nodes.size() : 0; }

int rschol_factor_node_info(const rschol_factor* f, int j, int* info) {
  if (!f || j < 0 || j >= (int)f->S.nodes.size()) return RSCHOL_E_BAD_INPUT;
  const Node& nd = f->S.nodes[j];
  info[0] = nd.c0;
  info[1] = nd.c1;
  info[2] = nd.compressed;
  info[3] = nd.m();
  info[4] = nd.nStored;
  info[5] = nd.compressed && nd.m() > 0 ? f->S.offRank[j] : 0;
  info[6] = (int)nd.H.size();
  info[7] = nd.interior;
  return RSCHOL_OK;
}

int rschol_factor_node_l11(rschol_factor* f, int j, double* out) {
  if (!f || j < 0 || j >= (int)f->S.nodes.size() || !out) return RSCHOL_E_BAD_INPUT;
  try {
    f->impl->node_l11(j, out);
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

int rschol_factor_node_l21(rschol_factor* f, int j, double* out) {
  if (!f || j < 0 || j >= (int)f->S.nodes.size() || !out) return RSCHOL_E_BAD_INPUT;
  try {
    f->impl->node_l21(j, out);
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

int rschol_factor_perm(const rschol_factor* f, int* perm) {
  if (!f || !perm) return RSCHOL_E_BAD_INPUT;
  std::memcpy(perm, f->ord.perm.data(), sizeof(int) * f->Afull.n);
  return RSCHOL_OK;
}

const char* rschol_factor_describe(rschol_factor* f) {
  if (!f) return "{}";
  std::ostringstream o;
  std::string s = describe(f->S);
  s.pop_back();
  o << s << ", \"precision\": \"" << (f->precision == RSCHOL_MIXED ? "mixed" : "fp64") << "\""
    << ", \"root_fp64\": " << ((f->precision == RSCHOL_MIXED && f->prm.root_fp64) ? 1 : 0)
    << ", \"schur_bf16\": " << ((f->precision == RSCHOL_MIXED && f->prm.schur_bf16) ? 1 : 0)
    << ", \"factor_launches\": " << f->impl->launches() << ", \"apply_launches\": " << f->impl->apply_launches()
    << ", \"factor_flops\": " << f->impl->flops() << ", \"apply_bytes\": " << f->impl->apply_bytes()
    << ", \"spmv_bytes\": " << f->pcg->spmvBytes << ", \"device_bytes\": " << f->impl->bytes()
    << ", \"symbolic_s\": " << f->tSymbolic << ", \"plan_s\": " << f->tPlan << ", \"numeric_s\": " << f->tNumeric
    << ", \"attempts\": " << f->attempts << ", \"schedule\": {\"tc_min_k\": "
    << (f->impl->tc_min_k() == INT_MAX ? -1 : f->impl->tc_min_k())
    << ", \"fused\": " << (f->impl->fused_chol() ? "true" : "false") << ", \"tuned_ms\": " << f->tunedMs
    << "}";
  {
    std::vector<double> cb;
    double cf = 0, total = 0;
    f->impl->chol_work(&cb, &cf);
    o << ", \"fused_cholesky\": {\"launches\": " << cb.size() << ", \"flops\": " << cf
      << ", \"algorithmic_bytes_per_launch\": [";
    for (size_t k = 0; k < cb.size(); ++k) {
      o << (k ? ", " : "") << cb[k];
      total += cb[k];
    }
    o << "], \"algorithmic_bytes\": " << total << "}";
  }
  o << ", \"batch_tuning\": [";
  bool first = true;
  for (const auto& row : f->impl->batch_tuning()) {   // per width class: class, RA, RC, cwR, cwC, ms
    o << (first ? "" : ", ") << "[" << row[0] << ", " << row[1] << ", " << row[2] << ", " << row[3] << ", " << row[4]
      << ", " << row[5] << "]";
    first = false;
  }
  o << "]}";
  f->desc = o.str();
  return f->desc.c_str();
}

int rschol_factor_stats(const rschol_factor* f, double* st) {
  if (!f || !st) return RSCHOL_E_BAD_INPUT;
  st[0] = f->tSymbolic;
  st[1] = f->tNumeric;
  st[2] = f->attempts;
  st[3] = f->diagRankConstant;
  st[4] = (double)f->impl->launches();
  st[5] = (double)f->impl->bytes();
  st[6] = (double)f->S.totalDraws;
  st[7] = f->impl->flops();
  return RSCHOL_OK;
}

}  // extern "C"

// ---- diagnostics: per-step-kind device time of the factorisation ------------
extern "C" int rschol_step_timing(rschol_factor* f, int enable, double* out) {
  if (!f) return RSCHOL_E_BAD_INPUT;
  f->impl->step_timing(enable != 0, out);
  return RSCHOL_OK;
}

// ---- diagnostics: the tensor-core GEMM against a host FP64 product -----------
extern "C" int rschol_selftest_gemm(int M, int N, int K, int tA, int tB, int split, int lower, double* out) {
  if (M <= 0 || N <= 0 || K < 0 || !out) return RSCHOL_E_BAD_INPUT;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return RSCHOL_E_NO_DEVICE;
  try {
    const int lda = tA ? M : K, ldb = tB ? K : N, ldc = N;
    const size_t na = (size_t)M * K, nb = (size_t)K * N, nc = (size_t)M * N;
    std::vector<float> A(std::max<size_t>(na, 1)), B(std::max<size_t>(nb, 1)), C(nc), C0(nc);
    uint64_t st = 0x9E3779B97F4A7C15ull;
    auto rnd = [&]() {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      return (float)((double)(st >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0);
    };
    for (auto& x : A) x = rnd();
    for (auto& x : B) x = rnd();
    for (auto& x : C0) x = rnd();
    const float alpha = -1.25f, beta = 0.5f;
    DevBuf dA, dB, dC, dT, dE;
    dA.alloc(sizeof(float) * A.size());
    dB.alloc(sizeof(float) * B.size());
    dC.alloc(sizeof(float) * nc);
    dT.alloc(sizeof(GemmTask<float>));
    dE.alloc(sizeof(int));
    RSCHOL_CUDA(cudaMemcpy(dA.p, A.data(), sizeof(float) * A.size(), cudaMemcpyHostToDevice));
    RSCHOL_CUDA(cudaMemcpy(dB.p, B.data(), sizeof(float) * B.size(), cudaMemcpyHostToDevice));
    RSCHOL_CUDA(cudaMemcpy(dC.p, C0.data(), sizeof(float) * nc, cudaMemcpyHostToDevice));
    RSCHOL_CUDA(cudaMemset(dE.p, 0, sizeof(int)));
    GemmTask<float> t{};
    t.A = dA.as<float>();
    t.B = dB.as<float>();
    t.C = dC.as<float>();
    t.M = M;
    t.N = N;
    t.K = K;
    t.lda = lda;
    t.ldb = ldb;
    t.ldc = ldc;
    t.tA = tA;
    t.tB = tB;
    t.lower = lower;
    t.alpha = alpha;
    t.beta = beta;
    const int bn = tc_tile_n(N);
    t.bn = bn;
    t.tilesN = (N + bn - 1) / bn;
    t.tileBase = 0;
    t.split = split ? 1 : 0;
    const int bf16 = split == 2;
    // K >= 1024 (and not lower): four K slices through the partial workspace
    const int tilesPer = ((M + 127) / 128) * t.tilesN;
    t.kSplit = 1;
    t.kLen = K;
    DevBuf dW, dIds, dBase;
    if (K >= 1024 && !lower) {
      const int al = bf16 ? 64 : 32;
      t.kLen = ((K + 3) / 4 + al - 1) / al * al;
      t.kSplit = (K + t.kLen - 1) / t.kLen;
      dW.alloc(sizeof(float) * (size_t)t.kSplit * tilesPer * 128 * bn);
      t.ws = dW.as<float>();
    }
    DevBuf dMaps;   // K-major aligned operands of a TF32 launch: TMA staging
    if (!bf16) {
      std::vector<TensorMapBytes> maps;
      if (encode_gemm_tmaps(&t, 1, bn, maps)) {
        dMaps.alloc(maps.size() * sizeof(TensorMapBytes));
        RSCHOL_CUDA(cudaMemcpy(dMaps.p, maps.data(), maps.size() * sizeof(TensorMapBytes), cudaMemcpyHostToDevice));
        t.tmA = dMaps.as<TensorMapBytes>() + 0;
        t.tmB = dMaps.as<TensorMapBytes>() + 1;
      }
    }
    out[2] = t.tmA ? 1.0 : 0.0;
    RSCHOL_CUDA(cudaMemcpy(dT.p, &t, sizeof(t), cudaMemcpyHostToDevice));
    launch_gemm_tc(dT.as<GemmTask<float>>(), 1, tilesPer * t.kSplit, dE.as<int>(), 0, bn, bf16);
    if (t.kSplit > 1) {
      const int id = 0;
      const long long base[2] = {0, (long long)M * N};
      dIds.alloc(sizeof(int));
      dBase.alloc(sizeof(base));
      RSCHOL_CUDA(cudaMemcpy(dIds.p, &id, sizeof(int), cudaMemcpyHostToDevice));
      RSCHOL_CUDA(cudaMemcpy(dBase.p, base, sizeof(base), cudaMemcpyHostToDevice));
      launch_gemm_splitk_reduce(dT.as<GemmTask<float>>(), dIds.as<int>(), 1, dBase.as<long long>(), base[1], 0);
    }
    RSCHOL_CUDA(cudaDeviceSynchronize());
    int err = 0;
    RSCHOL_CUDA(cudaMemcpy(&err, dE.p, sizeof(int), cudaMemcpyDeviceToHost));
    RSCHOL_CUDA(cudaMemcpy(C.data(), dC.p, sizeof(float) * nc, cudaMemcpyDeviceToHost));
    double worst = 0, worstAbs = 0;
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < N; ++j) {
        if (lower && j > i) continue;
        double s = 0, mag = 0;
        for (int k = 0; k < K; ++k) {
          const double a = tA ? A[(size_t)k * lda + i] : A[(size_t)i * lda + k];
          const double b = tB ? B[(size_t)j * ldb + k] : B[(size_t)k * ldb + j];
          s += a * b;
          mag += std::fabs(a * b);
        }
        const double ref = alpha * s + beta * (double)C0[(size_t)i * ldc + j];
        const double scale = std::fabs(alpha) * mag + std::fabs(beta * (double)C0[(size_t)i * ldc + j]);
        const double e = std::fabs((double)C[(size_t)i * ldc + j] - ref);
        worstAbs = std::max(worstAbs, e);
        worst = std::max(worst, scale > 0 ? e / scale : e);
      }
    out[0] = worst;
    out[1] = worstAbs;
    if (err) return RSCHOL_E_TIMEOUT;
  } catch (const std::exception&) {
    return RSCHOL_E_CUDA;
  }
  return RSCHOL_OK;
}

// ---- diagnostics: device time of one tensor-core GEMM launch -----------------
extern "C" int rschol_bench_gemm(int M, int N, int K, int split, int reps, double* ms) {
  if (M <= 0 || N <= 0 || K <= 0 || reps <= 0 || !ms || split < 0 || split > 2) return RSCHOL_E_BAD_INPUT;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return RSCHOL_E_NO_DEVICE;
  try {
    // C (M x N) = A (M x K) B^T (B: N x K), both row-major: the factor's update shape
    DevBuf dA, dB, dC, dT, dE;
    dA.alloc(sizeof(float) * (size_t)M * K);
    dB.alloc(sizeof(float) * (size_t)N * K);
    dC.alloc(sizeof(float) * (size_t)M * N);
    dT.alloc(sizeof(GemmTask<float>));
    dE.alloc(sizeof(int));
    RSCHOL_CUDA(cudaMemset(dA.p, 0, sizeof(float) * (size_t)M * K));
    RSCHOL_CUDA(cudaMemset(dB.p, 0, sizeof(float) * (size_t)N * K));
    RSCHOL_CUDA(cudaMemset(dC.p, 0, sizeof(float) * (size_t)M * N));
    RSCHOL_CUDA(cudaMemset(dE.p, 0, sizeof(int)));
    GemmTask<float> t{};
    t.A = dA.as<float>();
    t.B = dB.as<float>();
    t.C = dC.as<float>();
    t.M = M;
    t.N = N;
    t.K = K;
    t.lda = K;
    t.ldb = K;
    t.ldc = N;
    t.tA = 0;
    t.tB = 1;
    t.alpha = -1.f;
    t.beta = 1.f;
    const int bn = tc_tile_n(N);
    t.bn = bn;
    t.tilesN = (N + bn - 1) / bn;
    t.split = split ? 1 : 0;
    t.kSplit = 1;
    t.kLen = K;
    const int tiles = ((M + 127) / 128) * t.tilesN;
    DevBuf dMaps;
    if (split != 2) {
      std::vector<TensorMapBytes> maps;
      if (encode_gemm_tmaps(&t, 1, bn, maps)) {
        dMaps.alloc(maps.size() * sizeof(TensorMapBytes));
        RSCHOL_CUDA(cudaMemcpy(dMaps.p, maps.data(), maps.size() * sizeof(TensorMapBytes), cudaMemcpyHostToDevice));
        t.tmA = dMaps.as<TensorMapBytes>() + 0;
        t.tmB = dMaps.as<TensorMapBytes>() + 1;
      }
    }
    RSCHOL_CUDA(cudaMemcpy(dT.p, &t, sizeof(t), cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    RSCHOL_CUDA(cudaEventCreate(&e0));
    RSCHOL_CUDA(cudaEventCreate(&e1));
    launch_gemm_tc(dT.as<GemmTask<float>>(), 1, tiles, dE.as<int>(), 0, bn, split == 2);   // warm-up
    RSCHOL_CUDA(cudaEventRecord(e0, 0));
    for (int r = 0; r < reps; ++r) launch_gemm_tc(dT.as<GemmTask<float>>(), 1, tiles, dE.as<int>(), 0, bn, split == 2);
    RSCHOL_CUDA(cudaEventRecord(e1, 0));
    RSCHOL_CUDA(cudaEventSynchronize(e1));
    float t_ms = 0;
    RSCHOL_CUDA(cudaEventElapsedTime(&t_ms, e0, e1));
    RSCHOL_CUDA(cudaEventDestroy(e0));
    RSCHOL_CUDA(cudaEventDestroy(e1));
    int err = 0;
    RSCHOL_CUDA(cudaMemcpy(&err, dE.p, sizeof(int), cudaMemcpyDeviceToHost));
    *ms = t_ms / reps;
    if (err) return RSCHOL_E_TIMEOUT;
  } catch (const std::exception&) {
    return RSCHOL_E_CUDA;
  }
  return RSCHOL_OK;
}

// ---- allocation-free preconditioner apply ----------------------------------
// The permuted work vector lives in a file-scope device array instead of a
// buffer allocated on first use, so the call itself never allocates.  Its
// device address is looked up when a context is created (rschol_create):
// under lazy module loading the lookup loads this file's module, which
// allocates the array, so it must not happen inside the apply.
namespace {
constexpr int kNoAllocMaxN = RSCHOL_NOALLOC_MAX_N;
constexpr int kNoAllocMaxDevices = 64;
__device__ __align__(256) double g_noalloc_work[kNoAllocMaxN];
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};
}  // namespace

static cudaError_t noalloc_lookup(int device, double** addr) {
  *addr = nullptr;
  if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    // the caller (rschol_create) has made `device` current
    void* a = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_work);
    if (e != cudaSuccess) return e;
    g_noalloc_addr[device] = a;
  }
  *addr = static_cast<double*>(g_noalloc_addr[device]);
  return cudaSuccess;
}

extern "C" int rschol_precond_apply_device_noalloc(rschol_factor* f, const double* d_b, double* d_x, int nrhs) {
  if (!f || !d_b || !d_x || nrhs <= 0) return RSCHOL_E_BAD_INPUT;
  const int n = f->Afull.n;
  if (n > kNoAllocMaxN)
    return fail(f->ctx, RSCHOL_E_BAD_INPUT,
                "rschol_precond_apply_device_noalloc: n = " + std::to_string(n) + " exceeds the static work vector (" +
                    std::to_string(kNoAllocMaxN) + " unknowns); use rschol_precond_apply_device");
  double* work = f->ctx->noallocWork;
  if (!work)
    return fail(f->ctx, RSCHOL_E_CUDA,
                "rschol_precond_apply_device_noalloc: the static work vector's address was not found when the "
                "context was created");
  try {
    cudaStream_t s = f->ctx->stream;
    for (int k = 0; k < nrhs; ++k) {
      launch_gather(d_b + (size_t)k * n, f->dPerm.as<int>(), work, n, s);
      f->impl->apply(work, s);
      launch_scatter_perm(work, f->dPerm.as<int>(), d_x + (size_t)k * n, n, s);
    }
    RSCHOL_CUDA(cudaStreamSynchronize(s));
    if (f->impl->apply_error(s)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

// ---- continuous batching: a PCG session on one factor ---------------------
struct rschol_session {
  rschol_factor* f = nullptr;
  std::unique_ptr<PcgSession> ses;
  struct Req {
    int nrhs = 0, remaining = 0;
    bool breakdown = false;
    std::vector<rschol_pcg_info> info;
    double t0 = 0;
  };
  std::map<long long, Req> reqs;
};

extern "C" int rschol_factor_autotune(rschol_factor* f, int max_columns) {
  if (!f || max_columns < 1) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  try {
    f->impl->autotune_batch(std::min(64, max_columns), f->ctx->stream);
    RSCHOL_CUDA(cudaStreamSynchronize(f->ctx->stream));
    if (f->impl->apply_batch_error(f->ctx->stream)) return fail(f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
  } catch (const std::exception& e) {
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

extern "C" int rschol_factor_tune_schedule(rschol_factor* f, int repeats) {
  if (!f || repeats < 1) return RSCHOL_E_BAD_INPUT;
  AccountScope acct(&f->devBytes);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  try {
    cudaStream_t s = f->ctx->stream;
    RSCHOL_CUDA(cudaEventCreate(&e0));
    RSCHOL_CUDA(cudaEventCreate(&e1));
    std::vector<int> ks = {INT_MAX};
    if (f->precision == RSCHOL_MIXED) ks = {32, 64, 96, 128, 256, INT_MAX};
    int bestK = f->impl->tc_min_k();
    bool bestFused = f->impl->fused_chol();
    double best = 1e300;
    for (int k : ks)
      for (bool fused : {true, false}) {
        f->impl->set_schedule(k, fused);
        f->impl->plan();
        // the first run launches directly, the second captures the graph;
        // the timed ones replay it, as every later refactorisation does
        if (f->impl->run() != 0 || f->impl->run() != 0) continue;
        double ms = 0;
        bool ok = true;
        for (int r = 0; r < repeats && ok; ++r) {
          RSCHOL_CUDA(cudaEventRecord(e0, s));
          ok = f->impl->run() == 0;
          RSCHOL_CUDA(cudaEventRecord(e1, s));
          RSCHOL_CUDA(cudaEventSynchronize(e1));
          float t = 0;
          RSCHOL_CUDA(cudaEventElapsedTime(&t, e0, e1));
          ms += t;
        }
        if (ok && ms / repeats < best) {
          best = ms / repeats;
          bestK = k;
          bestFused = fused;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    e0 = e1 = nullptr;
    f->impl->set_schedule(bestK, bestFused);
    f->impl->plan();
    f->tunedMs = best < 1e300 ? best : 0;
  } catch (const std::exception& e) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return fail(f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return numeric_with_retry(f);
}

extern "C" rschol_session* rschol_session_create(rschol_factor* f, int max_columns) {
  if (!f || max_columns < 1 || max_columns > 64) return nullptr;
  AccountScope acct(&f->devBytes);
  try {
    Impl* impl = f->impl.get();
    cudaStream_t s = f->ctx->stream;
    const int k = std::min(max_columns, std::max(1, std::min(64, impl->batch_capacity())));
    std::unique_ptr<rschol_session> out(new rschol_session());
    out->f = f;
    out->ses.reset(new PcgSession(
        *f->pcg, k, f->dPerm.as<int>(), [impl, s](double* w, int kk) { impl->apply_batch(w, kk, s); },
        [impl, s]() { return impl->apply_batch_error(s); },
        [impl]() { return (long long)(impl->planGen << 32) + impl->batch_generation(); }));
    return out.release();
  } catch (const std::exception& e) {
    fail(f->ctx, RSCHOL_E_CUDA, e.what());
    return nullptr;
  }
}

extern "C" int rschol_session_columns(const rschol_session* s) { return s ? s->ses->kmax() : 0; }

extern "C" int rschol_session_add(rschol_session* s, long long tag, int nrhs, const double* b, double* x, double eps,
                                  int maxit) {
  if (!s || !b || !x || nrhs < 1 || maxit < 1 || s->reqs.count(tag)) return RSCHOL_E_BAD_INPUT;
  const int n = s->f->Afull.n;
  rschol_session::Req& r = s->reqs[tag];
  r.nrhs = r.remaining = nrhs;
  r.info.assign(nrhs, rschol_pcg_info{});
  r.t0 = now_s();
  for (int c = 0; c < nrhs; ++c) s->ses->add(tag, c, b + (size_t)c * n, x + (size_t)c * n, eps, maxit);
  return RSCHOL_OK;
}

extern "C" int rschol_session_step(rschol_session* s, long long* done_tags, int* ndone) {
  if (!s || !ndone) return RSCHOL_E_BAD_INPUT;
  *ndone = 0;
  AccountScope acct(&s->f->devBytes);
  try {
    std::vector<PcgSession::Column> fin = s->ses->step();
    const double t = now_s();
    for (const PcgSession::Column& c : fin) {
      rschol_session::Req& r = s->reqs[c.tag];
      rschol_pcg_info& i = r.info[c.col];
      i.iterations = c.iterations;
      i.residual = c.residual;
      i.true_residual = c.trueResidual;
      i.seconds = t - r.t0;
      if (c.breakdown) r.breakdown = true;
      if (--r.remaining == 0 && done_tags) done_tags[(*ndone)++] = c.tag;
    }
  } catch (const WaitTimeout&) {
    return fail(s->f->ctx, RSCHOL_E_TIMEOUT, kSolveWaitMsg);
  } catch (const std::exception& e) {
    return fail(s->f->ctx, RSCHOL_E_CUDA, e.what());
  }
  return RSCHOL_OK;
}

extern "C" int rschol_session_result(rschol_session* s, long long tag, rschol_pcg_info* info) {
  if (!s) return RSCHOL_E_BAD_INPUT;
  auto it = s->reqs.find(tag);
  if (it == s->reqs.end() || it->second.remaining > 0) return RSCHOL_E_BAD_INPUT;
  if (info)
    for (int c = 0; c < it->second.nrhs; ++c) info[c] = it->second.info[c];
  const int st = it->second.breakdown ? RSCHOL_E_BREAKDOWN : RSCHOL_OK;
  s->reqs.erase(it);
  return st;
}

extern "C" int rschol_session_counts(const rschol_session* s, int* active, int* queued) {
  if (!s) return RSCHOL_E_BAD_INPUT;
  if (active) *active = s->ses->active();
  if (queued) *queued = s->ses->queued();
  return RSCHOL_OK;
}

extern "C" void rschol_session_destroy(rschol_session* s) { delete s; }

