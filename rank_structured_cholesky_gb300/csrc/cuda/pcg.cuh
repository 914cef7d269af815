// Preconditioned conjugate gradients on the device (FP64 recurrences).
//
// PCG_SOLVER::solvePCG (src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363):
// x0 = 0, r = b, s = M^{-1} r, d = s, delta = r.s; per iteration
// q = A d (CSR SpMV with the caller's full A), alpha = delta / (d.q) (0 when
// d.q == 0, the reference's breakdown branch), x += alpha d, r -= alpha q,
// s = M^{-1} r, beta = (r.s) / delta, d = s + beta d, stop when
// ||r|| / ||b|| <= eps or after maxit iterations; the true residual
// ||b - A x|| / ||b|| is recomputed at the end.
//
// The whole solve runs in the factor's permuted ordering (A is permuted
// once), so the preconditioner needs no gather/scatter; dot products use a
// two-pass fixed-order reduction, so results are reproducible bit for bit.
#pragma once
#include <cuda_runtime.h>

#include <deque>
#include <functional>
#include <stdexcept>
#include <vector>

#include "common.cuh"

namespace rschol {

struct PcgResult {
  int iterations = 0;
  double residual = 0;
  double trueResidual = 0;
  bool breakdown = false;
};

class PcgEngine {
 public:
  // rowptr/colind/vals: CSR of the permuted full matrix (host).
  PcgEngine(int n, const std::vector<int>& rowptr, const std::vector<int>& colind, const std::vector<double>& vals,
            cudaStream_t s);
  ~PcgEngine();
  void set_values(const std::vector<double>& vals);
  double* values() { return vals_.as<double>(); }
  // d_b, d_x: permuted vectors on the device.  apply: in-place M^{-1}.
  PcgResult solve(const double* d_b, double* d_x, double eps, int maxit,
                  const std::function<void(double*)>& apply);
  // The same solve as one CUDA graph: the prologue, a conditional WHILE
  // node whose body is one iteration (its last kernel decides on the device
  // whether another follows: ||r|| / ||b|| > eps and fewer than maxit
  // iterations), and the true-residual epilogue -- one launch and one
  // read-back per solve instead of a host round trip per iteration.  Built on
  // the first solve for a (d_b, d_x, key) triple and replayed while they stay
  // the same; `key` must change whenever apply's buffers do (a new plan).
  // Same kernels, same order of operations: results are bitwise those of
  // solve().  RSCHOL_PCG_GRAPH=0 makes it call solve().
  PcgResult solve_graph(const double* d_b, double* d_x, double eps, int maxit,
                        const std::function<void(double*)>& apply, unsigned long long key);
  // k right-hand sides at once: B, X are n x k row-major (the k values of a
  // row contiguous), permuted; apply: in-place M^{-1} of such a block.
  // Every column follows the single-vector recurrences and stops on its own
  // (its alpha becomes 0 once ||r||/||b|| <= eps); results per column.
  std::vector<PcgResult> solve_batch(const double* d_B, double* d_X, int k, double eps, int maxit,
                                     const std::function<void(double*)>& apply);
  // y = A x on permuted device vectors
  void spmv(const double* x, double* y);
  long long launches = 0;
  double spmvBytes = 0;    // algorithmic bytes of one SpMV
  int n;

 private:
  friend class PcgSession;
  cudaStream_t stream_;
  DevBuf rowptr_, colind_, vals_, r_, d_, q_, s_, part_, scal_;
  double* hScal_ = nullptr;   // pinned
  // the captured solve (solve_graph) and what it was captured for
  void prologue(const double* b, double* x, const std::function<void(double*)>& apply);
  void iteration(double* x, const std::function<void(double*)>& apply);
  void epilogue(const double* b, const double* x);
  void drop_graph();
  cudaGraphExec_t gExec_ = nullptr;
  const double* gB_ = nullptr;
  double* gX_ = nullptr;
  unsigned long long gKey_ = 0;
  long long gPro_ = 0, gBody_ = 0, gEpi_ = 0;   // own kernel launches of the three parts
  DevBuf ctl_;                 // eps, maxit of the current solve (read by the graph's control kernels)
  double* hCtl_ = nullptr;     // pinned
  bool useGraph_ = true;
  int nblk_ = 0;
  int tpr_ = 8;
  // batched solves (allocated for kB_ right-hand sides on first use)
  int kB_ = 0;
  DevBuf rB_, dB_, qB_, sB_, partB_, scalB_;
  double* hScalB_ = nullptr;   // pinned, k x S_COUNT
};

// Continuous batching on one factor (one thread drives a session).  Columns
// are queued by add() and join the block at the next step(); every step()
// advances each active column by one PCG iteration (the reference's
// recurrences, rotated so that a column can join at the preconditioner
// step) and retires the columns that meet their stopping test, writing x to
// the column's host pointer.  Up to kmax columns are active at a time.
struct WaitTimeout : std::runtime_error {
  WaitTimeout() : std::runtime_error("preconditioner solve: a bounded wait gave up") {}
};

class PcgSession {
 public:
  struct Column {
    long long tag = 0;
    int col = 0;
    const double* b = nullptr;   // host, original order, n values
    double* xOut = nullptr;      // host, original order, n values
    double eps = 1e-8;
    int maxit = 0;
    int iterations = 0;
    double residual = 0, trueResidual = 0;
    bool breakdown = false, finished = false;
  };
  // apply(W, k): in-place M^{-1} of an n x k permuted block;
  // applyError(): 0, or non-zero when a wait of the last applies gave up;
  // applyGen(): changes whenever the buffers apply() uses move.
  // The iteration part of a step (apply, dots, SpMV, updates) is captured as
  // a CUDA graph once two consecutive steps have the same width, column block
  // and buffers, and replayed while they stay so (RSCHOL_SESSION_GRAPH=0: every
  // step launches its kernels directly); both run the same kernels.
  PcgSession(PcgEngine& pcg, int kmax, const int* dPerm, std::function<void(double*, int)> apply,
             std::function<int()> applyError, std::function<long long()> applyGen = {});
  ~PcgSession();
  void add(long long tag, int col, const double* b, double* x, double eps, int maxit);
  std::vector<Column> step();
  int active() const {   // retired columns leave the block at the next step
    int a = 0;
    for (const Column& c : cols_) a += c.finished ? 0 : 1;
    return a;
  }
  int queued() const { return (int)queue_.size(); }
  int kmax() const { return kmax_; }
  long long launches = 0;

 private:
  PcgEngine& pcg_;
  int kmax_;
  const int* perm_;
  std::function<void(double*, int)> apply_;
  std::function<int()> applyError_;
  std::function<long long()> applyGen_;
  struct GraphKey {
    int k = -1, set = -1;
    long long gen = -1, apply = -1;
    bool operator==(const GraphKey& o) const { return k == o.k && set == o.set && gen == o.gen && apply == o.apply; }
  };
  bool useGraph_ = true;
  long long gen_ = 0;                 // bumped when the session's own blocks are reallocated
  GraphKey gKey_, lastKey_;
  cudaGraphExec_t gExec_ = nullptr;   // the captured iteration for gKey_
  std::vector<Column> cols_;
  std::deque<Column> queue_;
  DevBuf x_[2], r_[2], d_[2], b_[2], s_, q_, part_, sc_;
  int cap_[2] = {0, 0}, capS_ = 0;   // columns the blocks hold
  int cur_ = 0;
  void reserve_set(int set, int k);
  double* hsc_ = nullptr;   // pinned, per column scalars
  std::vector<double> hscNew_;
};

// permuted <-> original order for k right-hand sides: the stacked vectors
// (column c at src + c n) <-> the n x k row-major block
void launch_gather_k(const double* src, const int* perm, double* dst, int n, int k, cudaStream_t s);
void launch_scatter_k(const double* src, const int* perm, double* dst, int n, int k, cudaStream_t s);

// dst[k] = src[idx[k]], k < count (value re-mapping on the device)
void launch_index_gather(const double* src, const int* idx, double* dst, long long count, cudaStream_t s);
// permuted <-> original order, nrhs = 1
void launch_gather(const double* src, const int* perm, double* dst, int n, cudaStream_t s);
void launch_scatter_perm(const double* src, const int* perm, double* dst, int n, cudaStream_t s);

}  // namespace rschol
