// Preconditioner apply x = (L L^T)^{-1} b with the GPU factor, in the
// permuted ordering (the caller keeps its vectors permuted).
//
// Same operator as FactorPreconditioner::solve -> FactorManager::solveSystem
// (src/rschol/solver/FactorPreconditioner.cpp:135-162,
// FactorManager.cpp:6245-6581, Supernode.cpp:4571-5250): interior nodes use
// their full factor panels (the rows the reference re-derives through
// A_{rest,I} L_I^{-T} L_I^{-1} are stored explicitly), compressed nodes use
// the (HODLR-expanded) dense L11 and the V U^T off-diagonal.
//
// Forward: interior supernodes in one launch, one thread block per
// (supernode, 128-row chunk of L21) taken in level order from a ticket
// counter; each waits (bounded) for its children's chunk blocks, assembles
// their update vectors (extend-add, fixed order) for the supernode's columns
// and its chunk, solves with L11 and forms its chunk of the update vector.
// Compressed levels bottom-up: a gather pass adds each row's fixed-order
// contribution list (interior-root update vectors, u_c = -V_c z_c of
// compressed descendants, formed by a launch after each level); y = X f with
// X = L11^{-1}, formed once per factorisation (inverted 64 x 64 diagonal
// blocks, then recursive doubling X_BA = -X_BB L_BA X_AA with batched GEMMs),
// so the triangular solve becomes a GEMV with no chain of dependent blocks;
// z = U^T y is reduced in fixed order by the last row block to finish.
// Backward mirrors this (s = V^T x_R, g = y - U s, x = X^T g), then the
// interior supernodes top-down in one launch (each waits for its parent's
// solve; chunk blocks form parts of L21^T x_R, the last one to finish sums
// them in fixed order and solves with L11^T).  No atomics touch
// the numbers: results are bitwise reproducible.
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <array>
#include <map>
#include <vector>

#include "factor.cuh"

namespace rschol {

constexpr int SOLVE_RB = 64;   // rows per compressed row block
constexpr int XT_COLS = 256;   // columns per tile of X = L11^{-1} in the apply GEMVs

template <class T>
struct SNode {
  const T* L;       // interior: [L11; L21] panel; compressed: L11 (HODLR expanded)
  const T* V;       // compressed: m x r
  const T* U;       // compressed: n x r
  const T* Dinv;    // interior: inverted 64 x 64 diagonal blocks of L11 (the last one h x h)
  const T* X;       // compressed: L11^{-1} (n x n, row-major, upper triangle zero)
  int ld, n, m, r, c0;
  int childBegin, childEnd;   // interior: children (range in the child list)
  int nb, nch;                // compressed: row blocks of L11; both: 128-row chunks of V / L21
  int syncOff;                // compressed: 2 completion counters; interior: backward chunk
                              // counter, forward completion count, backward solved flag
  int parentI;                // interior: parent if it is interior, else -1
  long long rowsOff;          // rows of this node in the row arena
  long long wuOff;            // interior: update vector; compressed: z (r), s (r), u = -V z (m)
  long long relOff;           // interior: target index in the parent front of each row
  long long cOff;             // compressed: first of its n+1 contribution-list offsets
  long long zpOff, spOff;     // compressed: partials of z (nb x r) and s (nch x r);
                              // interior (zpOff): partials of L21^T x_R (nch x n)
  long long zpOff2;           // compressed: tile partials of X f (n x ncb) and X^T g (n x nb)
  int ncb;                    // compressed: 256-column blocks of X
};

struct SPull {       // contribution source of a compressed supernode (plan time)
  int src;           // source node
  int a0, a1;        // source rows mapping into this node's columns
  int kind;          // 0: interior root update vector, 1: compressed V z
};

struct RowBlock {    // one thread block's work: (supernode, row block or chunk)
  int node, b;
};

struct XTile {       // a 64 x 256 tile of X = L11^{-1} (row block ib, column block jb)
  int node, ib, jb;
};

template <class T>
struct DinvTask {    // invert one lower-triangular diagonal block (h x h, h <= 64)
  const T* L;
  int ld, h;
  int pad;           // D is pad x pad, zero outside the h x h lower triangle
  int ldD;           // row stride of D
  T* D;
};

struct XStep {       // one batched GEMM launch (X = L11^{-1} doubling, batched apply)
  long long off;
  int count, tiles;
  int tc;            // on the tensor cores (batched apply: the transposed skinny form)
  int bn = 64;       // tensor-core tile width of the launch (X doubling)
  long long redOff = 0;   // batched apply: K-slice sums after the launch (first, count, grid); tiles = units
  int redCount = 0, redGrid = 0;
};

template <class T>
class SolveEngine {
 public:
  explicit SolveEngine(FactorEngine<T>& F);
  void plan();                           // after the factor plan
  // Queue the solve-side preprocessing of a fresh factor (inverted diagonal
  // blocks); returns its launches.
  int prepare(cudaStream_t s);
  // w (permuted, length n, device) := M^{-1} w, in place.
  void apply_inplace(double* d_w, cudaStream_t s);
  // Reads (synchronously) and clears the error word of the row-block waits:
  // 0, or 1 if a wait gave up (the result of that apply is undefined).
  int take_error(cudaStream_t s);
  // Batched apply: W (n x k, row-major: the k right-hand sides of a row are
  // contiguous) := M^{-1} W with one pass over the factor; k <=
  // batch_capacity().  take_error_batch: as take_error, for the batched path.
  void apply_batch(double* d_W, int k, cudaStream_t s);
  // Time the candidate tile shapes of every width class up to kmax on this
  // stream (run it while the GPU is otherwise quiet) and keep the fastest.
  void autotune_batch(int kmax, cudaStream_t s);
  // the tile shapes chosen for each width class so far: (class, RA, RC, cwR, cwC, ms) rows
  std::vector<std::array<double, 6>> batch_tuning() const;
  int batch_capacity() const;
  // bumped whenever the batched apply's buffers are reallocated or its tile
  // shapes retuned (a graph that captured an apply must then be captured again)
  long long batch_generation() const { return batchGen_; }
  int take_error_batch(cudaStream_t s);
  long long launches_per_apply() const { return launchesPerApply_; }
  double bytes_per_apply() const { return bytesPerApply_; }

 private:
  FactorEngine<T>& F_;
  std::vector<SNode<T>> nodes_;
  DevBuf dNodes_, dRows_, dRel_, dChild_, dWu_, dW_, dLevelNodes_, dCStart_, dCEnt_;
  DevBuf dDinv_, dDinvTasks_, dZp_, dSp_, dIp_, dYi_, dSync_, dTickF_, dIWork_, dIWorkB_;
  int nIWork_ = 0;
  size_t smemIFmax_ = 8, smemIBmax_ = 8;
  // single-vector apply: work lists with the small interior supernodes in
  // groups of eight (a warp each; group members in dSmall_)
  DevBuf dIWorkS_, dIWorkSB_, dSmall_;
  int nIWorkS_ = 0;
  size_t smemWarps_ = 0;
  DevBuf dX_, dT1_, dXGemm_;          // compressed L11^{-1}, its temporaries and GEMM tasks
  DevBuf dXp_, dTiles_;               // tile partials of the X products, tile lists
  std::vector<std::pair<long long, int>> cTiles_;   // per compressed level: (offset, count) of tiles
  std::vector<XStep> xSteps_;
  int nDinv_ = 0;
  int syncInts_ = 0;
  std::vector<long long> tickOff_;   // per compressed level: first ticket entry
  std::vector<int> cBlocks_;         // per compressed level: row blocks
  std::vector<int> cMaxCh_;          // per compressed level: most V chunks of a node
  std::vector<int> cVzGrid_;         // per compressed level: row blocks of the u = -V z launch
  std::vector<int> cRowGrid_;        // per compressed level: 8-row blocks of the largest supernode
  std::vector<int> cColGrid_;        // per compressed level: 256-column blocks of the largest supernode
  void plan_inverse(const std::vector<long long>& xOff);   // GEMM schedule of X = L11^{-1}
  std::vector<std::pair<long long, int>> iLevels_;  // (offset, count) into the interior work list
  std::vector<std::pair<long long, int>> cLevels_;  // (offset, count) into the level node list
  std::vector<size_t> smemIF_, smemIB_;
  long long launchesPerApply_ = 0;
  double bytesPerApply_ = 0;
  // batched apply: work buffers sized for the widest k seen (they only grow,
  // so a changing width frees nothing and never synchronises the device);
  // the GEMM task lists are built once per width and kept
  // Tile shapes of the batched apply (none changes any column's arithmetic):
  // the interior (row, column) pair tile RA x RC and the column groups of the
  // two skinny product forms, per width class (k rounded up to a power of
  // two).  Fixed heuristics unless the class was tuned by autotune_batch
  // (or, with RSCHOL_AUTOTUNE=1, on first use).
  struct BatchCfg {
    int ra = 1, rc = 1, cwR = 1, cwC = 1;
    double ms = 0;   // the winning candidate's time (0: not timed)
  };
  BatchCfg heuristic_cfg(int kp) const;
  const BatchCfg& config_for(int k, cudaStream_t s, bool tune);
  int width_class(int k) const;
  void apply_batch_cfg(double* W64, int k, cudaStream_t s, const BatchCfg& c);
  std::map<int, BatchCfg> tuned_;
  bool autotune_ = true;
  void plan_batch(int k, int cwR, int cwC);
  long long wuTotal_ = 0, ipTotal_ = 0;
  int maxNI_ = 0;                      // largest interior supernode width
  std::vector<int> cMRowGrid_;         // per compressed level: 8-row blocks of the largest m
  int kB_ = 0, kAllocB_ = 0;
  long long batchGen_ = 0;
  DevBuf dWuB_, dYB_, dIpB_, dSyncB_, dWB_;
  struct BatchPlan {
    DevBuf tasks, sums, ws;   // GEMM tasks, K-slice sums and their slice products
    std::vector<std::vector<XStep>> steps;   // [6 * level + phase]
  };
  std::map<int, BatchPlan> bPlans_;
  const BatchPlan* bPlan_ = nullptr;
};

}  // namespace rschol
