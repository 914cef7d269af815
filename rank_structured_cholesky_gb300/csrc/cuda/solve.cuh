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
// Forward: interior levels bottom-up, each node assembling its children's
// update vectors (extend-add, fixed order); compressed levels bottom-up,
// each node pulling the interior roots' update vectors and the compressed
// descendants' V z contributions.  Backward: compressed levels top-down,
// then interior levels top-down, each node gathering its rows from the
// already-solved vector.  No atomics: results are bitwise reproducible.
#pragma once
#include <cuda_runtime.h>

#include <stdexcept>
#include <vector>

#include "factor.cuh"

namespace rschol {

template <class T>
struct SNode {
  const T* L;       // interior: [L11; L21] panel; compressed: L11 (HODLR expanded)
  const T* V;       // compressed: m x r
  const T* U;       // compressed: n x r
  int ld, n, m, r, c0;
  int childBegin, childEnd;   // interior: children; compressed: pull list range
  long long rowsOff;          // rows of this node in the row arena
  long long wuOff;            // interior: update vector; compressed: z (r values)
  long long relOff;           // interior: target index in the parent front of each row
};

struct SPull {       // compressed-node forward pull
  int src;           // source node
  int a0, a1;        // source rows mapping into this node's columns
  int kind;          // 0: interior root update vector, 1: compressed V z
};

template <class T>
class SolveEngine {
 public:
  explicit SolveEngine(FactorEngine<T>& F);
  void plan();                           // after the factor plan
  // w (permuted, length n, device) := M^{-1} w, in place.  scratch-free.
  void apply_inplace(double* d_w, cudaStream_t s);
  long long launches_per_apply() const { return launchesPerApply_; }
  double bytes_per_apply() const { return bytesPerApply_; }

 private:
  FactorEngine<T>& F_;
  std::vector<SNode<T>> nodes_;
  DevBuf dNodes_, dRows_, dRel_, dChild_, dPull_, dWu_, dW_, dLevelNodes_;
  std::vector<std::pair<long long, int>> iLevels_, cLevels_;  // (offset, count) into level node list
  std::vector<size_t> smemIF_, smemIB_, smemCF_, smemCB_;
  int maxCompN_ = 0;
  long long launchesPerApply_ = 0;
  double bytesPerApply_ = 0;
};

}  // namespace rschol
