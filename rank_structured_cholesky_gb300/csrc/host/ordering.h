// Ordering and supernode partition (host side).
//
// Follows NestedDissection::SupernodalNestedDissection
// (src/rschol/ordering/NestedDissection.cpp:352-466):
//   1. nested dissection into a postordered list of components
//      (separators and leaf subdomains) with a parent per component;
//   2. elimination tree and column counts of the permuted upper pattern
//      (CSparse cs_etree / cs_counts with the identity postorder,
//      NestedDissection.cpp:409-429, CSparse_Interface.cpp:224-292);
//   3. BuildRelaxedSupernodes (NestedDissection.cpp:1266-1735);
//   4. ReorderNestedSeparators (NestedDissection.cpp:736-910) with the
//      SeparatorTree kd split (src/rschol/datastructure/SeparatorTree.cpp).
//
// Step 1 substitutes CHOLMOD's METIS-based cholmod_nested_dissection
// (CHOLMOD_Environment.cpp:326-432), which is not available: a geometric
// bisection on the unknowns' coordinates when they are given, otherwise a
// breadth-first level-structure bisection of the matrix graph.  Steps 2-4
// restate the reference's own code paths.
#pragma once
#include <cstdint>
#include <utility>
#include <vector>

namespace rschol {

struct Params {
  int max_dense_block = 200;      // maxDenseBlock (src/pcg_solver.cpp:100-110)
  int max_diag_block = 400;       // maxDiagonalBlock
  int explicit_threshold = 4000;  // Supernode::setDiagonalBlocks threshold (FactorManager.cpp:307-312)
  int nd_leaf = 64;               // nested-dissection leaf size
  double rank_constant = 0.4;     // FactorManager::RANK_CONSTANT
  double diag_rank_constant = 0.5;// FactorManager::DIAGONAL_RANK_CONSTANT
  int oversampling = 5;           // FactorManager::OVER_SAMPLING
  int rank_cap = 0;               // 0: reference heuristic; > 0: cap every rank
  int power_iters = 1;            // FactorManager::POWER_ITERATIONS
  int reorder_separators = 1;     // only honoured when coordinates are given
  int max_factor_attempts = 10;   // SparseSolver::_maxFactorAttempts
  double rank_alpha = 1.25;       // SparseSolver::_rankConstantAlpha
  uint32_t seed = 152;            // MathUtil::GENERATOR reseed in factorNumeric
  int root_fp64 = 0;              // mixed precision: the root separator's dense Cholesky in FP64
  int schur_bf16 = 0;             // mixed precision: split products as BF16 hi/lo instead of TF32
};

struct CSC {
  int n = 0;
  std::vector<int> p, i;
  std::vector<double> x;
};

struct Component {   // one entry of the nested dissection component list
  int size = 0;
  int numChildren = 0;
  int first = 0, last = -1;   // permuted column range
};

struct NodeSpec {
  int c0 = 0, c1 = -1;        // permuted column range (inclusive)
  bool compressed = false;    // _compressOffDiagonal
};

struct OrderingResult {
  std::vector<int> perm;      // perm[new] = old  (SparseSolver::_permutation)
  std::vector<int> iperm;     // iperm[old] = new
  std::vector<Component> comps;
  std::vector<int> compParent;
  std::vector<int> etree;     // elimination tree of the permuted matrix
  std::vector<int> colcount;  // cs_counts column counts
  std::vector<NodeSpec> nodes;
  // Per node, the diagonal block (HODLR leaf) ranges relative to the node's
  // first column; empty when the node has a single dense diagonal block.
  std::vector<std::vector<std::pair<int, int>>> diagBlocks;
};

// Nested dissection.  xyz may be null.
void nested_dissection(const CSC& A, const double* xyz, int ndLeaf,
                       std::vector<int>& perm, std::vector<Component>& comps,
                       std::vector<int>& compParent);

// CSparse-style elimination tree / column counts of the upper pattern C
// (CSC, entries with row < col only, no diagonal), with a given postorder.
std::vector<int> etree_upper(const CSC& C);
std::vector<int> column_counts(const CSC& C, const std::vector<int>& parent,
                               const std::vector<int>& post);

// BuildRelaxedSupernodes restated (nrelax 4/16/48, zrelax .8/.1/.05).
std::vector<NodeSpec> relaxed_supernodes(const std::vector<int>& parent,
                                         const std::vector<int>& colcount,
                                         const std::vector<Component>& comps,
                                         const std::vector<int>& compParent,
                                         int maxBlockSize);

// SeparatorTree restated for one set of points (LONGEST_AXIS split, no
// stored separator, full tree): returns the leaf-to-right point order
// (indices into pts) and the leaf ranges.
void separator_tree(const std::vector<const double*>& pts, int maxLeaf,
                    std::vector<int>& order, std::vector<std::pair<int, int>>& leaves);

OrderingResult build_ordering(const CSC& A, const double* xyz, const Params& prm);

// tril(P A P^T) as CSC with sorted rows (Ordering::reorderMatrix with
// lowerOnly = true, src/rschol/ordering/Ordering.cpp:162).
CSC permute_lower(const CSC& A, const std::vector<int>& perm, const std::vector<int>& iperm);

}  // namespace rschol
