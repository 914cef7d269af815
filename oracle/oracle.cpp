// TEST INFRASTRUCTURE (CPU oracle) -- the checker for the GPU library, never
// linked into it and never on its execution path.  Only tests/, the smoke
// check and bench.py's CPU-baseline leg load this file's library.
//
// A plain FP64 CPU restatement of the reference's numeric hot path for the
// configuration its driver selects (CHOLESKY, IN_PLACE, DECOMPOSE_TRANSPOSE,
// DECOMPOSE_FACTOR, fixed rank, COMPRESS_FULL_OFF_DIAGONAL, interior
// blocks on):
//   * FactorManager::factorNumeric  src/rschol/solver/FactorManager.cpp:357-804
//     (left-looking supernodal loop, reseeded generator, retry on
//     IndefiniteDiagonalError as SparseSolver::factorNumeric,
//     src/rschol/solver/SparseSolver.cpp:174-214);
//   * interior-block diagonal updates  FactorManager.cpp:2991-3090;
//   * factorCompressedDiagonal / explicitDiagonalDecomposition /
//     diagonalDecomposition  FactorManager.cpp:8907-9282 and
//     DiagonalBlock.cpp:316-1615 (HODLR diagonal);
//   * the off-diagonal randomized range finder with the implicit operator
//     (blockRandomMultiply_allRows 8193-8297, interactionMultiply_allRows
//     3755-3821, interactionTransMultiply_allRows 4897-4950,
//     interactionMultiply_nodeDescendents 3909-4015,
//     interactionMultiply_blockDescendents 4194-4320,
//     interiorBlockSchurMultiply 10792-10876), the QR, the identity-basis
//     fallback (9539-9638) and the projection V = L21 U (5691-5751);
//   * the solve: FactorPreconditioner::solve (FactorPreconditioner.cpp:
//     135-162), FactorManager::forwardSolve / backwardSolve with
//     interior blocks (6245-6581), Supernode::forwardSolve / backwardSolve;
//   * PCG_SOLVER::solvePCG (src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363).
// The row-oriented interior-block updates of the reference are computed
// here with the equivalent column-oriented sub-solves (same mathematics,
// different rounding order).
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../rank_structured_cholesky_gb300/csrc/host/ordering.h"
#include "../rank_structured_cholesky_gb300/csrc/host/problems.h"
#include "../rank_structured_cholesky_gb300/csrc/host/rng.h"
#include "../rank_structured_cholesky_gb300/csrc/host/symbolic.h"
#include "dense.h"

namespace oracle {

BlasTable g_blas;

using rschol::CSC;
using rschol::HNode;
using rschol::Node;
using rschol::Params;
using rschol::Symbolic;

struct HData {
  std::vector<double> leaf;   // dense lower factor of a leaf (size x size)
  std::vector<double> V, U;   // internal node: rows_b x r, cols_a x r
  int rank = 0;
};

struct Factor {
  Params prm;
  CSC Afull;
  rschol::OrderingResult ord;
  CSC A;   // tril(P A P^T)
  Symbolic S;
  std::vector<std::vector<HData>> hd;      // per node, per HODLR node
  std::vector<std::vector<double>> off;    // interior node stored rows (nStored x n)
  std::vector<std::vector<double>> V, U, UtU;
  std::vector<int> rank;
  std::vector<double> gauss;               // the factorisation's Gaussian stream
  std::vector<std::vector<int>> desc;      // interior descendants per interior node
  std::vector<std::vector<int>> compDesc;  // compressed descendants per compressed node
  std::vector<std::vector<int>> blockDesc; // interior blocks per compressed node
  std::vector<int> rowPos;                 // scratch: global row -> position, -1
  double diagRankConstant = 0.5;
  int attempts = 0;
  double tSymbolic = 0, tNumeric = 0;
  std::string err;
};

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// HODLR diagonal solve (DiagonalBlock::BlockNode::diagonalSolve, left side,
// DiagonalBlock.cpp:1151-1301 and 1306-1378).  X is size x k row-major.
static void hsolve(const Factor& F, int s, int h, double* X, int k, bool trans) {
  const Node& nd = F.S.nodes[s];
  const HNode& x = nd.H[h];
  const HData& d = F.hd[s][h];
  const int size = x.r1 - x.r0 + 1;
  if (x.isLeaf()) {
    trsm_left(size, k, d.leaf.data(), size, trans, X, k);
    return;
  }
  const int d1 = nd.H[x.left].r1 - nd.H[x.left].r0 + 1;
  const int d2 = size - d1;
  double* Y1 = X;
  double* Y2 = X + (size_t)d1 * k;
  std::vector<double> W((size_t)std::max(d.rank, 1) * k);
  if (trans) {
    hsolve(F, s, x.right, Y2, k, trans);
    gemm(d.rank, k, d2, 1.0, d.V.data(), d.rank, true, Y2, k, false, 0.0, W.data(), k);
    gemm(d1, k, d.rank, -1.0, d.U.data(), d.rank, false, W.data(), k, false, 1.0, Y1, k);
    hsolve(F, s, x.left, Y1, k, trans);
  } else {
    hsolve(F, s, x.left, Y1, k, trans);
    gemm(d.rank, k, d1, 1.0, d.U.data(), d.rank, true, Y1, k, false, 0.0, W.data(), k);
    gemm(d2, k, d.rank, -1.0, d.V.data(), d.rank, false, W.data(), k, false, 1.0, Y2, k);
    hsolve(F, s, x.right, Y2, k, trans);
  }
}

// ---------------------------------------------------------------------------
// Interior-block sub-solves over a node list (forwardSubSolve /
// backwardSubSolve, src/rschol/node/Supernode.cpp:5318-5966).  X is the
// stack of the listed nodes' rows (in list order), k columns.
struct NodeList {
  std::vector<int> nodes;
  std::vector<int> start;   // stack offset of each listed node
  int total = 0;
};

static NodeList make_list(const Factor& F, const std::vector<int>& nodes) {
  NodeList L;
  L.nodes = nodes;
  for (int d : nodes) {
    L.start.push_back(L.total);
    L.total += F.S.nodes[d].n;
  }
  return L;
}

// stack row of global column c, or -1 when its node is not listed
static int stack_row(const Factor& F, const NodeList& L, const std::vector<int>& listPos, int c) {
  int d = F.S.colNode[c];
  int q = listPos[d];
  if (q < 0) return -1;
  return L.start[q] + (c - F.S.nodes[d].c0);
}

static void sub_forward(const Factor& F, const NodeList& L, const std::vector<int>& listPos, double* X,
                        int k) {
  std::vector<double> T;
  for (size_t q = 0; q < L.nodes.size(); ++q) {
    int d = L.nodes[q];
    const Node& nd = F.S.nodes[d];
    double* Xd = X + (size_t)L.start[q] * k;
    hsolve(F, d, nd.hroot, Xd, k, false);   // a dense L11 is the HODLR root leaf
    if (nd.nStored == 0) continue;
    T.assign((size_t)nd.nStored * k, 0.0);
    gemm(nd.nStored, k, nd.n, 1.0, F.off[d].data(), nd.n, false, Xd, k, false, 0.0, T.data(), k);
    for (int r = 0; r < nd.nStored; ++r) {
      int sr = stack_row(F, L, listPos, nd.rows[r]);
      if (sr < 0) continue;
      double* dst = X + (size_t)sr * k;
      for (int c = 0; c < k; ++c) dst[c] -= T[(size_t)r * k + c];
    }
  }
}

static void sub_backward(const Factor& F, const NodeList& L, const std::vector<int>& listPos, double* X,
                         int k) {
  std::vector<double> G;
  for (int q = (int)L.nodes.size() - 1; q >= 0; --q) {
    int d = L.nodes[q];
    const Node& nd = F.S.nodes[d];
    double* Xd = X + (size_t)L.start[q] * k;
    if (nd.nStored > 0) {
      G.assign((size_t)nd.nStored * k, 0.0);
      for (int r = 0; r < nd.nStored; ++r) {
        int sr = stack_row(F, L, listPos, nd.rows[r]);
        if (sr < 0) continue;
        std::memcpy(&G[(size_t)r * k], X + (size_t)sr * k, sizeof(double) * k);
      }
      gemm(nd.n, k, nd.nStored, -1.0, F.off[d].data(), nd.n, true, G.data(), k, false, 1.0, Xd, k);
    }
    hsolve(F, d, nd.hroot, Xd, k, true);
  }
}

static int factor_hodlr(Factor& F, int j, const std::vector<double>& S11);

// ---------------------------------------------------------------------------
// Interior-node numeric factorisation (left-looking within the block).
static int factor_interior(Factor& F, int j) {
  const Node& nd = F.S.nodes[j];
  const int n = nd.n, ns = nd.nStored;
  std::vector<int>& rowPos = F.rowPos;
  for (int r = 0; r < nd.m(); ++r) rowPos[nd.rows[r]] = r;
  std::vector<double> D((size_t)n * n, 0.0);
  std::vector<double> O((size_t)ns * n, 0.0);
  // copyMatrixData (Supernode.cpp:284)
  for (int c = nd.c0; c <= nd.c1; ++c)
    for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
      int r = F.A.i[p];
      if (r <= nd.c1) D[(size_t)(r - nd.c0) * n + (c - nd.c0)] = F.A.x[p];
      else if (rowPos[r] < ns) O[(size_t)rowPos[r] * n + (c - nd.c0)] = F.A.x[p];
    }
  // buildUpdateMatrix + applyUpdate (Supernode.cpp:728-824, 947-1114)
  std::vector<double> C;
  for (int d : F.desc[j]) {
    const Node& dn = F.S.nodes[d];
    int q = 0;
    while (dn.interNode[q] != j) ++q;
    const int s0 = dn.interStart[q], s1 = dn.interStart[q + 1];
    const int k1 = s1 - s0, k2 = dn.nStored - s1;
    const double* L1 = F.off[d].data() + (size_t)s0 * dn.n;
    C.assign((size_t)(k1 + k2) * k1, 0.0);
    gemm(k1 + k2, k1, dn.n, 1.0, L1, dn.n, false, L1, dn.n, true, 0.0, C.data(), k1);
    for (int a = 0; a < k1; ++a) {
      int ra = dn.rows[s0 + a] - nd.c0;
      for (int b = 0; b < k1; ++b) D[(size_t)ra * n + (dn.rows[s0 + b] - nd.c0)] -= C[(size_t)a * k1 + b];
    }
    for (int a = 0; a < k2; ++a) {
      int ra = rowPos[dn.rows[s1 + a]];
      for (int b = 0; b < k1; ++b) O[(size_t)ra * n + (dn.rows[s0 + b] - nd.c0)] -= C[(size_t)(k1 + a) * k1 + b];
    }
  }
  for (int r = 0; r < nd.m(); ++r) rowPos[nd.rows[r]] = -1;
  if (nd.H.size() > 1) {
    // A hierarchical diagonal (an uncompressed supernode wider than
    // max_diag_block): the compressed supernodes' block-list walk over the
    // explicit Schur complement D, then the stored rows solved with the
    // expanded L11, L21 = S21 L11^-T (choleskyOffDiagonalSolve through
    // diagonalSolve, Supernode.cpp:3700-3760).
    const int info = factor_hodlr(F, j, D);
    if (info != 0) return info;
    if (ns > 0) {
      std::vector<double> X((size_t)n * ns);
      for (int r = 0; r < ns; ++r)
        for (int c = 0; c < n; ++c) X[(size_t)c * ns + r] = O[(size_t)r * n + c];
      hsolve(F, j, nd.hroot, X.data(), ns, false);
      for (int r = 0; r < ns; ++r)
        for (int c = 0; c < n; ++c) O[(size_t)r * n + c] = X[(size_t)c * ns + r];
    }
    F.off[j].swap(O);
    return 0;
  }
  int info = potrf(n, D.data(), n);
  if (info != 0) return info;
  trsm_right_lt(ns, n, D.data(), n, O.data(), n);
  F.hd[j][nd.hroot].leaf.swap(D);
  F.off[j].swap(O);
  return 0;
}

// ---------------------------------------------------------------------------
// Compressed-node numeric factorisation.
struct CompressedCtx {
  Factor* F;
  int j;
  std::vector<double> S11;          // n x n Schur complement of the diagonal
  // per interior block: node lists
};

// Nodes of interior block b interacting with compressed node j (or with
// any node from j onwards when fromOnwards).
static std::vector<int> block_nodes(const Factor& F, int b, int j, bool fromOnwards) {
  std::vector<int> out;
  const rschol::InteriorBlock& ib = F.S.interiors[b];
  for (int d = ib.n0; d <= ib.n1; ++d) {
    const Node& dn = F.S.nodes[d];
    for (int a : dn.interNode)
      if (a == j || (fromOnwards && a > j)) { out.push_back(d); break; }
  }
  return out;
}

// out (stack of L) += A_{S,cols} * X where X rows are indexed by colMap.
// colPos maps a global row of A (a column of the target node) to the row of X.
static void sparse_S_times(const Factor& F, const NodeList& L, const std::vector<int>& rowMap, const double* X,
                           int k, double* out) {
  for (size_t q = 0; q < L.nodes.size(); ++q) {
    const Node& dn = F.S.nodes[L.nodes[q]];
    for (int c = dn.c0; c <= dn.c1; ++c) {
      double* o = out + (size_t)(L.start[q] + c - dn.c0) * k;
      for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
        int xr = rowMap[F.A.i[p]];
        if (xr < 0) continue;
        const double a = F.A.x[p];
        const double* x = X + (size_t)xr * k;
        for (int t = 0; t < k; ++t) o[t] += a * x[t];
      }
    }
  }
}

// out (rows indexed by rowMap) += alpha * A_{rows,S} * W (W a stack of L).
static void sparse_times_S(const Factor& F, const NodeList& L, const std::vector<int>& rowMap, const double* W,
                           int k, double alpha, double* out) {
  for (size_t q = 0; q < L.nodes.size(); ++q) {
    const Node& dn = F.S.nodes[L.nodes[q]];
    for (int c = dn.c0; c <= dn.c1; ++c) {
      const double* w = W + (size_t)(L.start[q] + c - dn.c0) * k;
      for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
        int orow = rowMap[F.A.i[p]];
        if (orow < 0) continue;
        const double a = alpha * F.A.x[p];
        double* o = out + (size_t)orow * k;
        for (int t = 0; t < k; ++t) o[t] += a * w[t];
      }
    }
  }
}

struct OpMaps {
  std::vector<int> cMap;   // global row -> row in C (node columns), -1
  std::vector<int> rMap;   // global row -> position in node rows, -1
};

// L21 applied from the left:  out (m x k) = L21 * X  (X is n x k), i.e.
// interactionMultiply_allRows with useFactor (L11^{-T} first).
static void op_L21(Factor& F, int j, const OpMaps& M, const double* Xin, int k, double* out) {
  const Node& nd = F.S.nodes[j];
  const int n = nd.n, m = nd.m();
  std::vector<double> X(Xin, Xin + (size_t)n * k);
  hsolve(F, j, nd.hroot, X.data(), k, true);
  std::fill(out, out + (size_t)m * k, 0.0);
  // baseSystemMultiply: A21 * X
  for (int c = nd.c0; c <= nd.c1; ++c) {
    const double* x = &X[(size_t)(c - nd.c0) * k];
    for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
      int r = M.rMap[F.A.i[p]];
      if (r < 0) continue;
      double a = F.A.x[p];
      for (int t = 0; t < k; ++t) out[(size_t)r * k + t] += a * x[t];
    }
  }
  // compressed descendants: - V_d[R'] (U_d^T U_d) V_d[C]^T X[rowList]
  std::vector<double> Xs, T1, T2, T3;
  for (int d : F.compDesc[j]) {
    const Node& dn = F.S.nodes[d];
    int q = 0;
    while (dn.interNode[q] != j) ++q;
    const int s0 = dn.interStart[q], s1 = dn.interStart[q + 1];
    const int k1 = s1 - s0, k2 = dn.m() - s1, r = F.rank[d];
    if (k2 == 0 || r == 0) continue;
    Xs.assign((size_t)k1 * k, 0.0);
    for (int a = 0; a < k1; ++a)
      std::memcpy(&Xs[(size_t)a * k], &X[(size_t)(dn.rows[s0 + a] - nd.c0) * k], sizeof(double) * k);
    T1.assign((size_t)r * k, 0.0);
    gemm(r, k, k1, 1.0, F.V[d].data() + (size_t)s0 * r, r, true, Xs.data(), k, false, 0.0, T1.data(), k);
    T2.assign((size_t)r * k, 0.0);
    gemm(r, k, r, 1.0, F.UtU[d].data(), r, false, T1.data(), k, false, 0.0, T2.data(), k);
    T3.assign((size_t)k2 * k, 0.0);
    gemm(k2, k, r, 1.0, F.V[d].data() + (size_t)s1 * r, r, false, T2.data(), k, false, 0.0, T3.data(), k);
    for (int a = 0; a < k2; ++a) {
      int rr = M.rMap[dn.rows[s1 + a]];
      for (int t = 0; t < k; ++t) out[(size_t)rr * k + t] -= T3[(size_t)a * k + t];
    }
  }
  // interior blocks: - A_{R,S} L_S^{-T} L_S^{-1} A_{S,C} X
  std::vector<int> listPos(F.S.nodes.size(), -1);
  for (int b : F.blockDesc[j]) {
    const rschol::InteriorBlock& ib = F.S.interiors[b];
    if (ib.ancestors.back() == j) continue;   // j is the block's last interaction
    NodeList L = make_list(F, block_nodes(F, b, j, true));
    if (L.nodes.empty()) continue;
    for (size_t q = 0; q < L.nodes.size(); ++q) listPos[L.nodes[q]] = (int)q;
    std::vector<double> W((size_t)L.total * k, 0.0);
    sparse_S_times(F, L, M.cMap, X.data(), k, W.data());
    sub_forward(F, L, listPos, W.data(), k);
    sub_backward(F, L, listPos, W.data(), k);
    sparse_times_S(F, L, M.rMap, W.data(), k, -1.0, out);
    for (int d : L.nodes) listPos[d] = -1;
  }
}

// out (n x k) = L21^T * G  (G is m x k): interactionTransMultiply_allRows.
static void op_L21t(Factor& F, int j, const OpMaps& M, const double* G, int k, double* out) {
  const Node& nd = F.S.nodes[j];
  const int n = nd.n;
  std::fill(out, out + (size_t)n * k, 0.0);
  // baseSystemTransMultiply_left: A21^T G
  for (int c = nd.c0; c <= nd.c1; ++c) {
    double* o = out + (size_t)(c - nd.c0) * k;
    for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
      int r = M.rMap[F.A.i[p]];
      if (r < 0) continue;
      double a = F.A.x[p];
      for (int t = 0; t < k; ++t) o[t] += a * G[(size_t)r * k + t];
    }
  }
  std::vector<double> Gs, T1, T2, T3;
  for (int d : F.compDesc[j]) {
    const Node& dn = F.S.nodes[d];
    int q = 0;
    while (dn.interNode[q] != j) ++q;
    const int s0 = dn.interStart[q], s1 = dn.interStart[q + 1];
    const int k1 = s1 - s0, k2 = dn.m() - s1, r = F.rank[d];
    if (k2 == 0 || r == 0) continue;
    Gs.assign((size_t)k2 * k, 0.0);
    for (int a = 0; a < k2; ++a)
      std::memcpy(&Gs[(size_t)a * k], &G[(size_t)M.rMap[dn.rows[s1 + a]] * k], sizeof(double) * k);
    T1.assign((size_t)r * k, 0.0);
    gemm(r, k, k2, 1.0, F.V[d].data() + (size_t)s1 * r, r, true, Gs.data(), k, false, 0.0, T1.data(), k);
    T2.assign((size_t)r * k, 0.0);
    gemm(r, k, r, 1.0, F.UtU[d].data(), r, false, T1.data(), k, false, 0.0, T2.data(), k);
    T3.assign((size_t)k1 * k, 0.0);
    gemm(k1, k, r, 1.0, F.V[d].data() + (size_t)s0 * r, r, false, T2.data(), k, false, 0.0, T3.data(), k);
    for (int a = 0; a < k1; ++a) {
      int rr = dn.rows[s0 + a] - nd.c0;
      for (int t = 0; t < k; ++t) out[(size_t)rr * k + t] -= T3[(size_t)a * k + t];
    }
  }
  std::vector<int> listPos(F.S.nodes.size(), -1);
  for (int b : F.blockDesc[j]) {
    const rschol::InteriorBlock& ib = F.S.interiors[b];
    if (ib.ancestors.back() == j) continue;
    NodeList L = make_list(F, block_nodes(F, b, j, true));
    if (L.nodes.empty()) continue;
    for (size_t q = 0; q < L.nodes.size(); ++q) listPos[L.nodes[q]] = (int)q;
    std::vector<double> W((size_t)L.total * k, 0.0);
    sparse_S_times(F, L, M.rMap, G, k, W.data());
    sub_forward(F, L, listPos, W.data(), k);
    sub_backward(F, L, listPos, W.data(), k);
    sparse_times_S(F, L, M.cMap, W.data(), k, -1.0, out);
    for (int d : L.nodes) listPos[d] = -1;
  }
  hsolve(F, j, nd.hroot, out, k, false);
}

// Randomized range finder with one power iteration on an operator given by
// its application from the left (apply: n x k -> m x k) and the transpose.
// Returns U (n x r) and V = op * U (m x r), or the identity basis when r >= n.
static void range_finder(int m, int n, int r, int powerIters, const double* G,
                         const std::function<void(const double*, int, double*)>& apply,
                         const std::function<void(const double*, int, double*)>& applyT,
                         std::vector<double>& V, std::vector<double>& U, int& rankOut) {
  std::vector<double> Y((size_t)n * r), X((size_t)m * r);
  applyT(G, r, Y.data());
  for (int it = 0; it < powerIters; ++it) {
    apply(Y.data(), r, X.data());
    applyT(X.data(), r, Y.data());
  }
  if (r >= n) {
    r = n;
    U.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) U[(size_t)i * n + i] = 1.0;
  } else {
    thin_q(n, r, Y.data());
    U.swap(Y);
  }
  V.assign((size_t)m * r, 0.0);
  apply(U.data(), r, V.data());
  rankOut = r;
}

// factorCompressedDiagonal (FactorManager.cpp:8907-9036): walk node j's
// HODLR block list over its n x n Schur complement S11 (row-major; only the
// lower triangle and the blocks below the diagonal are read).  Used for
// compressed supernodes and for uncompressed supernodes whose diagonal is
// hierarchical (the reference factors every supernode's diagonal through its
// DiagonalBlock, FactorManager.cpp:640-652).  Returns 0 or a POTRF info.
static int factor_hodlr(Factor& F, int j, const std::vector<double>& S11) {
  const Node& nd = F.S.nodes[j];
  const int n = nd.n;
  std::vector<HData>& hd = F.hd[j];
  for (const rschol::BlockEntry& be : nd.blocks) {
    const HNode& x = nd.H[be.h];
    if (be.expl) {
      const int b0 = x.r0, size = x.r1 - x.r0 + 1;
      std::vector<double> Sb((size_t)size * size);
      for (int a = 0; a < size; ++a)
        std::memcpy(&Sb[(size_t)a * size], &S11[(size_t)(b0 + a) * n + b0], sizeof(double) * size);
      int info = potrf(size, Sb.data(), size);
      if (info != 0) return info;
      // BlockNode::compressExplicitBlock (DiagonalBlock.cpp:1384-1613), preorder
      std::function<void(int)> compress = [&](int h) {
        const HNode& y = nd.H[h];
        if (y.isLeaf()) {
          const int sz = y.r1 - y.r0 + 1;
          hd[h].leaf.assign((size_t)sz * sz, 0.0);
          for (int a = 0; a < sz; ++a)
            std::memcpy(&hd[h].leaf[(size_t)a * sz], &Sb[(size_t)(y.r0 - b0 + a) * size + (y.r0 - b0)],
                        sizeof(double) * sz);
          return;
        }
        const HNode& lc = nd.H[y.left];
        const HNode& rc = nd.H[y.right];
        const int rows = rc.r1 - rc.r0 + 1, cols = lc.r1 - lc.r0 + 1;
        const int r = F.S.hRank[j][h];
        const double* Fb = &Sb[(size_t)(rc.r0 - b0) * size + (lc.r0 - b0)];
        const rschol::SketchDraw* dr = nullptr;
        for (const auto& dd : F.S.draws)
          if (dd.node == j && dd.h == h) { dr = &dd; break; }
        const double* G = F.gauss.data() + dr->offset;
        std::vector<double> Y((size_t)cols * r), X((size_t)rows * r);
        gemm(cols, r, rows, 1.0, Fb, size, true, G, r, false, 0.0, Y.data(), r);
        for (int it = 0; it < F.prm.power_iters; ++it) {
          gemm(rows, r, cols, 1.0, Fb, size, false, Y.data(), r, false, 0.0, X.data(), r);
          gemm(cols, r, rows, 1.0, Fb, size, true, X.data(), r, false, 0.0, Y.data(), r);
        }
        thin_q(cols, r, Y.data());
        hd[h].U = Y;
        hd[h].V.assign((size_t)rows * r, 0.0);
        gemm(rows, r, cols, 1.0, Fb, size, false, hd[h].U.data(), r, false, 0.0, hd[h].V.data(), r);
        hd[h].rank = r;
        compress(y.left);
        compress(y.right);
      };
      compress(be.h);
    } else if (be.diag) {
      // updateDiagonal + factorDiagonal (DiagonalBlock.cpp:206-376)
      const int sz = x.r1 - x.r0 + 1;
      std::vector<double> Lb((size_t)sz * sz);
      for (int a = 0; a < sz; ++a)
        std::memcpy(&Lb[(size_t)a * sz], &S11[(size_t)(x.r0 + a) * n + x.r0], sizeof(double) * sz);
      for (int cur = be.h, anc = x.parent; anc >= 0; cur = anc, anc = nd.H[anc].parent) {
        if (nd.H[anc].right != cur) continue;
        const HNode& ac = nd.H[nd.H[anc].left];
        const int ar = hd[anc].rank, acols = ac.r1 - ac.r0 + 1;
        const int base = x.r0 - nd.H[nd.H[anc].right].r0;
        std::vector<double> W((size_t)sz * acols);
        gemm(sz, acols, ar, 1.0, hd[anc].V.data() + (size_t)base * ar, ar, false, hd[anc].U.data(), ar, true, 0.0,
             W.data(), acols);
        gemm(sz, sz, acols, -1.0, W.data(), acols, false, W.data(), acols, true, 1.0, Lb.data(), sz);
      }
      int info = potrf(sz, Lb.data(), sz);
      if (info != 0) return info;
      hd[be.h].leaf.swap(Lb);
    } else {
      // diagonalDecomposition (FactorManager.cpp:8998-9036): implicit sketch
      // of L_ba = (S_ba - ancestor couplings) L_aa^{-T}.
      const HNode& lc = nd.H[x.left];
      const HNode& rc = nd.H[x.right];
      const int rows = rc.r1 - rc.r0 + 1, cols = lc.r1 - lc.r0 + 1;
      const int r = F.S.hRank[j][be.h];
      const rschol::SketchDraw* dr = nullptr;
      for (const auto& dd : F.S.draws)
        if (dd.node == j && dd.h == be.h && dd.kind == 1) { dr = &dd; break; }
      auto Sba = [&](const double* Xin, int k, double* out, bool trans) {
        // trans: out (cols x k) = S'_ba^T Xin (rows x k); else out (rows x k) = S'_ba Xin (cols x k)
        const double* Sp = &S11[(size_t)rc.r0 * n + lc.r0];
        if (trans) gemm(cols, k, rows, 1.0, Sp, n, true, Xin, k, false, 0.0, out, k);
        else gemm(rows, k, cols, 1.0, Sp, n, false, Xin, k, false, 0.0, out, k);
        for (int cur = be.h, anc = x.parent; anc >= 0; cur = anc, anc = nd.H[anc].parent) {
          if (nd.H[anc].right != cur) continue;
          const HNode& ar = nd.H[nd.H[anc].right];
          const int rk = hd[anc].rank;
          const int aRows = nd.H[nd.H[anc].left].r1 - nd.H[nd.H[anc].left].r0 + 1;
          const double* V1 = hd[anc].V.data() + (size_t)(rc.r0 - ar.r0) * rk;
          const double* V2 = hd[anc].V.data() + (size_t)(lc.r0 - ar.r0) * rk;
          std::vector<double> W1((size_t)rk * k), W2((size_t)aRows * k), W3((size_t)rk * k);
          if (trans) {
            gemm(rk, k, rows, 1.0, V1, rk, true, Xin, k, false, 0.0, W1.data(), k);
            gemm(aRows, k, rk, 1.0, hd[anc].U.data(), rk, false, W1.data(), k, false, 0.0, W2.data(), k);
            gemm(rk, k, aRows, 1.0, hd[anc].U.data(), rk, true, W2.data(), k, false, 0.0, W3.data(), k);
            gemm(cols, k, rk, -1.0, V2, rk, false, W3.data(), k, false, 1.0, out, k);
          } else {
            gemm(rk, k, cols, 1.0, V2, rk, true, Xin, k, false, 0.0, W1.data(), k);
            gemm(aRows, k, rk, 1.0, hd[anc].U.data(), rk, false, W1.data(), k, false, 0.0, W2.data(), k);
            gemm(rk, k, aRows, 1.0, hd[anc].U.data(), rk, true, W2.data(), k, false, 0.0, W3.data(), k);
            gemm(rows, k, rk, -1.0, V1, rk, false, W3.data(), k, false, 1.0, out, k);
          }
        }
      };
      auto apply = [&](const double* Xin, int k, double* out) {
        std::vector<double> X(Xin, Xin + (size_t)cols * k);
        hsolve(F, j, x.left, X.data(), k, true);
        Sba(X.data(), k, out, false);
      };
      auto applyT = [&](const double* Gin, int k, double* out) {
        Sba(Gin, k, out, true);
        hsolve(F, j, x.left, out, k, false);
      };
      int rk = r;
      range_finder(rows, cols, r, F.prm.power_iters, F.gauss.data() + dr->offset, apply, applyT, hd[be.h].V,
                   hd[be.h].U, rk);
      hd[be.h].rank = rk;
    }
  }

  return 0;
}

static int factor_compressed(Factor& F, int j) {
  Node& nd = F.S.nodes[j];
  const int n = nd.n, m = nd.m();
  OpMaps M;
  M.cMap.assign(F.S.n, -1);
  M.rMap.assign(F.S.n, -1);
  for (int c = nd.c0; c <= nd.c1; ++c) M.cMap[c] = c - nd.c0;
  for (int r = 0; r < m; ++r) M.rMap[nd.rows[r]] = r;

  // Schur complement of the diagonal: A_CC - compressed descendants
  // (compressedDiagonalUpdate, Supernode.cpp:1266-1414) - interior blocks
  // (applyInteriorBlockDiagonalUpdate, FactorManager.cpp:3003-3090).
  std::vector<double> S11((size_t)n * n, 0.0);
  for (int c = nd.c0; c <= nd.c1; ++c)
    for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
      int r = F.A.i[p];
      if (r <= nd.c1) S11[(size_t)(r - nd.c0) * n + (c - nd.c0)] = F.A.x[p];
    }
  std::vector<double> T1, T2;
  for (int d : F.compDesc[j]) {
    const Node& dn = F.S.nodes[d];
    int q = 0;
    while (dn.interNode[q] != j) ++q;
    const int s0 = dn.interStart[q], k1 = dn.interStart[q + 1] - s0, r = F.rank[d];
    if (r == 0) continue;
    const double* Vc = F.V[d].data() + (size_t)s0 * r;
    T1.assign((size_t)r * k1, 0.0);
    gemm(r, k1, r, 1.0, F.UtU[d].data(), r, false, Vc, r, true, 0.0, T1.data(), k1);
    T2.assign((size_t)k1 * k1, 0.0);
    gemm(k1, k1, r, 1.0, Vc, r, false, T1.data(), k1, false, 0.0, T2.data(), k1);
    for (int a = 0; a < k1; ++a)
      for (int b = 0; b < k1; ++b)
        S11[(size_t)(dn.rows[s0 + a] - nd.c0) * n + (dn.rows[s0 + b] - nd.c0)] -= T2[(size_t)a * k1 + b];
  }
  {
    std::vector<int> listPos(F.S.nodes.size(), -1);
    for (int b : F.blockDesc[j]) {
      NodeList L = make_list(F, block_nodes(F, b, j, false));
      if (L.nodes.empty()) continue;
      for (size_t q = 0; q < L.nodes.size(); ++q) listPos[L.nodes[q]] = (int)q;
      // nonzero columns of A_{S,C}
      std::vector<int> colSel, colOf(n, -1);
      for (size_t q = 0; q < L.nodes.size(); ++q) {
        const Node& dn = F.S.nodes[L.nodes[q]];
        for (int c = dn.c0; c <= dn.c1; ++c)
          for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
            int cc = M.cMap[F.A.i[p]];
            if (cc >= 0 && colOf[cc] < 0) { colOf[cc] = 0; colSel.push_back(cc); }
          }
      }
      std::sort(colSel.begin(), colSel.end());
      const int kk = (int)colSel.size();
      if (kk == 0) { for (int d : L.nodes) listPos[d] = -1; continue; }
      for (int t = 0; t < kk; ++t) colOf[colSel[t]] = t;
      std::vector<double> W((size_t)L.total * kk, 0.0);
      for (size_t q = 0; q < L.nodes.size(); ++q) {
        const Node& dn = F.S.nodes[L.nodes[q]];
        for (int c = dn.c0; c <= dn.c1; ++c)
          for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p) {
            int cc = M.cMap[F.A.i[p]];
            if (cc >= 0) W[(size_t)(L.start[q] + c - dn.c0) * kk + colOf[cc]] += F.A.x[p];
          }
      }
      sub_forward(F, L, listPos, W.data(), kk);
      std::vector<double> WtW((size_t)kk * kk, 0.0);
      gemm(kk, kk, L.total, 1.0, W.data(), kk, true, W.data(), kk, false, 0.0, WtW.data(), kk);
      for (int a = 0; a < kk; ++a)
        for (int b = 0; b < kk; ++b) S11[(size_t)colSel[a] * n + colSel[b]] -= WtW[(size_t)a * kk + b];
      for (int d : L.nodes) listPos[d] = -1;
    }
  }

  // factorCompressedDiagonal: walk the HODLR block list.
  {
    const int info = factor_hodlr(F, j, S11);
    if (info != 0) return info;
  }

  // Off-diagonal compression (offDiagonalDecomposition + fullBasisProject).
  if (m > 0) {
    const int r = F.S.offRank[j];
    const rschol::SketchDraw* dr = nullptr;
    for (const auto& dd : F.S.draws)
      if (dd.node == j && dd.kind == 2) { dr = &dd; break; }
    auto apply = [&](const double* X, int k, double* out) { op_L21(F, j, M, X, k, out); };
    auto applyT = [&](const double* G, int k, double* out) { op_L21t(F, j, M, G, k, out); };
    int rk = r;
    range_finder(m, n, r, F.prm.power_iters, F.gauss.data() + dr->offset, apply, applyT, F.V[j], F.U[j], rk);
    F.rank[j] = rk;
    F.UtU[j].assign((size_t)rk * rk, 0.0);
    gemm(rk, rk, n, 1.0, F.U[j].data(), rk, true, F.U[j].data(), rk, false, 0.0, F.UtU[j].data(), rk);
  }
  return 0;
}

static void build_descendant_lists(Factor& F) {
  const int nn = (int)F.S.nodes.size();
  F.desc.assign(nn, {});
  F.compDesc.assign(nn, {});
  F.blockDesc.assign(nn, {});
  for (int d = 0; d < nn; ++d) {
    const Node& dn = F.S.nodes[d];
    for (size_t q = 0; q < dn.interNode.size(); ++q) {
      int a = dn.interNode[q];
      if (dn.compressed) F.compDesc[a].push_back(d);
      else if (F.S.nodes[a].interior == dn.interior) F.desc[a].push_back(d);
    }
  }
  for (size_t b = 0; b < F.S.interiors.size(); ++b)
    for (int a : F.S.interiors[b].ancestors) F.blockDesc[a].push_back((int)b);
}

static int numeric(Factor& F) {
  const int nn = (int)F.S.nodes.size();
  F.hd.assign(nn, {});
  for (int s = 0; s < nn; ++s) F.hd[s].assign(F.S.nodes[s].H.size(), HData());
  F.off.assign(nn, {});
  F.V.assign(nn, {});
  F.U.assign(nn, {});
  F.UtU.assign(nn, {});
  F.rank.assign(nn, 0);
  F.rowPos.assign(F.S.n, -1);
  // MathUtil::GENERATOR.seed(152) at the start of every numeric factorisation
  rschol::MT19937 gen(F.prm.seed);
  F.gauss.assign((size_t)F.S.totalDraws, 0.0);
  gen.gaussianMatrix(F.S.totalDraws, F.gauss.data());
  for (int j = 0; j < nn; ++j) {
    int info = F.S.nodes[j].compressed ? factor_compressed(F, j) : factor_interior(F, j);
    if (info != 0) return j + 1;
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Preconditioner apply (FactorPreconditioner::solve).
static void apply_precond(Factor& F, const double* b, double* x) {
  const int N = F.S.n;
  std::vector<double> w(N);
  for (int i = 0; i < N; ++i) w[i] = b[F.ord.perm[i]];
  const int nn = (int)F.S.nodes.size();
  std::vector<int> listPos(nn, -1);
  auto block_list = [&](int bi) {
    const rschol::InteriorBlock& ib = F.S.interiors[bi];
    std::vector<int> all;
    for (int d = ib.n0; d <= ib.n1; ++d) all.push_back(d);
    return make_list(F, all);
  };
  // forward
  for (int j = 0; j < nn; ++j) {
    const Node& nd = F.S.nodes[j];
    if (!nd.compressed) {
      const rschol::InteriorBlock& ib = F.S.interiors[nd.interior];
      NodeList L = block_list(nd.interior);
      for (size_t q = 0; q < L.nodes.size(); ++q) listPos[L.nodes[q]] = (int)q;
      const int c0 = F.S.nodes[ib.n0].c0, c1 = F.S.nodes[ib.n1].c1;
      double* y = &w[c0];
      sub_forward(F, L, listPos, y, 1);
      std::vector<double> t(y, y + (c1 - c0 + 1));
      sub_backward(F, L, listPos, t.data(), 1);
      for (int c = c0; c <= c1; ++c)
        for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p)
          if (F.A.i[p] > c1) w[F.A.i[p]] -= F.A.x[p] * t[c - c0];
      for (int d : L.nodes) listPos[d] = -1;
      j = ib.n1;
      continue;
    }
    hsolve(F, j, nd.hroot, &w[nd.c0], 1, false);
    const int r = F.rank[j];
    if (r > 0) {
      std::vector<double> z(r, 0.0);
      gemm(r, 1, nd.n, 1.0, F.U[j].data(), r, true, &w[nd.c0], 1, false, 0.0, z.data(), 1);
      for (int a = 0; a < nd.m(); ++a) {
        double s = 0;
        for (int t = 0; t < r; ++t) s += F.V[j][(size_t)a * r + t] * z[t];
        w[nd.rows[a]] -= s;
      }
    }
  }
  // backward
  for (int j = nn - 1; j >= 0; --j) {
    const Node& nd = F.S.nodes[j];
    if (!nd.compressed) {
      const rschol::InteriorBlock& ib = F.S.interiors[nd.interior];
      NodeList L = block_list(nd.interior);
      for (size_t q = 0; q < L.nodes.size(); ++q) listPos[L.nodes[q]] = (int)q;
      const int c0 = F.S.nodes[ib.n0].c0, c1 = F.S.nodes[ib.n1].c1;
      std::vector<double> t(c1 - c0 + 1, 0.0);
      for (int c = c0; c <= c1; ++c)
        for (int p = F.A.p[c]; p < F.A.p[c + 1]; ++p)
          if (F.A.i[p] > c1) t[c - c0] -= F.A.x[p] * w[F.A.i[p]];
      sub_forward(F, L, listPos, t.data(), 1);
      for (int c = c0; c <= c1; ++c) w[c] += t[c - c0];
      sub_backward(F, L, listPos, &w[c0], 1);
      for (int d : L.nodes) listPos[d] = -1;
      j = ib.n0;
      continue;
    }
    const int r = F.rank[j];
    if (r > 0) {
      std::vector<double> z(r, 0.0);
      for (int a = 0; a < nd.m(); ++a)
        for (int t = 0; t < r; ++t) z[t] += F.V[j][(size_t)a * r + t] * w[nd.rows[a]];
      gemm(nd.n, 1, r, -1.0, F.U[j].data(), r, false, z.data(), 1, false, 1.0, &w[nd.c0], 1);
    }
    hsolve(F, j, nd.hroot, &w[nd.c0], 1, true);
  }
  for (int i = 0; i < N; ++i) x[F.ord.perm[i]] = w[i];
}

static void spmv(const CSC& A, const double* x, double* y) {
  std::fill(y, y + A.n, 0.0);
  for (int c = 0; c < A.n; ++c) {
    double xc = x[c];
    for (int p = A.p[c]; p < A.p[c + 1]; ++p) y[A.i[p]] += A.x[p] * xc;
  }
}

static double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

}  // namespace oracle

// ---------------------------------------------------------------------------
// C interface used by the tests and the CPU baseline.
using oracle::Factor;

extern "C" {

// The synthetic problems of the library (rank_structured_cholesky_gb300/
// csrc/host/problems.cpp, compiled into this oracle too), so that CPU-only
// callers need not load the GPU library to build their inputs.
void* oracle_problem_diffusion(int dim, int nx, int ny, int nz, double sigma, unsigned seed, int nrhs) {
  try {
    return new rschol::Problem(rschol::make_diffusion(dim, nx, ny, nz, sigma, seed, nrhs));
  } catch (const std::exception&) {
    return nullptr;
  }
}

void* oracle_problem_elasticity(int ne, double E, double nu, unsigned seed, int nrhs) {
  try {
    return new rschol::Problem(rschol::make_elasticity(ne, E, nu, seed, nrhs));
  } catch (const std::exception&) {
    return nullptr;
  }
}

// sizes[0..2] = n, nnz, nrhs
void oracle_problem_sizes(const void* p, long long* sizes) {
  const rschol::Problem& P = *(const rschol::Problem*)p;
  sizes[0] = P.n;
  sizes[1] = (long long)P.rowind.size();
  sizes[2] = P.nrhs;
}

void oracle_problem_get(const void* p, int* colptr, int* rowind, double* vals, double* xyz, double* rhs) {
  const rschol::Problem& P = *(const rschol::Problem*)p;
  std::memcpy(colptr, P.colptr.data(), sizeof(int) * P.colptr.size());
  std::memcpy(rowind, P.rowind.data(), sizeof(int) * P.rowind.size());
  std::memcpy(vals, P.vals.data(), sizeof(double) * P.vals.size());
  std::memcpy(xyz, P.xyz.data(), sizeof(double) * P.xyz.size());
  std::memcpy(rhs, P.rhs.data(), sizeof(double) * P.rhs.size());
}

void oracle_problem_free(void* p) { delete (rschol::Problem*)p; }

void oracle_set_blas(void* dgemm, void* dtrsm, void* dpotrf, void* dgeqrf, void* dorgqr) {
  oracle::g_blas.gemm = (oracle::dgemm_t)dgemm;
  oracle::g_blas.trsm = (oracle::dtrsm_t)dtrsm;
  oracle::g_blas.potrf = (oracle::dpotrf_t)dpotrf;
  oracle::g_blas.geqrf = (oracle::dgeqrf_t)dgeqrf;
  oracle::g_blas.orgqr = (oracle::dorgqr_t)dorgqr;
}

// params: max_dense, max_diag, explicit_thr, nd_leaf, oversampling, rank_cap,
// power_iters, reorder, rank_constant, diag_rank_constant
void* oracle_create(int n, const int* colptr, const int* rowind, const double* vals, const double* xyz,
                    const int* iparams, const double* dparams) {
  std::unique_ptr<Factor> F(new Factor());
  try {
    Factor& f = *F;
    f.prm.max_dense_block = iparams[0];
    f.prm.max_diag_block = iparams[1];
    f.prm.explicit_threshold = iparams[2];
    f.prm.nd_leaf = iparams[3];
    f.prm.oversampling = iparams[4];
    f.prm.rank_cap = iparams[5];
    f.prm.power_iters = iparams[6];
    f.prm.reorder_separators = iparams[7];
    f.prm.rank_constant = dparams[0];
    f.prm.diag_rank_constant = dparams[1];
    f.Afull.n = n;
    f.Afull.p.assign(colptr, colptr + n + 1);
    f.Afull.i.assign(rowind, rowind + colptr[n]);
    f.Afull.x.assign(vals, vals + colptr[n]);
    double t0 = oracle::now();
    f.ord = rschol::build_ordering(f.Afull, xyz, f.prm);
    f.A = rschol::permute_lower(f.Afull, f.ord.perm, f.ord.iperm);
    f.S = rschol::build_symbolic(f.A, f.ord, f.prm);
    oracle::build_descendant_lists(f);
    f.tSymbolic = oracle::now() - t0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "oracle_create: %s\n", e.what());
    return nullptr;
  }
  return F.release();
}

void oracle_free(void* h) { delete (Factor*)h; }

// Numeric factorisation with the reference's retry policy
// (SparseSolver.cpp:174-214): an indefinite diagonal factored through a
// DiagonalBlock -- every compressed node's, and an uncompressed node's whose
// diagonal is hierarchical (IndefiniteDiagonalError, DiagonalBlock.cpp:372-376,
// 429-435) -- is retried with a larger diagonal rank constant; a non-positive
// pivot of an uncompressed node's dense diagonal is where the reference aborts
// (Supernode.cpp:3681-3689), so it is returned at once.  Returns 0 or the
// 1-based index of the node whose diagonal was not positive definite.
int oracle_factor(void* h) {
  Factor& F = *(Factor*)h;
  double t0 = oracle::now();
  double dc = F.prm.diag_rank_constant;
  int status = 0;
  F.attempts = 0;
  for (int attempt = 0; attempt < F.prm.max_factor_attempts; ++attempt) {
    rschol::assign_ranks(F.S, F.prm, F.prm.rank_constant, dc);
    F.attempts++;
    status = oracle::numeric(F);
    if (status == 0) break;
    const rschol::Node& bad = F.S.nodes[status - 1];
    if (!bad.compressed && bad.H.size() <= 1) break;
    dc *= F.prm.rank_alpha;
  }
  F.diagRankConstant = dc;
  F.tNumeric = oracle::now() - t0;
  return status;
}

void oracle_apply(void* h, const double* b, double* x, int nrhs) {
  Factor& F = *(Factor*)h;
  for (int k = 0; k < nrhs; ++k) oracle::apply_precond(F, b + (size_t)k * F.S.n, x + (size_t)k * F.S.n);
}

// PCG_SOLVER::solvePCG with x0 = 0.  Returns iterations; writes the final
// recurrence residual and the true residual ||b - Ax|| / ||b||.
int oracle_pcg(void* h, const double* b, double* xout, double eps, int maxit, double* recRes, double* trueRes) {
  Factor& F = *(Factor*)h;
  const int N = F.S.n;
  std::vector<double> x(N, 0.0), r(b, b + N), d(N), q(N), s(N), bb(b, b + N);
  oracle::apply_precond(F, r.data(), d.data());
  double deltaNew = oracle::dot(r, d);
  const double bnorm = std::sqrt(oracle::dot(bb, bb));
  double maxR = 2.0 * eps;
  int i = 0;
  while (i < maxit && maxR > eps) {
    oracle::spmv(F.Afull, d.data(), q.data());
    double alpha = oracle::dot(d, q);
    if (std::fabs(alpha) > 0.0) alpha = deltaNew / alpha;
    for (int k = 0; k < N; ++k) x[k] += alpha * d[k];
    for (int k = 0; k < N; ++k) r[k] -= alpha * q[k];
    oracle::apply_precond(F, r.data(), s.data());
    double deltaOld = deltaNew;
    deltaNew = oracle::dot(r, s);
    double beta = deltaNew / deltaOld;
    for (int k = 0; k < N; ++k) d[k] = s[k] + beta * d[k];
    maxR = std::sqrt(oracle::dot(r, r)) / bnorm;
    ++i;
  }
  oracle::spmv(F.Afull, x.data(), q.data());
  double t = 0;
  for (int k = 0; k < N; ++k) t += (b[k] - q[k]) * (b[k] - q[k]);
  if (recRes) *recRes = maxR;
  if (trueRes) *trueRes = std::sqrt(t) / bnorm;
  if (xout) std::memcpy(xout, x.data(), sizeof(double) * N);
  return i;
}

// --- introspection for parity tests -----------------------------------------
int oracle_num_nodes(void* h) { return (int)((Factor*)h)->S.nodes.size(); }

// info[0..7] = c0, c1, compressed, m, nStored, rank, hodlr nodes, interior block
void oracle_node_info(void* h, int j, int* info) {
  Factor& F = *(Factor*)h;
  const rschol::Node& nd = F.S.nodes[j];
  info[0] = nd.c0;
  info[1] = nd.c1;
  info[2] = nd.compressed;
  info[3] = nd.m();
  info[4] = nd.nStored;
  info[5] = F.rank.empty() ? 0 : F.rank[j];
  info[6] = (int)nd.H.size();
  info[7] = nd.interior;
}

// Dense expanded L11 (n x n, row-major, lower; HODLR blocks as V U^T).
void oracle_node_l11(void* h, int j, double* out) {
  Factor& F = *(Factor*)h;
  const rschol::Node& nd = F.S.nodes[j];
  const int n = nd.n;
  std::fill(out, out + (size_t)n * n, 0.0);
  for (size_t q = 0; q < nd.H.size(); ++q) {
    const rschol::HNode& x = nd.H[q];
    const oracle::HData& d = F.hd[j][q];
    if (x.isLeaf()) {
      const int sz = x.r1 - x.r0 + 1;
      for (int a = 0; a < sz; ++a)
        for (int b = 0; b <= a; ++b) out[(size_t)(x.r0 + a) * n + x.r0 + b] = d.leaf[(size_t)a * sz + b];
    } else {
      const rschol::HNode& lc = nd.H[x.left];
      const rschol::HNode& rc = nd.H[x.right];
      const int rows = rc.r1 - rc.r0 + 1, cols = lc.r1 - lc.r0 + 1;
      oracle::gemm(rows, cols, d.rank, 1.0, d.V.data(), d.rank, false, d.U.data(), d.rank, true, 0.0,
                   out + (size_t)rc.r0 * n + lc.r0, n);
    }
  }
}

// Off-diagonal factor rows: interior node -> stored rows (nStored x n);
// compressed node -> V U^T (m x n).
void oracle_node_l21(void* h, int j, double* out) {
  Factor& F = *(Factor*)h;
  const rschol::Node& nd = F.S.nodes[j];
  if (!nd.compressed) {
    std::memcpy(out, F.off[j].data(), sizeof(double) * F.off[j].size());
    return;
  }
  const int r = F.rank[j];
  if (r == 0) return;
  oracle::gemm(nd.m(), nd.n, r, 1.0, F.V[j].data(), r, false, F.U[j].data(), r, true, 0.0, out, nd.n);
}

void oracle_node_rows(void* h, int j, int* out) {
  Factor& F = *(Factor*)h;
  const rschol::Node& nd = F.S.nodes[j];
  std::memcpy(out, nd.rows.data(), sizeof(int) * nd.rows.size());
}

void oracle_perm(void* h, int* perm) {
  Factor& F = *(Factor*)h;
  std::memcpy(perm, F.ord.perm.data(), sizeof(int) * F.S.n);
}

void oracle_times(void* h, double* t) {
  Factor& F = *(Factor*)h;
  t[0] = F.tSymbolic;
  t[1] = F.tNumeric;
  t[2] = F.attempts;
  t[3] = F.diagRankConstant;
}

// Gaussian stream as drawn by the factorisation (first count values).
void oracle_gaussians(void* h, long long count, double* out) {
  Factor& F = *(Factor*)h;
  rschol::MT19937 gen(F.prm.seed);
  gen.gaussianMatrix(count, out);
}

}  // extern "C"
