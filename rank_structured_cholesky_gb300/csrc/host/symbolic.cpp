#include "symbolic.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <functional>
#include <sstream>
#include <stdexcept>
#include <string>

#include "parallel.h"

namespace rschol {

int block_rank(int nRows, int nCols, double c, int oversampling, int cap) {
  // FactorManager::blockRank / diagonalBlockRank (FactorManager.cpp:7283-7338)
  double nz = std::sqrt((double)std::min(nCols, nRows));
  int bs = (int)(nz * std::log2(nz) * c);
  bs += oversampling;
  bs = std::max(bs, 16);
  bs = std::min(bs, nRows);
  bs = std::min(bs, nCols);
  if (cap > 0) bs = std::min(bs, cap);
  return bs;
}

namespace {

// The row structure of supernode s: the rows of its columns below its
// diagonal block and the rows of its children there, ascending; then its
// interactions (runs of rows owned by one ancestor) and its parent, the owner
// of its first row.  mark[] holds the calling thread's stamps.
void fill_node(Symbolic& S, const CSC& A, int s, const std::vector<int>& kids, std::vector<int>& mark) {
  Node& nd = S.nodes[s];
  std::vector<int> rows;
  for (int c = nd.c0; c <= nd.c1; ++c)
    for (int p = A.p[c]; p < A.p[c + 1]; ++p) {
      int r = A.i[p];
      if (r > nd.c1 && mark[r] != s) { mark[r] = s; rows.push_back(r); }
    }
  for (int ch : kids)
    for (int r : S.nodes[ch].rows)
      if (r > nd.c1 && mark[r] != s) { mark[r] = s; rows.push_back(r); }
  std::sort(rows.begin(), rows.end());
  nd.rows.swap(rows);
  nd.interNode.clear();
  nd.interStart.clear();
  for (int k = 0; k < (int)nd.rows.size(); ++k) {
    int owner = S.colNode[nd.rows[k]];
    if (nd.interNode.empty() || nd.interNode.back() != owner) {
      nd.interNode.push_back(owner);
      nd.interStart.push_back(k);
    }
  }
  nd.interStart.push_back((int)nd.rows.size());
  nd.parent = nd.interNode.empty() ? -1 : nd.interNode[0];
}

// Supernodes in ascending order: the children of s are complete before s.
void fill_rows_serial(Symbolic& S, const CSC& A) {
  const int nn = (int)S.nodes.size();
  S.children.assign(nn, {});
  std::vector<int> mark(A.n, -1);
  for (int s = 0; s < nn; ++s) {
    fill_node(S, A, s, S.children[s], mark);
    if (S.nodes[s].parent >= 0) S.children[S.nodes[s].parent].push_back(s);
  }
}

// The same sets with disjoint subtrees filled concurrently.  The supernodal
// tree is predicted before any row is known: the first row below supernode s
// is the smallest elimination-tree parent of its columns that lies beyond its
// last column (a column's rows below its etree parent are rows of that
// parent), so the parent of s is that row's owner.  Subtrees of the predicted
// tree no larger than 1/(4T) of the columns are filled by T workers, the
// supernodes above them afterwards in ascending order.  Every supernode's
// parent is then checked against the owner of its computed first row: if
// all agree, each supernode received exactly the children the serial
// recursion gives it (by induction in ascending order), so the sets are
// identical to the serial ones; otherwise returns false and the caller fills
// them serially.  Columns permuted within a supernode after the etree was
// computed do not change which supernode owns a column.
bool fill_rows_parallel(Symbolic& S, const CSC& A, const std::vector<int>& etree) {
  const int nn = (int)S.nodes.size();
  const int T = host_threads();
  if (T <= 1 || nn < 64 || A.n < 4096 || (int)etree.size() != A.n) return false;
  std::vector<int> pred(nn, -1);
  for (int s = 0; s < nn; ++s) {
    const Node& nd = S.nodes[s];
    int first = A.n;
    for (int c = nd.c0; c <= nd.c1; ++c)
      if (etree[c] > nd.c1 && etree[c] < first) first = etree[c];
    if (first < A.n) pred[s] = S.colNode[first];
    if (pred[s] >= 0 && pred[s] <= s) return false;
  }
  std::vector<std::vector<int>> kids(nn);
  std::vector<long long> size(nn, 0);
  for (int s = 0; s < nn; ++s) {
    size[s] += S.nodes[s].n;
    if (pred[s] >= 0) {
      kids[pred[s]].push_back(s);
      size[pred[s]] += size[s];
    }
  }
  long long total = 0;
  std::vector<int> stack;
  for (int s = 0; s < nn; ++s)
    if (pred[s] < 0) {
      total += size[s];
      stack.push_back(s);
    }
  const long long target = std::max(1LL, total / (4LL * T));
  std::vector<char> top(nn, 0), isRoot(nn, 0);
  std::vector<int> roots;
  while (!stack.empty()) {
    const int s = stack.back();
    stack.pop_back();
    if (size[s] > target && !kids[s].empty()) {
      top[s] = 1;
      for (int ch : kids[s]) stack.push_back(ch);
    } else {
      isRoot[s] = 1;
      roots.push_back(s);
    }
  }
  // members of each chosen subtree, ascending
  std::vector<int> owner(nn, -1), slot(nn, -1);
  for (int k = 0; k < (int)roots.size(); ++k) slot[roots[k]] = k;
  std::vector<std::vector<int>> members(roots.size());
  for (int s = nn - 1; s >= 0; --s)
    if (isRoot[s]) owner[s] = s;
    else if (!top[s]) owner[s] = owner[pred[s]];
  for (int s = 0; s < nn; ++s)
    if (owner[s] >= 0) members[slot[owner[s]]].push_back(s);
  std::vector<int> queue(roots.size());
  for (size_t k = 0; k < roots.size(); ++k) queue[k] = (int)k;
  std::stable_sort(queue.begin(), queue.end(),
                   [&](int a, int b) { return size[roots[a]] > size[roots[b]]; });
  std::atomic<size_t> next(0);
  run_workers(T, [&](int) {
    std::vector<int> mark(A.n, -1);
    for (size_t q; (q = next.fetch_add(1)) < queue.size();)
      for (int s : members[queue[q]]) fill_node(S, A, s, kids[s], mark);
  });
  std::vector<int> mark(A.n, -1);
  for (int s = 0; s < nn; ++s)
    if (top[s]) fill_node(S, A, s, kids[s], mark);
  for (int s = 0; s < nn; ++s)
    if (S.nodes[s].parent != pred[s]) return false;
  S.children.swap(kids);
  return true;
}

// DiagonalBlock::init + buildTraversal + buildBlockList for one supernode.
void build_hodlr(Node& nd, const std::vector<std::pair<int, int>>& leaves, int explicitThreshold) {
  nd.H.clear();
  nd.blocks.clear();
  std::vector<std::pair<int, int>> L = leaves;
  if (L.empty()) L.push_back({0, nd.n - 1});   // setDiagonalBlocks: one block for IN_PLACE
  std::vector<int> level;
  for (auto& r : L) {
    HNode h;
    h.r0 = r.first;
    h.r1 = r.second;
    nd.H.push_back(h);
    level.push_back((int)nd.H.size() - 1);
  }
  while (level.size() > 1) {
    if (level.size() % 2 != 0)
      throw std::runtime_error("number of diagonal blocks must be a power of two");
    std::vector<int> next;
    for (size_t k = 0; k < level.size() / 2; ++k) {
      HNode h;
      h.left = level[2 * k];
      h.right = level[2 * k + 1];
      h.r0 = nd.H[h.left].r0;
      h.r1 = nd.H[h.right].r1;
      nd.H.push_back(h);
      int id = (int)nd.H.size() - 1;
      nd.H[h.left].parent = id;
      nd.H[h.right].parent = id;
      next.push_back(id);
    }
    level.swap(next);
  }
  nd.hroot = level[0];
  nd.hasExplicit = false;
  const int nLeaves = (int)L.size();
  std::function<void(int, int)> traverse = [&](int h, int thr) {
    HNode& x = nd.H[h];
    int rows = x.r1 - x.r0 + 1;
    if (!x.isLeaf() && rows > thr) traverse(x.left, thr);
    if (rows <= thr) {
      nd.hasExplicit = true;
      nd.H[h].explicitBuild = true;
    }
    nd.blocks.push_back({h, nd.H[h].isLeaf(), nd.H[h].explicitBuild});
    if (!nd.H[h].isLeaf() && rows > thr) traverse(nd.H[h].right, thr);
  };
  if (nLeaves > 1 && explicitThreshold > 0) {
    traverse(nd.hroot, explicitThreshold);
  } else {
    traverse(nd.hroot, -1);   // plain in-order traversal of every block
    nd.hasExplicit = false;
  }
}

}  // namespace

Symbolic build_symbolic(const CSC& A, const OrderingResult& ord, const Params& prm) {
  Symbolic S;
  S.n = A.n;
  const int nn = (int)ord.nodes.size();
  S.nodes.resize(nn);
  S.colNode.assign(A.n, -1);
  for (int s = 0; s < nn; ++s) {
    Node& nd = S.nodes[s];
    nd.c0 = ord.nodes[s].c0;
    nd.c1 = ord.nodes[s].c1;
    nd.n = nd.c1 - nd.c0 + 1;
    nd.compressed = ord.nodes[s].compressed;
    for (int c = nd.c0; c <= nd.c1; ++c) S.colNode[c] = s;
  }
  // Row structure: the system rows of each supernode's columns plus the
  // rows propagated from every supernode below it (findSystemRows +
  // propagateFillIn; propagating to the first ancestor only yields the same
  // sets).  IN_PLACE keeps fill from compressed supernodes.
  if (!fill_rows_parallel(S, A, ord.etree)) fill_rows_serial(S, A);
  // Diagonal blocks.
  for (int s = 0; s < nn; ++s) build_hodlr(S.nodes[s], ord.diagBlocks[s], prm.explicit_threshold);
  // Interior blocks: maximal runs of uncompressed supernodes.
  int s = 0;
  while (s < nn) {
    int e = s;
    while (e < nn && !S.nodes[e].compressed) ++e;
    if (e > s) {
      InteriorBlock ib;
      ib.n0 = s;
      ib.n1 = e - 1;
      std::vector<int> anc;
      for (int k = s; k < e; ++k) {
        Node& nd = S.nodes[k];
        nd.interior = (int)S.interiors.size();
        nd.nStored = 0;
        for (size_t q = 0; q < nd.interNode.size(); ++q) {
          if (nd.interNode[q] <= ib.n1) nd.nStored = nd.interStart[q + 1];
          else anc.push_back(nd.interNode[q]);
        }
      }
      std::sort(anc.begin(), anc.end());
      anc.erase(std::unique(anc.begin(), anc.end()), anc.end());
      ib.ancestors = anc;
      S.interiors.push_back(ib);
      s = e;
    } else {
      S.nodes[s].nStored = 0;   // compressed: every interaction is compressed
      ++s;
    }
  }
  assign_ranks(S, prm, prm.rank_constant, prm.diag_rank_constant);
  return S;
}

void assign_ranks(Symbolic& S, const Params& prm, double rankConstant, double diagRankConstant) {
  // FactorManager constructor clamps both constants to >= RANK_CONSTANT.
  const double rc = std::max(rankConstant, 0.4);
  const double dc = std::max(diagRankConstant, 0.4);
  const int nn = (int)S.nodes.size();
  S.offRank.assign(nn, 0);
  S.hRank.assign(nn, {});
  S.draws.clear();
  long long off = 0;
  for (int s = 0; s < nn; ++s) {
    Node& nd = S.nodes[s];
    S.hRank[s].assign(nd.H.size(), 0);
    for (size_t h = 0; h < nd.H.size(); ++h) {
      const HNode& x = nd.H[h];
      if (x.isLeaf()) continue;
      const HNode& a = nd.H[x.left];
      const HNode& b = nd.H[x.right];
      S.hRank[s][h] = block_rank(b.r1 - b.r0 + 1, a.r1 - a.r0 + 1, dc, prm.oversampling, prm.rank_cap);
    }
    // Block list order: explicit subtrees draw in preorder
    // (BlockNode::compressExplicitBlock), recursive off-diagonal blocks draw
    // once (diagonalBlockRandomMultiply).
    std::function<void(int)> pre = [&](int h) {
      const HNode& x = nd.H[h];
      if (x.isLeaf()) return;
      SketchDraw d;
      d.node = s;
      d.kind = 0;
      d.h = h;
      d.rows = nd.H[x.right].r1 - nd.H[x.right].r0 + 1;
      d.rank = S.hRank[s][h];
      d.offset = off;
      off += (long long)d.rows * d.rank;
      S.draws.push_back(d);
      pre(x.left);
      pre(x.right);
    };
    for (const BlockEntry& be : nd.blocks) {
      if (be.expl) {
        pre(be.h);
      } else if (!be.diag) {
        const HNode& x = nd.H[be.h];
        SketchDraw d;
        d.node = s;
        d.kind = 1;
        d.h = be.h;
        d.rows = nd.H[x.right].r1 - nd.H[x.right].r0 + 1;
        d.rank = S.hRank[s][be.h];
        d.offset = off;
        off += (long long)d.rows * d.rank;
        S.draws.push_back(d);
      }
    }
    if (nd.compressed && nd.m() > 0) {
      int r = block_rank(nd.m(), nd.n, rc, prm.oversampling, prm.rank_cap);
      S.offRank[s] = r;
      SketchDraw d;
      d.node = s;
      d.kind = 2;
      d.rows = nd.m();
      d.rank = r;
      d.offset = off;
      off += (long long)d.rows * d.rank;
      S.draws.push_back(d);
    }
  }
  S.totalDraws = off;
}

std::string unsupported_reason(const Symbolic& S, const Params& prm) {
  for (size_t k = 0; k < S.nodes.size(); ++k) {
    const Node& nd = S.nodes[k];
    if (!nd.compressed && nd.H.size() > 1)
      return "uncompressed supernode " + std::to_string(k) + " has " + std::to_string(nd.n) +
             " columns, more than max_diag_block = " + std::to_string(prm.max_diag_block) +
             ": a hierarchical diagonal on an uncompressed supernode is not supported on the device (raise "
             "max_diag_block to at least " + std::to_string(nd.n) + ")";
  }
  return std::string();
}

std::string describe(const Symbolic& S) {
  std::ostringstream o;
  long long storedL = 0, compressedVU = 0, denseDiag = 0;
  int nComp = 0, maxN = 0, maxM = 0, nH = 0;
  for (size_t s = 0; s < S.nodes.size(); ++s) {
    const Node& nd = S.nodes[s];
    if (nd.compressed) {
      nComp++;
      maxN = std::max(maxN, nd.n);
      maxM = std::max(maxM, nd.m());
      compressedVU += (long long)S.offRank[s] * (nd.m() + nd.n);
      if (nd.H.size() > 1) nH++;
      denseDiag += (long long)nd.n * nd.n;
    } else {
      storedL += (long long)nd.n * (nd.n + nd.nStored);
    }
  }
  o << "{\"n\": " << S.n << ", \"supernodes\": " << S.nodes.size() << ", \"compressed\": " << nComp
    << ", \"hodlr_nodes\": " << nH << ", \"interior_blocks\": " << S.interiors.size()
    << ", \"max_compressed_cols\": " << maxN << ", \"max_compressed_rows\": " << maxM
    << ", \"interior_factor_entries\": " << storedL << ", \"compressed_vu_entries\": " << compressedVU
    << ", \"compressed_diag_entries\": " << denseDiag << ", \"gaussian_draws\": " << S.totalDraws << "}";
  return o.str();
}

}  // namespace rschol
