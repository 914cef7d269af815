// Symbolic structure of the rank-structured factor (host side).
//
// Restates FactorManager::factorSymbolic (src/rschol/solver/
// FactorManager.cpp:280-350) for the IN_PLACE / interior-block
// configuration selected by the reference's driver:
//   * Supernode::BuildBasicFactor / BuildOffDiagonalInteractions
//     (src/rschol/node/Supernode.cpp:7070, 6500, 11771-11967): the row
//     structure of every supernode and its grouping into interactions with
//     ancestor supernodes;
//   * Supernode::setDiagonalBlocks + DiagonalBlock::init / buildTraversal /
//     buildBlockList (Supernode.cpp:3897-3951, DiagonalBlock.cpp:92-173,
//     735-795): the HODLR tree of each supernode's diagonal block, its
//     EXPLICIT / RECURSIVE build types and the block processing order;
//   * Supernode::addNodeAppend with IN_PLACE (Supernode.cpp:12120-12249):
//     every interaction of a compressed node is a compressed interaction;
//   * FactorManager::identifyInteriorBlocks (FactorManager.cpp:9977-10045):
//     maximal runs of uncompressed supernodes; their interactions with
//     supernodes outside the run become implicit (not stored);
//   * the fixed-rank policy blockRank / diagonalBlockRank
//     (FactorManager.cpp:7283-7338) and the order in which the
//     factorisation draws Gaussian sketch matrices from the reseeded
//     generator (FactorManager.cpp:384, 8221; DiagonalBlock.cpp:1440).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "ordering.h"

namespace rschol {

struct HNode {                 // DiagonalBlock::BlockNode
  int r0 = 0, r1 = -1;         // full block range, relative to the supernode
  int left = -1, right = -1, parent = -1;
  bool explicitBuild = false;  // _buildType == EXPLICIT_BUILD
  bool isLeaf() const { return left < 0; }
  // internal node: off-diagonal block rows = right child range,
  // columns = left child range
};

struct BlockEntry {            // DiagonalBlock::BlockEntry
  int h = 0;
  bool diag = false;
  bool expl = false;
};

struct Node {
  int c0 = 0, c1 = -1, n = 0;
  bool compressed = false;
  std::vector<int> rows;       // all off-diagonal rows (permuted), ascending
  std::vector<int> interNode;  // ancestor supernode of each interaction
  std::vector<int> interStart; // interaction k = rows[interStart[k], interStart[k+1])
  int parent = -1;             // supernode of rows[0] (supernodal etree parent)
  int interior = -1;           // interior block index, -1 for compressed nodes
  int nStored = 0;             // explicitly stored rows (prefix of rows)
  std::vector<HNode> H;        // HODLR tree of the diagonal
  int hroot = 0;
  std::vector<BlockEntry> blocks;
  bool hasExplicit = false;
  int m() const { return (int)rows.size(); }
};

struct InteriorBlock {
  int n0 = 0, n1 = -1;               // node range (inclusive)
  std::vector<int> ancestors;        // compressed nodes it interacts with, ascending
};

// One contiguous run of Gaussian draws consumed by the factorisation.
struct SketchDraw {
  int node = -1;
  int kind = 0;        // 0: explicit HODLR off-diagonal compress, 1: recursive
                       // HODLR off-diagonal sketch, 2: off-diagonal sketch
  int h = -1;          // HODLR node (kinds 0, 1)
  int rows = 0, rank = 0;
  long long offset = 0;   // first Gaussian of this draw in the stream
};

struct Symbolic {
  int n = 0;
  std::vector<Node> nodes;
  std::vector<int> colNode;            // supernode owning each column
  std::vector<InteriorBlock> interiors;
  std::vector<std::vector<int>> children;  // supernodal etree children
  // Ranks for the current rank constants.
  std::vector<int> offRank;            // per node: off-diagonal rank (0 if none)
  std::vector<std::vector<int>> hRank; // per node, per HODLR node: rank of its off-diagonal block
  std::vector<SketchDraw> draws;
  long long totalDraws = 0;
};

int block_rank(int nRows, int nCols, double c, int oversampling, int cap);

Symbolic build_symbolic(const CSC& Alower, const OrderingResult& ord, const Params& prm);

// Recompute ranks and the Gaussian stream layout for the given rank
// constants (SparseSolver::factorNumeric's retry bumps the diagonal one).
void assign_ranks(Symbolic& S, const Params& prm, double rankConstant, double diagRankConstant);

// Why the device factorisation cannot take this structure ("" when it can):
// an uncompressed supernode wider than max_diag_block has a hierarchical
// diagonal, which only the compressed levels factor on the device.
std::string unsupported_reason(const Symbolic& S, const Params& prm);

std::string describe(const Symbolic& S);

}  // namespace rschol
