#include "ordering.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <functional>
#include <future>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <string>
#include <cstdlib>

#include "parallel.h"

namespace rschol {

// ---------------------------------------------------------------------------
// Nested dissection (substitute for cholmod_nested_dissection).
// Produces components in postorder (children before parents); within a
// component unknowns keep their original relative order.
// ---------------------------------------------------------------------------
namespace {

struct NDState {
  const CSC* A;
  const double* xyz;
  int leaf;
  std::vector<int> mark;      // scratch: membership stamp
  std::vector<int> level;     // scratch: local index of a vertex in the set being split
  int stamp = 0;
  std::vector<std::vector<int>> compMembers;
  std::vector<int> compParent;
  std::vector<int> compChildren;
};

int new_component(NDState& S, std::vector<int>&& members, int nChildren) {
  S.compMembers.push_back(std::move(members));
  S.compParent.push_back(-1);
  S.compChildren.push_back(nChildren);
  return (int)S.compMembers.size() - 1;
}

// Split by a coordinate plane.  Returns false when the set cannot be split
// geometrically (all points coincide along every axis).
bool geometric_split(NDState& S, const std::vector<int>& set, std::vector<int>& L,
                     std::vector<int>& R, std::vector<int>& sep) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int v : set)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], S.xyz[3 * (size_t)v + d]);
      hi[d] = std::max(hi[d], S.xyz[3 * (size_t)v + d]);
    }
  int axis = 0;
  double best = -1.0;
  for (int d = 0; d < 3; ++d)
    if (hi[d] - lo[d] > best) { best = hi[d] - lo[d]; axis = d; }
  if (!(best > 0.0)) return false;
  // The plane through the median coordinate (the element a full sort would
  // put at size / 2) balances the two sides.
  std::vector<double> all;
  all.reserve(set.size());
  for (int v : set) all.push_back(S.xyz[3 * (size_t)v + axis]);
  std::nth_element(all.begin(), all.begin() + all.size() / 2, all.end());
  const double target = all[all.size() / 2];
  for (int v : set) {
    double c = S.xyz[3 * (size_t)v + axis];
    if (c < target) L.push_back(v);
    else if (c > target) R.push_back(v);
    else sep.push_back(v);
  }
  // Guarantee separation for general geometry: any L-R edge moves its L end
  // into the separator.
  ++S.stamp;
  for (int v : R) S.mark[v] = S.stamp;
  std::vector<int> keepL;
  keepL.reserve(L.size());
  for (int v : L) {
    bool cross = false;
    for (int p = S.A->p[v]; p < S.A->p[v + 1]; ++p)
      if (S.mark[S.A->i[p]] == S.stamp) { cross = true; break; }
    if (cross) sep.push_back(v);
    else keepL.push_back(v);
  }
  L.swap(keepL);
  std::sort(sep.begin(), sep.end());
  return true;
}

// Breadth-first level-structure bisection of the graph induced on set.
void graph_split(NDState& S, const std::vector<int>& set, std::vector<int>& L,
                 std::vector<int>& R, std::vector<int>& sep) {
  ++S.stamp;
  const int inSet = S.stamp;
  for (int v : set) S.mark[v] = inSet;
  auto bfs = [&](int root, std::vector<std::vector<int>>& levels) {
    ++S.stamp;
    const int seen = S.stamp;
    levels.clear();
    levels.push_back({root});
    S.mark[root] = seen;
    while (true) {
      std::vector<int> next;
      for (int v : levels.back())
        for (int p = S.A->p[v]; p < S.A->p[v + 1]; ++p) {
          int w = S.A->i[p];
          if (S.mark[w] == inSet) { S.mark[w] = seen; next.push_back(w); }
        }
      if (next.empty()) break;
      std::sort(next.begin(), next.end());
      levels.push_back(std::move(next));
    }
    // restore membership stamp for the next sweep
    for (auto& lv : levels)
      for (int v : lv) S.mark[v] = inSet;
  };
  std::vector<std::vector<int>> levels;
  bfs(set[0], levels);
  int far = levels.back()[0];
  bfs(far, levels);
  size_t reached = 0;
  for (auto& lv : levels) reached += lv.size();
  // middle level by cumulative count
  size_t half = reached / 2, cum = 0;
  int m = 0;
  for (int l = 0; l < (int)levels.size(); ++l) {
    if (cum + levels[l].size() > half) { m = l; break; }
    cum += levels[l].size();
  }
  ++S.stamp;
  const int used = S.stamp;
  for (int l = 0; l < (int)levels.size(); ++l)
    for (int v : levels[l]) {
      S.mark[v] = used;
      if (l < m) L.push_back(v);
      else if (l == m) sep.push_back(v);
      else R.push_back(v);
    }
  for (int v : set)
    if (S.mark[v] != used) R.push_back(v);
  std::sort(L.begin(), L.end());
  std::sort(R.begin(), R.end());
  std::sort(sep.begin(), sep.end());
}

// ---------------------------------------------------------------------------
// Multilevel vertex-separator bisection for matrices without coordinates
// (the role METIS's node bisection plays inside cholmod_nested_dissection,
// CHOLMOD_Environment.cpp:326-432): heavy-edge-matching coarsening, greedy
// graph-growing bisection of the coarsest graph, Fiduccia-Mattheyses
// refinement of the edge cut at every level on the way back, and a minimum
// vertex cover of the final cut edges (Koenig's theorem) as the separator.
// Deterministic: every choice depends on the graph and vertex order only.
// ---------------------------------------------------------------------------
struct WGraph {   // weighted undirected graph (CSR, no self loops)
  int n = 0;
  std::vector<int> xadj, adj, ew, vw;
  long long totalW = 0;
};

// The subgraph of A induced on set (local index k <-> set[k]).
WGraph induced_graph(NDState& S, const std::vector<int>& set) {
  WGraph G;
  G.n = (int)set.size();
  ++S.stamp;
  const int in = S.stamp;
  for (int k = 0; k < G.n; ++k) {
    S.mark[set[k]] = in;
    S.level[set[k]] = k;
  }
  G.xadj.assign(G.n + 1, 0);
  for (int k = 0; k < G.n; ++k) {
    const int v = set[k];
    int deg = 0;
    for (int p = S.A->p[v]; p < S.A->p[v + 1]; ++p) {
      const int w = S.A->i[p];
      if (w != v && S.mark[w] == in) ++deg;
    }
    G.xadj[k + 1] = G.xadj[k] + deg;
  }
  G.adj.resize(G.xadj[G.n]);
  for (int k = 0; k < G.n; ++k) {
    const int v = set[k];
    int q = G.xadj[k];
    for (int p = S.A->p[v]; p < S.A->p[v + 1]; ++p) {
      const int w = S.A->i[p];
      if (w != v && S.mark[w] == in) G.adj[q++] = S.level[w];
    }
  }
  G.ew.assign(G.adj.size(), 1);
  G.vw.assign(G.n, 1);
  G.totalW = G.n;
  return G;
}

// Heavy-edge matching: each unmatched vertex (in order of increasing
// degree, ties by index) is matched with its unmatched neighbour of heaviest
// edge (ties: lighter vertex, then lower index).  Returns the coarse graph
// and cmap (fine -> coarse).
WGraph coarsen(const WGraph& G, std::vector<int>& cmap) {
  std::vector<int> order(G.n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return G.xadj[a + 1] - G.xadj[a] < G.xadj[b + 1] - G.xadj[b]; });
  std::vector<int> match(G.n, -1);
  for (int v : order) {
    if (match[v] >= 0) continue;
    int best = -1, bw = -1, bvw = 0;
    for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p) {
      const int u = G.adj[p];
      if (match[u] >= 0) continue;
      if (G.ew[p] > bw || (G.ew[p] == bw && (G.vw[u] < bvw || (G.vw[u] == bvw && u < best)))) {
        best = u;
        bw = G.ew[p];
        bvw = G.vw[u];
      }
    }
    if (best >= 0) {
      match[v] = best;
      match[best] = v;
    } else {
      match[v] = v;
    }
  }
  cmap.assign(G.n, -1);
  WGraph C;
  for (int v = 0; v < G.n; ++v) {
    if (cmap[v] >= 0) continue;
    cmap[v] = C.n;
    if (match[v] != v) cmap[match[v]] = C.n;
    ++C.n;
  }
  C.vw.assign(C.n, 0);
  for (int v = 0; v < G.n; ++v) C.vw[cmap[v]] += G.vw[v];
  C.totalW = G.totalW;
  // coarse adjacency: fine vertices grouped by coarse vertex, edges summed
  std::vector<int> first(C.n, -1), second(C.n, -1);
  for (int v = 0; v < G.n; ++v) {
    const int c = cmap[v];
    if (first[c] < 0) first[c] = v;
    else second[c] = v;
  }
  std::vector<int> slot(C.n, -1);
  C.xadj.assign(C.n + 1, 0);
  std::vector<int> nbr, wgt;
  for (int c = 0; c < C.n; ++c) {
    nbr.clear();
    wgt.clear();
    for (int v : {first[c], second[c]}) {
      if (v < 0) continue;
      for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p) {
        const int d = cmap[G.adj[p]];
        if (d == c) continue;
        if (slot[d] < 0) {
          slot[d] = (int)nbr.size();
          nbr.push_back(d);
          wgt.push_back(0);
        }
        wgt[slot[d]] += G.ew[p];
      }
    }
    for (int d : nbr) slot[d] = -1;
    C.adj.insert(C.adj.end(), nbr.begin(), nbr.end());
    C.ew.insert(C.ew.end(), wgt.begin(), wgt.end());
    C.xadj[c + 1] = (int)C.adj.size();
  }
  return C;
}

long long cut_weight(const WGraph& G, const std::vector<char>& part) {
  long long cut = 0;
  for (int v = 0; v < G.n; ++v)
    for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p)
      if (part[v] != part[G.adj[p]]) cut += G.ew[p];
  return cut / 2;
}

// Fiduccia-Mattheyses passes on the edge cut: vertices move, highest gain
// first (ties: lower index), each at most once per pass, while neither side
// grows beyond maxSide; the pass is rolled back to its best prefix.
void fm_refine(const WGraph& G, std::vector<char>& part, long long maxSide, int passes) {
  long long w[2] = {0, 0};
  for (int v = 0; v < G.n; ++v) w[(int)part[v]] += G.vw[v];
  std::vector<long long> gain(G.n);
  std::vector<char> locked(G.n);
  std::vector<int> moves;
  for (int pass = 0; pass < passes; ++pass) {
    for (int v = 0; v < G.n; ++v) {
      long long g = 0;
      for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p) g += part[G.adj[p]] != part[v] ? G.ew[p] : -G.ew[p];
      gain[v] = g;
    }
    std::fill(locked.begin(), locked.end(), 0);
    using Item = std::pair<long long, int>;   // (gain, -vertex): max gain, then lowest index
    std::priority_queue<Item> pq;
    for (int v = 0; v < G.n; ++v) {
      bool boundary = false;
      for (int p = G.xadj[v]; p < G.xadj[v + 1] && !boundary; ++p) boundary = part[G.adj[p]] != part[v];
      if (boundary) pq.push({gain[v], -v});
    }
    moves.clear();
    long long cut = 0, best = 0;   // relative to the pass start
    size_t bestLen = 0;
    long long bestImb = std::llabs(w[0] - w[1]);
    const size_t patience = 64 + (size_t)G.n / 64;
    while (!pq.empty()) {
      const Item it = pq.top();
      pq.pop();
      const int v = -it.second;
      if (locked[v] || it.first != gain[v]) continue;   // moved already, or a stale entry
      const int from = part[v], to = 1 - from;
      if (w[to] + G.vw[v] > maxSide) continue;
      locked[v] = 1;
      part[v] = (char)to;
      w[from] -= G.vw[v];
      w[to] += G.vw[v];
      cut -= gain[v];
      moves.push_back(v);
      for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p) {
        const int u = G.adj[p];
        if (locked[u]) continue;
        gain[u] += part[u] == to ? -2LL * G.ew[p] : 2LL * G.ew[p];
        pq.push({gain[u], -u});
      }
      const long long imb = std::llabs(w[0] - w[1]);
      if (cut < best || (cut == best && imb < bestImb)) {
        best = cut;
        bestLen = moves.size();
        bestImb = imb;
      }
      if (moves.size() - bestLen > patience) break;
    }
    for (size_t k = moves.size(); k > bestLen; --k) {   // roll back past the best prefix
      const int v = moves[k - 1];
      const int from = part[v], to = 1 - from;
      part[v] = (char)to;
      w[from] -= G.vw[v];
      w[to] += G.vw[v];
    }
    if (bestLen == 0) break;
  }
}

// Greedy graph growing: side 0 grows breadth-first from `seed` (continuing
// from the lowest unvisited vertex when a component is exhausted) until it
// holds half the vertex weight.
std::vector<char> grow_bisection(const WGraph& G, int seed) {
  std::vector<char> part(G.n, 1);
  std::vector<char> seen(G.n, 0);
  long long w0 = 0;
  const long long half = G.totalW / 2;
  std::vector<int> queue;
  queue.reserve(G.n);
  size_t head = 0;
  int nextStart = 0;
  queue.push_back(seed);
  seen[seed] = 1;
  while (w0 < half) {
    if (head == queue.size()) {
      while (nextStart < G.n && seen[nextStart]) ++nextStart;
      if (nextStart >= G.n) break;
      queue.push_back(nextStart);
      seen[nextStart] = 1;
    }
    const int v = queue[head++];
    part[v] = 0;
    w0 += G.vw[v];
    for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p) {
      const int u = G.adj[p];
      if (!seen[u]) {
        seen[u] = 1;
        queue.push_back(u);
      }
    }
  }
  return part;
}

// Minimum vertex cover of the cut edges (bipartite: side-0 vs side-1
// boundary vertices) by a maximum matching and Koenig's construction.
std::vector<int> cut_cover(const WGraph& G, const std::vector<char>& part) {
  std::vector<int> mate(G.n, -1);
  std::vector<int> left;   // side-0 boundary vertices
  for (int v = 0; v < G.n; ++v) {
    if (part[v] != 0) continue;
    for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p)
      if (part[G.adj[p]] == 1) { left.push_back(v); break; }
  }
  // augmenting paths (iterative DFS from each free left vertex)
  std::vector<int> visitStamp(G.n, -1), parentL(G.n, -1), iter(G.n, 0);
  for (size_t k = 0; k < left.size(); ++k) {
    const int root = left[k];
    std::vector<int> stack{root};
    iter[root] = G.xadj[root];
    visitStamp[root] = (int)k;
    int freeR = -1;
    while (!stack.empty() && freeR < 0) {
      const int v = stack.back();
      bool pushed = false;
      while (iter[v] < G.xadj[v + 1]) {
        const int u = G.adj[iter[v]++];
        if (part[u] != 1 || visitStamp[u] == (int)k) continue;
        visitStamp[u] = (int)k;
        parentL[u] = v;
        if (mate[u] < 0) { freeR = u; break; }
        const int w = mate[u];
        if (visitStamp[w] == (int)k) continue;
        visitStamp[w] = (int)k;
        iter[w] = G.xadj[w];
        stack.push_back(w);
        pushed = true;
        break;
      }
      if (freeR < 0 && !pushed) stack.pop_back();
    }
    for (int u = freeR; u >= 0;) {   // flip the path
      const int v = parentL[u];
      const int next = mate[v];
      mate[v] = u;
      mate[u] = v;
      u = next;
    }
  }
  // Z: reachable from free left vertices by alternating paths
  std::vector<char> inZ(G.n, 0);
  std::vector<int> stack;
  for (int v : left)
    if (mate[v] < 0) { inZ[v] = 1; stack.push_back(v); }
  while (!stack.empty()) {
    const int v = stack.back();
    stack.pop_back();
    for (int p = G.xadj[v]; p < G.xadj[v + 1]; ++p) {
      const int u = G.adj[p];
      if (part[u] != 1 || inZ[u] || mate[v] == u) continue;
      inZ[u] = 1;
      const int w = mate[u];
      if (w >= 0 && !inZ[w]) { inZ[w] = 1; stack.push_back(w); }
    }
  }
  std::vector<int> cover;
  for (int v = 0; v < G.n; ++v) {
    bool boundary = false;
    for (int p = G.xadj[v]; p < G.xadj[v + 1] && !boundary; ++p) boundary = part[G.adj[p]] != part[v];
    if (!boundary) continue;
    if ((part[v] == 0 && !inZ[v]) || (part[v] == 1 && inZ[v])) cover.push_back(v);
  }
  return cover;
}

bool bfs_nd() {
  static const bool bfs = [] {
    const char* e = std::getenv("RSCHOL_GRAPH_ND");
    return e && std::string(e) == "bfs";
  }();
  return bfs;
}

void multilevel_split(NDState& S, const std::vector<int>& set, std::vector<int>& L, std::vector<int>& R,
                      std::vector<int>& sep) {
  std::vector<WGraph> levels;
  std::vector<std::vector<int>> maps;
  levels.push_back(induced_graph(S, set));
  while (levels.back().n > 120 && levels.size() < 48) {
    std::vector<int> cmap;
    WGraph C = coarsen(levels.back(), cmap);
    if (C.n > (int)(0.92 * levels.back().n)) break;   // matching stalled
    maps.push_back(std::move(cmap));
    levels.push_back(std::move(C));
  }
  auto maxSide = [](const WGraph& G) {
    long long mx = 0;
    for (int w : G.vw) mx = std::max<long long>(mx, w);
    return std::max((long long)std::ceil(0.55 * (double)G.totalW), (G.totalW + 1) / 2 + mx);
  };
  // coarsest level: the best of a few grown bisections
  const WGraph& C = levels.back();
  std::vector<char> part;
  long long bestCut = -1;
  const int seeds[4] = {0, C.n / 3, (2 * C.n) / 3, C.n - 1};
  for (int k = 0; k < 4; ++k) {
    if (k > 0 && seeds[k] == seeds[k - 1]) continue;
    std::vector<char> p = grow_bisection(C, seeds[k]);
    fm_refine(C, p, maxSide(C), 8);
    const long long cut = cut_weight(C, p);
    if (bestCut < 0 || cut < bestCut) {
      bestCut = cut;
      part.swap(p);
    }
  }
  for (int l = (int)levels.size() - 2; l >= 0; --l) {   // project and refine
    std::vector<char> fine(levels[l].n);
    for (int v = 0; v < levels[l].n; ++v) fine[v] = part[maps[l][v]];
    fm_refine(levels[l], fine, maxSide(levels[l]), 4);
    part.swap(fine);
  }
  const WGraph& G = levels.front();
  std::vector<int> cover = cut_cover(G, part);
  std::vector<char> inSep(G.n, 0);
  for (int v : cover) inSep[v] = 1;
  for (int k = 0; k < G.n; ++k) {
    if (inSep[k]) sep.push_back(set[k]);
    else if (part[k] == 0) L.push_back(set[k]);
    else R.push_back(set[k]);
  }
  if (sep.empty() && !L.empty() && !R.empty()) {   // disconnected halves: a one-vertex separator
    sep.push_back(R.back());
    R.pop_back();
  }
  std::sort(L.begin(), L.end());
  std::sort(R.begin(), R.end());
  std::sort(sep.begin(), sep.end());
}

// Split set into L, R and the separator; false: keep it as one component.
bool split(NDState& S, const std::vector<int>& set, std::vector<int>& L, std::vector<int>& R,
           std::vector<int>& sep) {
  if ((int)set.size() <= S.leaf) return false;
  bool ok = false;
  if (S.xyz) ok = geometric_split(S, set, L, R, sep);
  if (!ok) {
    // without coordinates: the level-structure bisection and the multilevel
    // one, keeping the smaller separator (ties: the better balanced split)
    L.clear();
    R.clear();
    sep.clear();
    graph_split(S, set, L, R, sep);
    if (!bfs_nd()) {
      std::vector<int> L2, R2, sep2;
      multilevel_split(S, set, L2, R2, sep2);
      const bool valid = !(sep2.empty() || L2.empty() || R2.empty());
      auto imb = [](const std::vector<int>& a, const std::vector<int>& b) {
        return std::abs((long long)a.size() - (long long)b.size());
      };
      if (valid && (sep2.size() < sep.size() || (sep2.size() == sep.size() && imb(L2, R2) < imb(L, R)))) {
        L.swap(L2);
        R.swap(R2);
        sep.swap(sep2);
      }
    }
  }
  return !(sep.empty() || (L.empty() && R.empty()));
}

int dissect(NDState& S, std::vector<int> set) {
  std::vector<int> L, R, sep;
  if (!split(S, set, L, R, sep)) return new_component(S, std::move(set), 0);
  std::vector<int> kids;
  if (!L.empty()) kids.push_back(dissect(S, std::move(L)));
  if (!R.empty()) kids.push_back(dissect(S, std::move(R)));
  int c = new_component(S, std::move(sep), (int)kids.size());
  for (int k : kids) S.compParent[k] = c;
  return c;
}

// Move the components of a subtree dissected in its own state Sub (root
// subRoot) to the end of S; returns the root's index in S.  The splits do
// not depend on the scratch stamps, so a subtree comes out exactly as the
// serial recursion makes it, and appending L's subtree, then R's, then the
// separator keeps the serial postorder.
int adopt(NDState& S, NDState& Sub, int subRoot) {
  const int base = (int)S.compMembers.size();
  for (size_t k = 0; k < Sub.compMembers.size(); ++k) {
    S.compMembers.push_back(std::move(Sub.compMembers[k]));
    S.compParent.push_back(Sub.compParent[k] >= 0 ? Sub.compParent[k] + base : -1);
    S.compChildren.push_back(Sub.compChildren[k]);
  }
  return subRoot + base;
}

// The top `depth` levels of the recursion with the two halves dissected
// concurrently, each in a state of its own; below that (or for small sets)
// the serial recursion.
int dissect_parallel(NDState& S, std::vector<int> set, int depth) {
  if (depth <= 0 || set.size() < 20000) return dissect(S, std::move(set));
  std::vector<int> L, R, sep;
  if (!split(S, set, L, R, sep)) return new_component(S, std::move(set), 0);
  auto fresh = [&]() {
    NDState T;
    T.A = S.A;
    T.xyz = S.xyz;
    T.leaf = S.leaf;
    T.mark.assign(S.mark.size(), 0);
    T.level.assign(S.mark.size(), 0);
    return T;
  };
  NDState SL = fresh(), SR = fresh();
  int rootL = -1, rootR = -1;
  std::future<int> fl;
  if (!L.empty())
    fl = std::async(std::launch::async, [&SL, &L, depth]() { return dissect_parallel(SL, std::move(L), depth - 1); });
  if (!R.empty()) rootR = dissect_parallel(SR, std::move(R), depth - 1);
  if (fl.valid()) rootL = fl.get();
  std::vector<int> kids;
  if (rootL >= 0) kids.push_back(adopt(S, SL, rootL));
  if (rootR >= 0) kids.push_back(adopt(S, SR, rootR));
  int c = new_component(S, std::move(sep), (int)kids.size());
  for (int k : kids) S.compParent[k] = c;
  return c;
}

}  // namespace

void nested_dissection(const CSC& A, const double* xyz, int ndLeaf, std::vector<int>& perm,
                       std::vector<Component>& comps, std::vector<int>& compParent) {
  NDState S;
  S.A = &A;
  S.xyz = xyz;
  S.leaf = std::max(1, ndLeaf);
  S.mark.assign(A.n, 0);
  S.level.assign(A.n, 0);
  std::vector<int> all(A.n);
  std::iota(all.begin(), all.end(), 0);
  // Disconnected pieces are handled by the bisection itself.  The top levels
  // run their two halves concurrently: log2 of the host threads, at most four
  // levels (16 threads).
  int depth = 0;
  while (depth < 4 && (2 << depth) <= host_threads()) ++depth;
  if (A.n > 0) dissect_parallel(S, std::move(all), depth);
  perm.clear();
  perm.reserve(A.n);
  comps.assign(S.compMembers.size(), Component());
  int col = 0;
  for (size_t c = 0; c < S.compMembers.size(); ++c) {
    comps[c].size = (int)S.compMembers[c].size();
    comps[c].numChildren = S.compChildren[c];
    comps[c].first = col;
    comps[c].last = col + comps[c].size - 1;
    col += comps[c].size;
    for (int v : S.compMembers[c]) perm.push_back(v);
  }
  compParent = S.compParent;
}

// ---------------------------------------------------------------------------
// Elimination tree and column counts (Davis, "Direct Methods for Sparse
// Linear Systems", SIAM 2006, algorithms etree / counts / leaf).
// ---------------------------------------------------------------------------
std::vector<int> etree_upper(const CSC& C) {
  const int n = C.n;
  std::vector<int> parent(n, -1), ancestor(n, -1);
  for (int k = 0; k < n; ++k) {
    parent[k] = -1;
    ancestor[k] = -1;
    for (int p = C.p[k]; p < C.p[k + 1]; ++p) {
      int i = C.i[p];
      while (i != -1 && i < k) {
        int inext = ancestor[i];
        ancestor[i] = k;
        if (inext == -1) parent[i] = k;
        i = inext;
      }
    }
  }
  return parent;
}

std::vector<int> column_counts(const CSC& C, const std::vector<int>& parent,
                               const std::vector<int>& post) {
  const int n = C.n;
  // AT = C^T: for each column j of AT, the rows i with C(j,i) != 0.
  std::vector<int> cnt(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int p = C.p[j]; p < C.p[j + 1]; ++p) cnt[C.i[p]]++;
  std::vector<int> ATp(n + 1, 0);
  for (int j = 0; j < n; ++j) ATp[j + 1] = ATp[j] + cnt[j];
  std::vector<int> ATi(ATp[n]), fill(ATp.begin(), ATp.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int p = C.p[j]; p < C.p[j + 1]; ++p) ATi[fill[C.i[p]]++] = j;

  std::vector<int> delta(n), ancestor(n), maxfirst(n, -1), prevleaf(n, -1), first(n, -1);
  for (int k = 0; k < n; ++k) {
    int j = post[k];
    delta[j] = (first[j] == -1) ? 1 : 0;
    for (; j != -1 && first[j] == -1; j = parent[j]) first[j] = k;
  }
  for (int i = 0; i < n; ++i) ancestor[i] = i;
  auto leaf = [&](int i, int j, int& jleaf) -> int {
    jleaf = 0;
    if (i <= j || first[j] <= maxfirst[i]) return -1;
    maxfirst[i] = first[j];
    int jprev = prevleaf[i];
    prevleaf[i] = j;
    jleaf = (jprev == -1) ? 1 : 2;
    if (jleaf == 1) return i;
    int q;
    for (q = jprev; q != ancestor[q]; q = ancestor[q]) {}
    for (int s = jprev, sp; s != q; s = sp) { sp = ancestor[s]; ancestor[s] = q; }
    return q;
  };
  for (int k = 0; k < n; ++k) {
    int j = post[k];
    if (parent[j] != -1) delta[parent[j]]--;
    for (int p = ATp[j]; p < ATp[j + 1]; ++p) {
      int i = ATi[p], jleaf;
      int q = leaf(i, j, jleaf);
      if (jleaf >= 1) delta[j]++;
      if (jleaf == 2) delta[q]--;
    }
    if (parent[j] != -1) ancestor[j] = parent[j];
  }
  for (int j = 0; j < n; ++j)
    if (parent[j] != -1) delta[parent[j]] += delta[j];
  return delta;
}

// ---------------------------------------------------------------------------
// BuildRelaxedSupernodes (NestedDissection.cpp:1266-1735): fundamental
// supernodes inside uncompressed components, whole separators as single
// supernodes for compressed components, then CHOLMOD-style relaxed
// amalgamation that never merges a separator supernode.
// ---------------------------------------------------------------------------
std::vector<NodeSpec> relaxed_supernodes(const std::vector<int>& Parent,
                                         const std::vector<int>& columnCounts,
                                         const std::vector<Component>& seps,
                                         const std::vector<int>& sepParent,
                                         int maxBlockSize) {
  const int n = (int)Parent.size();
  const int nrelax0 = 4, nrelax1 = 16, nrelax2 = 48;
  const double zrelax0 = 0.8, zrelax1 = 0.1, zrelax2 = 0.05;
  std::vector<int> Wi(n, 0), Wj(n, 0), Sparent(n, 0), Snz(n, 0), Merged(n, 0), Super(n + 1, 0);
  std::vector<char> IsSeparator(n + 1, 0);
  for (int j = 0; j < n; ++j)
    if (Parent[j] >= 0) Wi[Parent[j]]++;

  std::vector<char> compressNode(seps.size(), 0);
  for (size_t s = 0; s < seps.size(); ++s)
    if (seps[s].size > maxBlockSize && seps[s].numChildren > 0) {
      compressNode[s] = 1;
      for (int pi = sepParent[s]; pi >= 0; pi = sepParent[pi]) compressNode[pi] = 1;
    }

  int nfsuper = 0;
  int col = 0;
  bool newSegment = true;
  for (size_t s = 0; s < seps.size(); ++s) {
    const Component& sep = seps[s];
    if (compressNode[s]) {
      Super[nfsuper] = sep.first;
      IsSeparator[nfsuper] = 1;
      nfsuper += 1;
      newSegment = true;
    } else {
      if (newSegment) {
        Super[nfsuper] = sep.first;
        nfsuper += 1;
        col = sep.first + 1;
        newSegment = false;
      }
      for (; col <= sep.last; ++col)
        if (Parent[col - 1] != col || columnCounts[col - 1] != columnCounts[col] + 1 || Wi[col] > 1)
          Super[nfsuper++] = col;
    }
  }
  Super[nfsuper] = n;

  int* Nscol = Wi.data();
  int* SuperMap = Wj.data();
  for (int s = 0; s < nfsuper; ++s)
    for (int k = Super[s]; k < Super[s + 1]; ++k) SuperMap[k] = s;
  for (int s = 0; s < nfsuper; ++s) {
    int j = Super[s + 1] - 1;
    int parent = Parent[j];
    Sparent[s] = (parent == -1) ? -1 : SuperMap[parent];
  }
  int* Zeros = Wj.data();
  for (int s = 0; s < nfsuper; ++s) {
    Merged[s] = -1;
    Nscol[s] = Super[s + 1] - Super[s];
    Zeros[s] = 0;
    Snz[s] = columnCounts[Super[s]];
  }
  for (int s = nfsuper - 2; s >= 0; --s) {
    int ss = Sparent[s];
    if (ss == -1) continue;
    if (IsSeparator[s] || IsSeparator[s + 1]) continue;
    for (ss = Sparent[s]; Merged[ss] != -1; ss = Merged[ss]) {}
    int sparent = ss;
    for (ss = Sparent[s]; Merged[ss] != -1;) {
      int snext = Merged[ss];
      Merged[ss] = sparent;
      ss = snext;
    }
    if (sparent != s + 1) continue;
    int nscol0 = Nscol[s], nscol1 = Nscol[s + 1], ns = nscol0 + nscol1;
    int totzeros = Zeros[s + 1];
    bool merge;
    if (ns <= nrelax0) {
      merge = true;
    } else {
      double lnz0 = Snz[s], lnz1 = Snz[s + 1];
      double xnewzeros = nscol0 * (lnz1 + nscol0 - lnz0);
      int newzeros = nscol0 * (Snz[s + 1] + nscol0 - Snz[s]);
      if (xnewzeros == 0) {
        merge = true;
      } else {
        double xtotzeros = ((double)totzeros) + xnewzeros;
        double xns = (double)ns;
        double xtotsize = (xns * (xns + 1) / 2) + xns * (lnz1 - nscol1);
        double z = xtotzeros / xtotsize;
        totzeros += newzeros;
        merge = ((ns <= nrelax1 && z < zrelax0) || (ns <= nrelax2 && z < zrelax1) || (z < zrelax2));
      }
    }
    if (merge) {
      Zeros[s] = totzeros;
      Merged[s + 1] = s;
      Snz[s] = nscol0 + Snz[s + 1];
      Nscol[s] += Nscol[s + 1];
    }
  }
  int nsuper = 0;
  for (int s = 0; s < nfsuper; ++s)
    if (Merged[s] == -1) {
      Super[nsuper] = Super[s];
      Snz[nsuper] = Snz[s];
      IsSeparator[nsuper] = IsSeparator[s];
      nsuper++;
    }
  Super[nsuper] = n;
  std::vector<NodeSpec> nodes(nsuper);
  for (int s = 0; s < nsuper; ++s) {
    nodes[s].c0 = Super[s];
    nodes[s].c1 = Super[s + 1] - 1;
    nodes[s].compressed = IsSeparator[s] != 0;
  }
  return nodes;
}

// ---------------------------------------------------------------------------
// SeparatorTree<T> with LONGEST_AXIS splits, FIXED zero-thickness separator
// (so findChildSizes always halves), storeSeparator = false, fullTree = true
// (src/rschol/datastructure/SeparatorTree.cpp:80-560).
// ---------------------------------------------------------------------------
namespace {

struct SepTreeBuilder {
  const std::vector<const double*>* pts;
  std::vector<int> order;
  std::vector<std::pair<int, int>> leaves;

  // Returns the height of the subtree; appends leaves left to right.
  int build(std::vector<int>& data, int maxLeaf) {
    double lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int v : data)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], (*pts)[v][d]);
        hi[d] = std::max(hi[d], (*pts)[v][d]);
      }
    int split = 0;
    double maxLength = -1.0;
    for (int d = 0; d < 3; ++d)
      if (hi[d] - lo[d] > maxLength) { split = d; maxLength = hi[d] - lo[d]; }
    if ((int)data.size() <= maxLeaf) {
      emit(data);
      return 0;
    }
    const std::vector<const double*>& P = *pts;
    std::sort(data.begin(), data.end(),
              [&](int a, int b) { return P[a][split] < P[b][split]; });
    int leftSize = (int)data.size() / 2;
    std::vector<int> leftData(data.begin(), data.begin() + leftSize);
    std::vector<int> rightData(data.begin() + leftSize, data.end());
    if (leftData.size() == data.size() || rightData.empty()) {
      emit(data);
      return 0;
    }
    int lh, rh;
    if ((int)rightData.size() > maxLeaf && (int)leftData.size() <= maxLeaf)
      lh = build(leftData, (int)leftData.size() - 1);
    else
      lh = build(leftData, maxLeaf);
    if ((int)leftData.size() > maxLeaf && (int)rightData.size() <= maxLeaf)
      rh = build(rightData, (int)rightData.size() - 1);
    else
      rh = build(rightData, maxLeaf);
    return 1 + std::max(lh, rh);
  }

  void emit(const std::vector<int>& data) {
    int start = leaves.empty() ? 0 : leaves.back().second + 1;
    leaves.push_back({start, start + (int)data.size() - 1});
    for (int v : data) order.push_back(v);
  }
};

}  // namespace

void separator_tree(const std::vector<const double*>& pts, int maxLeaf, std::vector<int>& order,
                    std::vector<std::pair<int, int>>& leaves) {
  SepTreeBuilder B;
  B.pts = &pts;
  std::vector<int> data(pts.size());
  std::iota(data.begin(), data.end(), 0);
  B.build(data, maxLeaf);
  order = std::move(B.order);
  leaves = std::move(B.leaves);
}

// ---------------------------------------------------------------------------
OrderingResult build_ordering(const CSC& A, const double* xyz, const Params& prm) {
  OrderingResult R;
  nested_dissection(A, xyz, prm.nd_leaf, R.perm, R.comps, R.compParent);
  const int n = A.n;
  R.iperm.assign(n, 0);
  for (int k = 0; k < n; ++k) R.iperm[R.perm[k]] = k;

  // Upper pattern (no diagonal) of P A P^T, rows sorted.
  CSC C;
  C.n = n;
  C.p.assign(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int p = A.p[j]; p < A.p[j + 1]; ++p) {
      int a = R.iperm[A.i[p]], b = R.iperm[j];
      if (a < b) C.p[b + 1]++;
    }
  for (int j = 0; j < n; ++j) C.p[j + 1] += C.p[j];
  C.i.resize(C.p[n]);
  {
    std::vector<int> fill(C.p.begin(), C.p.end() - 1);
    for (int j = 0; j < n; ++j)
      for (int p = A.p[j]; p < A.p[j + 1]; ++p) {
        int a = R.iperm[A.i[p]], b = R.iperm[j];
        if (a < b) C.i[fill[b]++] = a;
      }
    parallel_chunks(n, 16384, [&](long long b, long long e) {
      for (long long j = b; j < e; ++j) std::sort(C.i.begin() + C.p[j], C.i.begin() + C.p[j + 1]);
    });
  }
  R.etree = etree_upper(C);
  std::vector<int> post(n);
  std::iota(post.begin(), post.end(), 0);  // the reference passes the identity postorder
  R.colcount = column_counts(C, R.etree, post);
  R.nodes = relaxed_supernodes(R.etree, R.colcount, R.comps, R.compParent, prm.max_dense_block);

  // ReorderNestedSeparators (IN_PLACE: every node is considered).
  std::vector<double> zero(3, 0.0);
  R.diagBlocks.assign(R.nodes.size(), {});
  const bool reorder = prm.reorder_separators && xyz != nullptr;
  for (size_t s = 0; s < R.nodes.size(); ++s) {
    const NodeSpec& nd = R.nodes[s];
    int size = nd.c1 - nd.c0 + 1;
    if (size <= prm.max_diag_block) continue;
    std::vector<const double*> pts(size);
    for (int k = 0; k < size; ++k) {
      int old = R.perm[nd.c0 + k];
      pts[k] = xyz ? &xyz[3 * (size_t)old] : zero.data();
    }
    std::vector<int> order;
    std::vector<std::pair<int, int>> leaves;
    separator_tree(pts, prm.max_diag_block, order, leaves);
    if (reorder) {
      std::vector<int> olds(size);
      for (int k = 0; k < size; ++k) olds[k] = R.perm[nd.c0 + order[k]];
      for (int k = 0; k < size; ++k) R.perm[nd.c0 + k] = olds[k];
    }
    R.diagBlocks[s] = leaves;
  }
  for (int k = 0; k < n; ++k) R.iperm[R.perm[k]] = k;
  return R;
}

CSC permute_lower(const CSC& A, const std::vector<int>& perm, const std::vector<int>& iperm) {
  const int n = A.n;
  CSC L;
  L.n = n;
  L.p.assign(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int p = A.p[j]; p < A.p[j + 1]; ++p)
      if (iperm[A.i[p]] >= iperm[j]) L.p[iperm[j] + 1]++;
  for (int j = 0; j < n; ++j) L.p[j + 1] += L.p[j];
  L.i.resize(L.p[n]);
  L.x.resize(L.p[n]);
  std::vector<int> fill(L.p.begin(), L.p.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int p = A.p[j]; p < A.p[j + 1]; ++p) {
      int r = iperm[A.i[p]], c = iperm[j];
      if (r >= c) {
        L.i[fill[c]] = r;
        L.x[fill[c]] = A.x.empty() ? 0.0 : A.x[p];
        fill[c]++;
      }
    }
  parallel_chunks(n, 16384, [&](long long b, long long e) {
    std::vector<std::pair<int, double>> tmp;
    for (long long j = b; j < e; ++j) {
      tmp.clear();
      for (int p = L.p[j]; p < L.p[j + 1]; ++p) tmp.push_back({L.i[p], L.x[p]});
      std::sort(tmp.begin(), tmp.end(),
                [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
      for (int p = L.p[j], k = 0; p < L.p[j + 1]; ++p, ++k) { L.i[p] = tmp[k].first; L.x[p] = tmp[k].second; }
    }
  });
  (void)perm;
  return L;
}

}  // namespace rschol
