// Host-only entry points of the C ABI: synthetic problem generators and the
// symbolic summary used by benchmarks and tests (declared in
// include/rschol_gpu.h).
#include <cstring>
#include <exception>
#include <string>

#include "ordering.h"
#include "problems.h"
#include "rng.h"
#include "symbolic.h"

extern "C" {

void* rschol_problem_diffusion(int dim, int nx, int ny, int nz, double sigma, unsigned seed, int nrhs) {
  try {
    return new rschol::Problem(rschol::make_diffusion(dim, nx, ny, nz, sigma, seed, nrhs));
  } catch (const std::exception&) {
    return nullptr;
  }
}

void* rschol_problem_elasticity(int ne, double E, double nu, unsigned seed, int nrhs) {
  try {
    return new rschol::Problem(rschol::make_elasticity(ne, E, nu, seed, nrhs));
  } catch (const std::exception&) {
    return nullptr;
  }
}

int rschol_problem_n(const void* p) { return ((const rschol::Problem*)p)->n; }
long long rschol_problem_nnz(const void* p) { return (long long)((const rschol::Problem*)p)->rowind.size(); }
int rschol_problem_nrhs(const void* p) { return ((const rschol::Problem*)p)->nrhs; }

void rschol_problem_get(const void* p, int* colptr, int* rowind, double* vals, double* xyz, double* rhs) {
  const rschol::Problem& P = *(const rschol::Problem*)p;
  if (colptr) std::memcpy(colptr, P.colptr.data(), sizeof(int) * P.colptr.size());
  if (rowind) std::memcpy(rowind, P.rowind.data(), sizeof(int) * P.rowind.size());
  if (vals) std::memcpy(vals, P.vals.data(), sizeof(double) * P.vals.size());
  if (xyz) std::memcpy(xyz, P.xyz.data(), sizeof(double) * P.xyz.size());
  if (rhs) std::memcpy(rhs, P.rhs.data(), sizeof(double) * P.rhs.size());
}

void rschol_problem_free(void* p) { delete (rschol::Problem*)p; }

// MT19937 draws with the reference's conventions, for known-answer tests.
void rschol_mt_draws(unsigned seed, long long count, unsigned* out) {
  rschol::MT19937 g(seed);
  g.rawDraws(count, out);
}

void rschol_mt_gaussians(unsigned seed, long long count, double* out) {
  rschol::MT19937 g(seed);
  g.gaussianMatrix(count, out);
}

}  // extern "C"

// ---- symbolic known-answer entry points --------------------------------------
extern "C" {

int rschol_block_rank(int nRows, int nCols, double c, int oversampling, int cap) {
  return rschol::block_rank(nRows, nCols, c, oversampling, cap);
}

// SeparatorTree order of npts points (3 coordinates each); returns the
// number of leaves, order[npts] and leafFirst[nLeaves + 1].
int rschol_separator_tree(int npts, const double* xyz, int maxLeaf, int* order, int* leafFirst) {
  std::vector<const double*> pts(npts);
  for (int i = 0; i < npts; ++i) pts[i] = xyz + 3 * (size_t)i;
  std::vector<int> ord;
  std::vector<std::pair<int, int>> leaves;
  rschol::separator_tree(pts, maxLeaf, ord, leaves);
  for (int i = 0; i < npts; ++i) order[i] = ord[i];
  for (size_t k = 0; k < leaves.size(); ++k) leafFirst[k] = leaves[k].first;
  leafFirst[leaves.size()] = npts;
  return (int)leaves.size();
}

// Elimination tree and column counts (identity postorder) of the upper
// pattern (row < col) given as CSC.
void rschol_etree_counts(int n, const int* colptr, const int* rowind, int* parent, int* counts) {
  rschol::CSC C;
  C.n = n;
  C.p.assign(colptr, colptr + n + 1);
  C.i.assign(rowind, rowind + colptr[n]);
  std::vector<int> par = rschol::etree_upper(C);
  std::vector<int> post(n);
  for (int i = 0; i < n; ++i) post[i] = i;
  std::vector<int> cnt = rschol::column_counts(C, par, post);
  for (int i = 0; i < n; ++i) {
    parent[i] = par[i];
    counts[i] = cnt[i];
  }
}

// BuildRelaxedSupernodes; components given by size / children / first
// column / parent.  Returns the number of supernodes; superFirst[nsuper+1].
int rschol_relaxed_supernodes(int n, const int* parent, const int* counts, int ncomp, const int* compSize,
                              const int* compChildren, const int* compFirst, const int* compParent, int maxBlock,
                              int* superFirst, int* compressed) {
  std::vector<rschol::Component> comps(ncomp);
  for (int c = 0; c < ncomp; ++c) {
    comps[c].size = compSize[c];
    comps[c].numChildren = compChildren[c];
    comps[c].first = compFirst[c];
    comps[c].last = compFirst[c] + compSize[c] - 1;
  }
  std::vector<int> par(parent, parent + n), cnt(counts, counts + n), cp(compParent, compParent + ncomp);
  std::vector<rschol::NodeSpec> nodes = rschol::relaxed_supernodes(par, cnt, comps, cp, maxBlock);
  for (size_t s = 0; s < nodes.size(); ++s) {
    superFirst[s] = nodes[s].c0;
    compressed[s] = nodes[s].compressed;
  }
  superFirst[nodes.size()] = n;
  return (int)nodes.size();
}

}  // extern "C"
