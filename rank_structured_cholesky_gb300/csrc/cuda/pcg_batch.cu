// Batched PCG: k right-hand sides in lockstep on one factor (the c4 form of
// PCG_SOLVER::solvePCG, src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363).
// Vectors are n x k row-major blocks; every column sum follows one fixed
// order that depends on n alone (below), so each column's arithmetic is
// reproducible and the same whatever k is.  A column that reaches its tolerance keeps alpha = 0 from
// then on (x and r frozen), as if its own loop had stopped.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "pcg.cuh"

namespace rschol {

namespace {

constexpr int BT = 256;                 // threads per block
constexpr int BBLOCKS = 152 * 4;        // fixed grid of the vector kernels
constexpr int KMAX = 64;

enum { S_DELTA = 0, S_ALPHA, S_BETA, S_RREL, S_BNORM, S_DQ, S_ACTIVE, S_BREAK, S_FRESH, S_COUNT };
enum { F_ALPHA = 0, F_RNORM, F_BETA, F_DELTA0, F_BNORM, F_TRUE, F_SLOT };

// Row tiles and the order of every column sum.  Rows are cut into tiles of
// 32.  A tile's 32 row values meet in a pairwise tree (rows s and s ^ 1,
// then pairs of pairs, ...); warp w of the fixed grid adds the sums of tiles
// w, w + W, w + 2W, ... (W warps) in order; the 8 warps of a block are added
// in order; finish_k_kernel adds the blocks.  This order depends on n alone.
// How lanes cover (tile row, column) pairs depends on k: with KP (k rounded
// up to a power of two) columns, KL = min(KP, 32) lanes run along the
// columns and G = 32 / KL along the tile rows.  For G > 1 each lane holds
// rows g + G j of a tile and the tree is a butterfly (across lanes, then
// within the lane); for G = 1 a lane walks the tile's rows in order and
// builds the same tree on a five-entry stack (two columns per lane at KP =
// 64).  So every lane has work at any k, loads are coalesced along rows
// (small k) or along columns (large k), and a column's arithmetic does not
// depend on k.
template <int KP>
struct Lay {
  static constexpr int CPL = KP > 32 ? 2 : 1;   // columns per lane
  static constexpr int KL = KP > 32 ? 32 : KP;  // lanes along the columns
  static constexpr int G = 32 / KL;             // lanes along the tile rows
  static constexpr int SPL = 32 / G;            // tile rows per lane
};

// trailing one bits of s: the tree level a stack entry is stored at
__host__ __device__ constexpr int trailing_ones(int s) { return (s & 1) ? 1 + trailing_ones(s >> 1) : 0; }

// Rows S.. of a tile for the G = 1 layout: push row S's value on the stack,
// combining it with the stored left subtrees (compile-time indices).
template <int S, int CPL, class Leaf>
__device__ __forceinline__ void tree_rows(int row0, int n, int k, int cl, double (&st)[CPL][5], double (&W)[CPL],
                                          Leaf& leaf) {
  if constexpr (S < 32) {
    const int row = row0 + S;
#pragma unroll
    for (int q = 0; q < CPL; ++q) {
      const int c = cl + 32 * q;
      double v = (row < n && c < k) ? leaf(row, c) : 0.0;
#pragma unroll
      for (int b = 0; b < trailing_ones(S); ++b) v = st[q][b] + v;
      if constexpr (S < 31) st[q][trailing_ones(S)] = v;
      else W[q] += v;
    }
    tree_rows<S + 1, CPL>(row0, n, k, cl, st, W, leaf);
  }
}

// Column sums of leaf(row, c) over the rows of this warp's tiles, reduced
// to part[blockIdx.x * k + c].  Every thread of the block must call it.
template <int KP, class Leaf>
__device__ __forceinline__ void tile_sums(int n, int k, Leaf&& leaf, double* part) {
  using L = Lay<KP>;
  __shared__ double red[BT / 32][KMAX];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane / L::KL, cl = lane % L::KL;
  const int nt = (n + 31) / 32;
  double W[L::CPL];
#pragma unroll
  for (int q = 0; q < L::CPL; ++q) W[q] = 0.0;
  for (int tile = blockIdx.x * (BT / 32) + warp; tile < nt; tile += gridDim.x * (BT / 32)) {
    if constexpr (L::G == 1) {
      double st[L::CPL][5];
      tree_rows<0, L::CPL>(tile * 32, n, k, cl, st, W, leaf);
    } else {
      double v[L::SPL];
#pragma unroll
      for (int j = 0; j < L::SPL; ++j) {
        const int row = tile * 32 + g + L::G * j;
        v[j] = (row < n && cl < k) ? leaf(row, cl) : 0.0;
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        if (o < L::G) {   // partner row in lane ^ (o * KL)
#pragma unroll
          for (int j = 0; j < L::SPL; ++j) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o * L::KL);
        } else {          // partner row in this lane
          const int jo = o / L::G;
#pragma unroll
          for (int j = 0; j < L::SPL; ++j)
            if ((j & jo) == 0) {
              const double t = v[j] + v[j ^ jo];
              v[j] = t;
              v[j ^ jo] = t;
            }
        }
      }
      W[0] += v[0];
    }
  }
  if (g == 0)
#pragma unroll
    for (int q = 0; q < L::CPL; ++q)
      if (cl + 32 * q < k) red[warp][cl + 32 * q] = W[q];
  __syncthreads();
  if ((int)threadIdx.x < k) {
    double t = 0.0;
    for (int w = 0; w < BT / 32; ++w) t += red[w][threadIdx.x];
    part[(size_t)blockIdx.x * k + threadIdx.x] = t;
  }
}

// y = A x, and the partials of the column dots x . y.  Each y value is the
// serial sum over its row's nonzeros.
template <int KP>
__global__ void __launch_bounds__(BT) spmv_k_kernel(int n, int k, const int* __restrict__ rp,
                                                     const int* __restrict__ ci, const double* __restrict__ v,
                                                     const double* __restrict__ x, double* __restrict__ y,
                                                     double* __restrict__ part) {
  tile_sums<KP>(n, k, [&](int row, int c) {
    double s = 0.0;
    for (int p = rp[row]; p < rp[row + 1]; ++p) s += v[p] * x[(size_t)ci[p] * k + c];
    const size_t o = (size_t)row * k + c;
    y[o] = s;
    return x[o] * s;
  }, part);
}

template <int KP>
__global__ void __launch_bounds__(BT) dot_k_kernel(const double* __restrict__ a, const double* __restrict__ b, int n,
                                                   int k, double* __restrict__ part) {
  tile_sums<KP>(n, k, [&](int row, int c) {
    const size_t o = (size_t)row * k + c;
    return a[o] * b[o];
  }, part);
}

// Column scalars from the block partials: a warp per column, lane l adds
// blocks l, l + 32, ... in order, then a fixed butterfly over the lanes.
__global__ void __launch_bounds__(256) finish_k_kernel(const double* __restrict__ part, int count, int k,
                                                       double* __restrict__ sc, int mode) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= k) return;
  double t = 0.0;
  for (int b = lane; b < count; b += 32) t += part[(size_t)b * k + c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane != 0) return;
  double* s = sc + (size_t)c * S_COUNT;
  switch (mode) {
    case F_ALPHA:
      s[S_DQ] = t;
      if (s[S_ACTIVE] == 0.0) s[S_ALPHA] = 0.0;
      else if (fabs(t) > 0.0) s[S_ALPHA] = s[S_DELTA] / t;
      else { s[S_ALPHA] = 0.0; s[S_BREAK] = 1.0; }
      break;
    case F_RNORM:
      if (s[S_ACTIVE] != 0.0) s[S_RREL] = sqrt(t) / s[S_BNORM];
      break;
    case F_BETA:
      if (s[S_ACTIVE] != 0.0) {
        s[S_BETA] = t / s[S_DELTA];
        s[S_DELTA] = t;
      } else {
        s[S_BETA] = 0.0;
      }
      break;
    case F_DELTA0: s[S_DELTA] = t; break;
    case F_BNORM: s[S_BNORM] = sqrt(t); s[S_ACTIVE] = 1.0; break;
    case F_TRUE: s[S_RREL] = sqrt(t) / s[S_BNORM]; break;
    case F_SLOT:   // t = r.s; a column that has just joined starts its recurrence (d = s)
      if (s[S_FRESH] != 0.0) {
        s[S_DELTA] = t;
        s[S_BETA] = 0.0;
        s[S_FRESH] = 0.0;
      } else {
        s[S_BETA] = t / s[S_DELTA];
        s[S_DELTA] = t;
      }
      break;
  }
}

template <int KP>
__global__ void __launch_bounds__(BT) update_xr_k_kernel(double* __restrict__ x, double* __restrict__ r,
                                                         const double* __restrict__ d, const double* __restrict__ q,
                                                         const double* __restrict__ sc, int n, int k,
                                                         double* __restrict__ part) {
  tile_sums<KP>(n, k, [&](int row, int c) {
    const double al = sc[(size_t)c * S_COUNT + S_ALPHA];
    const size_t o = (size_t)row * k + c;
    x[o] += al * d[o];
    const double ri = r[o] - al * q[o];
    r[o] = ri;
    return ri * ri;
  }, part);
}

__global__ void __launch_bounds__(BT) update_d_k_kernel(double* __restrict__ d, const double* __restrict__ s,
                                                        const double* __restrict__ sc, int n, int k) {
  const long long tot = (long long)n * k;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e % k);
    d[e] = s[e] + sc[(size_t)c * S_COUNT + S_BETA] * d[e];
  }
}

template <int KP>
__global__ void __launch_bounds__(BT) residual_k_kernel(const double* __restrict__ b, const double* __restrict__ q,
                                                        int n, int k, double* __restrict__ part) {
  tile_sums<KP>(n, k, [&](int row, int c) {
    const size_t o = (size_t)row * k + c;
    const double e = b[o] - q[o];
    return e * e;
  }, part);
}

int kp_of(int k) {
  int p = 1;
  while (p < k) p <<= 1;
  return p;
}

#define RSCHOL_KP_SWITCH(k, LAUNCH)                                         \
  switch (kp_of(k)) {                                                       \
    case 1: LAUNCH(1); break;                                               \
    case 2: LAUNCH(2); break;                                               \
    case 4: LAUNCH(4); break;                                               \
    case 8: LAUNCH(8); break;                                               \
    case 16: LAUNCH(16); break;                                             \
    case 32: LAUNCH(32); break;                                             \
    case 64: LAUNCH(64); break;                                             \
    default: throw std::runtime_error("batched PCG: more than 64 columns"); \
  }

void spmv_k(cudaStream_t st, int n, int k, const int* rp, const int* ci, const double* v, const double* x, double* y,
            double* part) {
#define L_(KP) spmv_k_kernel<KP><<<BBLOCKS, BT, 0, st>>>(n, k, rp, ci, v, x, y, part)
  RSCHOL_KP_SWITCH(k, L_)
#undef L_
}
void dot_k(cudaStream_t st, const double* a, const double* b, int n, int k, double* part) {
#define L_(KP) dot_k_kernel<KP><<<BBLOCKS, BT, 0, st>>>(a, b, n, k, part)
  RSCHOL_KP_SWITCH(k, L_)
#undef L_
}
void update_xr_k(cudaStream_t st, double* x, double* r, const double* d, const double* q, const double* sc, int n,
                 int k, double* part) {
#define L_(KP) update_xr_k_kernel<KP><<<BBLOCKS, BT, 0, st>>>(x, r, d, q, sc, n, k, part)
  RSCHOL_KP_SWITCH(k, L_)
#undef L_
}
void residual_k(cudaStream_t st, const double* b, const double* q, int n, int k, double* part) {
#define L_(KP) residual_k_kernel<KP><<<BBLOCKS, BT, 0, st>>>(b, q, n, k, part)
  RSCHOL_KP_SWITCH(k, L_)
#undef L_
}
void update_d_k(cudaStream_t st, double* d, const double* s, const double* sc, int n, int k) {
  const long long tot = (long long)n * k;
  update_d_k_kernel<<<(unsigned)std::min<long long>((tot + BT - 1) / BT, BBLOCKS * 4), BT, 0, st>>>(d, s, sc, n, k);
}

__global__ void gather_k_kernel(const double* __restrict__ src, const int* __restrict__ perm,
                                double* __restrict__ dst, int n, int k) {
  const long long tot = (long long)n * k;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / k, c = e - i * k;
    dst[e] = src[c * n + perm[i]];
  }
}

__global__ void scatter_k_kernel(const double* __restrict__ src, const int* __restrict__ perm,
                                 double* __restrict__ dst, int n, int k) {
  const long long tot = (long long)n * k;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / k, c = e - i * k;
    dst[c * n + perm[i]] = src[e];
  }
}

// Session column moves: new column j takes old column map.src[j] of the
// (x, r, d, b) blocks, or (when map.src[j] < 0) starts a joining column:
// x = d = 0, r = b = column -1 - map.src[j] of the n x m block bnew.
struct ColMap {
  int src[64];
};

__global__ void __launch_bounds__(BT) relayout_kernel(int n, int kOld, int kNew, ColMap map,
                                                      const double* __restrict__ xo, const double* __restrict__ ro,
                                                      const double* __restrict__ dd, const double* __restrict__ bo,
                                                      double* __restrict__ xn, double* __restrict__ rn,
                                                      double* __restrict__ dn, double* __restrict__ bn,
                                                      const double* __restrict__ bnew, int m) {
  const long long tot = (long long)n * kNew;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / kNew;
    const int j = (int)(e - i * kNew);
    const int src = map.src[j];
    if (src >= 0) {
      const long long o = i * kOld + src;
      xn[e] = xo[o];
      rn[e] = ro[o];
      dn[e] = dd[o];
      bn[e] = bo[o];
    } else {
      const double bv = bnew[i * m + (-1 - src)];
      xn[e] = 0.0;
      rn[e] = bv;
      dn[e] = 0.0;
      bn[e] = bv;
    }
  }
}

// Finished columns out of the n x k block, back to the original order:
// dst[c * n + perm[i]] = x[i * k + map.src[c]], c < count.
__global__ void __launch_bounds__(BT) extract_kernel(int n, int k, int count, ColMap map, const int* __restrict__ perm,
                                                     const double* __restrict__ x, double* __restrict__ dst) {
  const long long tot = (long long)n * count;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / count;
    const int c = (int)(e - i * count);
    dst[(long long)c * n + perm[i]] = x[i * k + map.src[c]];
  }
}

}  // namespace

void launch_gather_k(const double* src, const int* perm, double* dst, int n, int k, cudaStream_t s) {
  gather_k_kernel<<<BBLOCKS * 2, BT, 0, s>>>(src, perm, dst, n, k);
  RSCHOL_LAUNCH_CHECK();
}
void launch_scatter_k(const double* src, const int* perm, double* dst, int n, int k, cudaStream_t s) {
  scatter_k_kernel<<<BBLOCKS * 2, BT, 0, s>>>(src, perm, dst, n, k);
  RSCHOL_LAUNCH_CHECK();
}

std::vector<PcgResult> PcgEngine::solve_batch(const double* B, double* X, int k, double eps, int maxit,
                                              const std::function<void(double*)>& apply) {
  if (k < 1 || k > KMAX) throw std::runtime_error("solve_batch: 1..64 right-hand sides per batch");
  cudaStream_t st = stream_;
  const size_t nk = (size_t)n * k;
  if (k != kB_) {
    for (auto* b : {&rB_, &dB_, &qB_, &sB_}) b->alloc(sizeof(double) * std::max<size_t>(1, nk));
    partB_.alloc(sizeof(double) * BBLOCKS * k);
    scalB_.alloc(sizeof(double) * S_COUNT * k);
    if (hScalB_) cudaFreeHost(hScalB_);
    hScalB_ = nullptr;
    RSCHOL_CUDA(cudaMallocHost((void**)&hScalB_, sizeof(double) * S_COUNT * k));
    kB_ = k;
  }
  double* r = rB_.as<double>();
  double* d = dB_.as<double>();
  double* q = qB_.as<double>();
  double* s = sB_.as<double>();
  double* part = partB_.as<double>();
  double* sc = scalB_.as<double>();
  const int* rp = rowptr_.as<int>();
  const int* ci = colind_.as<int>();
  const double* v = vals_.as<double>();
  launches = 0;
  std::vector<PcgResult> res(k);
  RSCHOL_CUDA(cudaMemsetAsync(sc, 0, sizeof(double) * S_COUNT * k, st));
  RSCHOL_CUDA(cudaMemsetAsync(X, 0, sizeof(double) * nk, st));
  RSCHOL_CUDA(cudaMemcpyAsync(r, B, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
  dot_k(st, B, B, n, k, part);
  finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_BNORM);
  RSCHOL_CUDA(cudaMemcpyAsync(s, r, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
  apply(s);
  dot_k(st, r, s, n, k, part);
  finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_DELTA0);
  RSCHOL_CUDA(cudaMemcpyAsync(d, s, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
  RSCHOL_LAUNCH_CHECK();
  launches += 4;
  std::vector<char> active(k, 1);
  int nActive = k, i = 0;
  while (i < maxit && nActive > 0) {
    spmv_k(st, n, k, rp, ci, v, d, q, part);
    finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_ALPHA);
    update_xr_k(st, X, r, d, q, sc, n, k, part);
    finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_RNORM);
    RSCHOL_CUDA(cudaMemcpyAsync(s, r, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
    apply(s);
    dot_k(st, r, s, n, k, part);
    finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_BETA);
    update_d_k(st, d, s, sc, n, k);
    RSCHOL_LAUNCH_CHECK();
    launches += 7;
    RSCHOL_CUDA(cudaMemcpyAsync(hScalB_, sc, sizeof(double) * S_COUNT * k, cudaMemcpyDeviceToHost, st));
    RSCHOL_CUDA(cudaStreamSynchronize(st));
    ++i;
    bool changed = false;
    for (int c = 0; c < k; ++c) {
      if (!active[c]) continue;
      const double* h = hScalB_ + (size_t)c * S_COUNT;
      res[c].iterations = i;
      res[c].residual = h[S_RREL];
      if (h[S_BREAK] != 0.0) res[c].breakdown = true;
      if (!(h[S_RREL] > eps) || res[c].breakdown) {   // converged, NaN or broken down: stop this column
        active[c] = 0;
        --nActive;
        hScalB_[(size_t)c * S_COUNT + S_ACTIVE] = 0.0;
        changed = true;
      }
    }
    if (changed && nActive > 0)
      for (int c = 0; c < k; ++c)
        if (!active[c])
          RSCHOL_CUDA(cudaMemcpyAsync(sc + (size_t)c * S_COUNT + S_ACTIVE, hScalB_ + (size_t)c * S_COUNT + S_ACTIVE,
                                      sizeof(double), cudaMemcpyHostToDevice, st));
  }
  // true residuals ||b - A x|| / ||b||
  spmv_k(st, n, k, rp, ci, v, X, q, part);
  residual_k(st, B, q, n, k, part);
  finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_TRUE);
  RSCHOL_LAUNCH_CHECK();
  launches += 3;
  RSCHOL_CUDA(cudaMemcpyAsync(hScalB_, sc, sizeof(double) * S_COUNT * k, cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  for (int c = 0; c < k; ++c) res[c].trueResidual = hScalB_[(size_t)c * S_COUNT + S_RREL];
  return res;
}

// ---- continuous batching: columns join and leave at iteration boundaries ----
//
// Every active column follows PCG_SOLVER::solvePCG's recurrences exactly; the
// loop is rotated so that a column can enter at the preconditioner step:
//   s = M^{-1} r;  t = r.s;  joining column: delta = t, d = s;
//                            otherwise: beta = t / delta, delta = t, d = s + beta d;
//   q = A d;  alpha = delta / (d.q);  x += alpha d;  r -= alpha q;  ||r|| / ||b||.
// A joining column has x = 0, r = b, d = 0, so its first pass is the
// reference's set-up followed by its first iteration; every later pass is one
// iteration.  The stopping test after each pass is the reference's.  Column
// arithmetic never mixes columns, so a column's iterates do not depend on the
// other columns in the block.

PcgSession::PcgSession(PcgEngine& pcg, int kmax, const int* dPerm,
                       std::function<void(double*, int)> apply, std::function<int()> applyError,
                       std::function<long long()> applyGen)
    : pcg_(pcg), kmax_(kmax), perm_(dPerm), apply_(std::move(apply)), applyError_(std::move(applyError)),
      applyGen_(std::move(applyGen)) {
  const char* g = std::getenv("RSCHOL_SESSION_GRAPH");
  useGraph_ = !(g && g[0] == '0');
  if (kmax < 1 || kmax > KMAX) throw std::runtime_error("PcgSession: 1..64 columns");
  part_.alloc(sizeof(double) * BBLOCKS * kmax);
  sc_.alloc(sizeof(double) * S_COUNT * kmax);
  RSCHOL_CUDA(cudaMallocHost((void**)&hsc_, sizeof(double) * S_COUNT * kmax));
  hscNew_.assign((size_t)S_COUNT * kmax, 0.0);
}

PcgSession::~PcgSession() {
  if (gExec_) cudaGraphExecDestroy(gExec_);
  if (hsc_) cudaFreeHost(hsc_);
}

// The column blocks grow (doubling, up to kmax) when more columns are active
// than they hold; they never shrink while the session lives.
void PcgSession::reserve_set(int set, int k) {
  if (cap_[set] >= k) return;
  const size_t nk = sizeof(double) * std::max<size_t>(1, (size_t)pcg_.n * k);
  for (auto* v : {&x_[set], &r_[set], &d_[set], &b_[set]}) v->alloc(nk);
  cap_[set] = k;
  ++gen_;
}

void PcgSession::add(long long tag, int col, const double* b, double* x, double eps, int maxit) {
  Column c;
  c.tag = tag;
  c.col = col;
  c.b = b;
  c.xOut = x;
  c.eps = eps;
  c.maxit = maxit;
  queue_.push_back(c);
}

std::vector<PcgSession::Column> PcgSession::step() {
  const int n = pcg_.n;
  cudaStream_t st = pcg_.stream_;
  std::vector<Column> done;
  // 1. membership: the surviving columns keep their order, queued ones join
  const int kOld = (int)cols_.size();
  std::vector<Column> next;
  ColMap map{};
  for (int j = 0; j < kOld; ++j)
    if (!cols_[j].finished) {
      map.src[next.size()] = j;
      next.push_back(cols_[j]);
    }
  const int kNext = (int)std::min<size_t>(next.size() + queue_.size(), (size_t)kmax_);
  if (kNext > capS_) {   // scratch blocks (they also stage the joining columns)
    const int c = std::min(kmax_, std::max(kNext, 2 * capS_));
    const size_t nk = sizeof(double) * std::max<size_t>(1, (size_t)n * c);
    s_.alloc(nk);
    q_.alloc(nk);
    capS_ = c;
    ++gen_;
  }
  int m = 0;
  while (!queue_.empty() && (int)next.size() < kmax_) {
    Column c = queue_.front();
    queue_.pop_front();
    RSCHOL_CUDA(cudaMemcpyAsync(s_.as<double>() + (size_t)m * n, c.b, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    map.src[next.size()] = -1 - m;
    next.push_back(c);
    ++m;
  }
  const int k = (int)next.size();
  if (k != kOld || m > 0) {
    if (m > 0) launch_gather_k(s_.as<double>(), perm_, q_.as<double>(), n, m, st);
    if (k > 0) {
      const int o = cur_, w = 1 - cur_;
      if (cap_[w] < k) reserve_set(w, std::min(kmax_, std::max(k, std::max(2 * cap_[w], cap_[o]))));
      const long long nk = (long long)n * k;
      relayout_kernel<<<(unsigned)std::min<long long>((nk + BT - 1) / BT, BBLOCKS * 4), BT, 0, st>>>(
          n, kOld, k, map, x_[o].as<double>(), r_[o].as<double>(), d_[o].as<double>(), b_[o].as<double>(),
          x_[w].as<double>(), r_[w].as<double>(), d_[w].as<double>(), b_[w].as<double>(), q_.as<double>(), m);
      RSCHOL_LAUNCH_CHECK();
      cur_ = w;
      // per-column scalars follow their columns
      std::fill(hscNew_.begin(), hscNew_.end(), 0.0);
      for (int j = 0; j < k; ++j) {
        double* dst = hscNew_.data() + (size_t)j * S_COUNT;
        if (map.src[j] >= 0) {
          std::copy(hsc_ + (size_t)map.src[j] * S_COUNT, hsc_ + (size_t)(map.src[j] + 1) * S_COUNT, dst);
        } else {
          dst[S_ACTIVE] = 1.0;
          dst[S_FRESH] = 1.0;
        }
      }
      std::copy(hscNew_.begin(), hscNew_.begin() + (size_t)k * S_COUNT, hsc_);
      RSCHOL_CUDA(cudaMemcpyAsync(sc_.p, hsc_, sizeof(double) * S_COUNT * k, cudaMemcpyHostToDevice, st));
      if (m > 0) {   // ||b|| of every column (the same value again for the old ones)
        dot_k(st, b_[cur_].as<double>(), b_[cur_].as<double>(), n, k, part_.as<double>());
        finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part_.as<double>(), BBLOCKS, k, sc_.as<double>(), F_BNORM);
        RSCHOL_LAUNCH_CHECK();
      }
    }
  }
  cols_ = std::move(next);
  if (k == 0) return done;
  double* X = x_[cur_].as<double>();
  double* R = r_[cur_].as<double>();
  double* D = d_[cur_].as<double>();
  double* B = b_[cur_].as<double>();
  double* S = s_.as<double>();
  double* Q = q_.as<double>();
  double* part = part_.as<double>();
  double* sc = sc_.as<double>();
  const int* rp = pcg_.rowptr_.as<int>();
  const int* ci = pcg_.colind_.as<int>();
  const double* v = pcg_.vals_.as<double>();
  const size_t nkBytes = sizeof(double) * (size_t)n * k;
  auto iteration = [&]() {
    // 2. s = M^{-1} r; t = r.s; d = s + beta d
    RSCHOL_CUDA(cudaMemcpyAsync(S, R, nkBytes, cudaMemcpyDeviceToDevice, st));
    apply_(S, k);
    dot_k(st, R, S, n, k, part);
    finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_SLOT);
    update_d_k(st, D, S, sc, n, k);
    // 3. q = A d; alpha; x += alpha d; r -= alpha q; ||r|| / ||b||
    spmv_k(st, n, k, rp, ci, v, D, Q, part);
    finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_ALPHA);
    update_xr_k(st, X, R, D, Q, sc, n, k, part);
    finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_RNORM);
    RSCHOL_LAUNCH_CHECK();
  };
  const GraphKey key{k, cur_, gen_, applyGen_ ? applyGen_() : 0};
  if (useGraph_ && gExec_ && key == gKey_) {
    RSCHOL_CUDA(cudaGraphLaunch(gExec_, st));
  } else if (useGraph_ && key == lastKey_) {
    // the previous step ran this iteration directly (so the apply's plan and
    // tile shapes for k exist): capture it once and replay it from now on
    if (gExec_) {
      RSCHOL_CUDA(cudaGraphExecDestroy(gExec_));
      gExec_ = nullptr;
    }
    cudaGraph_t g = nullptr;
    RSCHOL_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      iteration();
    } catch (...) {
      cudaStreamEndCapture(st, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    RSCHOL_CUDA(cudaStreamEndCapture(st, &g));
    const cudaError_t ie = cudaGraphInstantiate(&gExec_, g, 0);
    cudaGraphDestroy(g);
    RSCHOL_CUDA(ie);
    gKey_ = key;
    RSCHOL_CUDA(cudaGraphLaunch(gExec_, st));
  } else {
    iteration();
  }
  lastKey_ = key;
  launches += 8;
  RSCHOL_CUDA(cudaMemcpyAsync(hsc_, sc, sizeof(double) * S_COUNT * k, cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  if (applyError_ && applyError_()) throw WaitTimeout();
  // 4. the stopping test of every column
  std::vector<int> fin;
  for (int j = 0; j < k; ++j) {
    Column& c = cols_[j];
    const double* h = hsc_ + (size_t)j * S_COUNT;
    ++c.iterations;
    c.residual = h[S_RREL];
    if (h[S_BREAK] != 0.0) c.breakdown = true;
    if (!(h[S_RREL] > c.eps) || c.breakdown || c.iterations >= c.maxit) {
      c.finished = true;
      fin.push_back(j);
    }
  }
  if (fin.empty()) return done;
  // 5. finished columns: true residual ||b - A x|| / ||b|| and x in the original order
  spmv_k(st, n, k, rp, ci, v, X, Q, part);
  residual_k(st, B, Q, n, k, part);
  finish_k_kernel<<<(k + 7) / 8, 256, 0, st>>>(part, BBLOCKS, k, sc, F_TRUE);
  ColMap fmap{};
  for (size_t c = 0; c < fin.size(); ++c) fmap.src[c] = fin[c];
  const long long nf = (long long)n * (long long)fin.size();
  extract_kernel<<<(unsigned)std::min<long long>((nf + BT - 1) / BT, BBLOCKS * 4), BT, 0, st>>>(
      n, k, (int)fin.size(), fmap, perm_, X, S);
  RSCHOL_LAUNCH_CHECK();
  launches += 4;
  for (size_t c = 0; c < fin.size(); ++c)
    RSCHOL_CUDA(cudaMemcpyAsync(cols_[fin[c]].xOut, S + c * (size_t)n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                st));
  // the true residuals land in S_RREL; the other scalars are as they were
  std::vector<double> rr(k);
  RSCHOL_CUDA(cudaMemcpyAsync(hsc_, sc, sizeof(double) * S_COUNT * k, cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  for (int j : fin) {
    cols_[j].trueResidual = hsc_[(size_t)j * S_COUNT + S_RREL];
    done.push_back(cols_[j]);
  }
  return done;
}

}  // namespace rschol
