// Batched PCG: k right-hand sides in lockstep on one factor (the c4 form of
// PCG_SOLVER::solvePCG, src/rschol/linearalgebra/PCG_SOLVER.cpp:226-363).
// Vectors are n x k row-major blocks; every kernel keeps one partial sum per
// column and block, reduced in a fixed order, so each column's arithmetic is
// reproducible.  A column that reaches its tolerance keeps alpha = 0 from
// then on (x and r frozen), as if its own loop had stopped.
#include <algorithm>
#include <cmath>

#include "pcg.cuh"

namespace rschol {

namespace {

constexpr int BT = 256;                 // threads per block
constexpr int BBLOCKS = 152 * 4;        // fixed grid of the vector kernels
constexpr int KMAX = 64;

enum { S_DELTA = 0, S_ALPHA, S_BETA, S_RREL, S_BNORM, S_DQ, S_ACTIVE, S_BREAK, S_FRESH, S_COUNT };
enum { F_ALPHA = 0, F_RNORM, F_BETA, F_DELTA0, F_BNORM, F_TRUE, F_SLOT };

// Per-column block sums: each thread holds up to two columns (lane, lane+32)
// of its rows; warps add in smem in warp order.  part[blockIdx.x * k + c].
__device__ void block_sum_cols(const double (&acc)[2], int k, double* part) {
  __shared__ double red[BT / 32][KMAX];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < 2; ++q)
    if (lane + 32 * q < k) red[warp][lane + 32 * q] = acc[q];
  __syncthreads();
  if (threadIdx.x < k) {
    double s = 0.0;
    for (int w = 0; w < BT / 32; ++w) s += red[w][threadIdx.x];
    part[(size_t)blockIdx.x * k + threadIdx.x] = s;
  }
}

// y = A x (a warp per row, lanes across the columns), and the partials of
// the column dots x . y.
__global__ void __launch_bounds__(BT) spmv_k_kernel(int n, int k, const int* __restrict__ rp,
                                                     const int* __restrict__ ci, const double* __restrict__ v,
                                                     const double* __restrict__ x, double* __restrict__ y,
                                                     double* __restrict__ part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[2] = {0.0, 0.0};
  for (int row = blockIdx.x * (BT / 32) + warp; row < n; row += gridDim.x * (BT / 32)) {
    double s[2] = {0.0, 0.0};
    for (int p = rp[row]; p < rp[row + 1]; ++p) {
      const double a = v[p];
      const double* xr = x + (size_t)ci[p] * k;
      for (int q = 0; q < 2; ++q)
        if (lane + 32 * q < k) s[q] += a * xr[lane + 32 * q];
    }
    for (int q = 0; q < 2; ++q)
      if (lane + 32 * q < k) {
        const size_t o = (size_t)row * k + lane + 32 * q;
        y[o] = s[q];
        acc[q] += x[o] * s[q];
      }
  }
  block_sum_cols(acc, k, part);
}

__global__ void __launch_bounds__(BT) dot_k_kernel(const double* __restrict__ a, const double* __restrict__ b, int n,
                                                   int k, double* __restrict__ part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[2] = {0.0, 0.0};
  for (int row = blockIdx.x * (BT / 32) + warp; row < n; row += gridDim.x * (BT / 32))
    for (int q = 0; q < 2; ++q)
      if (lane + 32 * q < k) {
        const size_t o = (size_t)row * k + lane + 32 * q;
        acc[q] += a[o] * b[o];
      }
  block_sum_cols(acc, k, part);
}

// Column scalars from the block partials (thread c: column c, fixed order).
__global__ void finish_k_kernel(const double* __restrict__ part, int count, int k, double* __restrict__ sc,
                                int mode) {
  const int c = threadIdx.x;
  if (c >= k) return;
  double t = 0.0;
  for (int b = 0; b < count; ++b) t += part[(size_t)b * k + c];
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

__global__ void __launch_bounds__(BT) update_xr_k_kernel(double* __restrict__ x, double* __restrict__ r,
                                                         const double* __restrict__ d, const double* __restrict__ q,
                                                         const double* __restrict__ sc, int n, int k,
                                                         double* __restrict__ part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double al[2] = {0.0, 0.0};
  for (int qq = 0; qq < 2; ++qq)
    if (lane + 32 * qq < k) al[qq] = sc[(size_t)(lane + 32 * qq) * S_COUNT + S_ALPHA];
  double acc[2] = {0.0, 0.0};
  for (int row = blockIdx.x * (BT / 32) + warp; row < n; row += gridDim.x * (BT / 32))
    for (int qq = 0; qq < 2; ++qq)
      if (lane + 32 * qq < k) {
        const size_t o = (size_t)row * k + lane + 32 * qq;
        x[o] += al[qq] * d[o];
        const double ri = r[o] - al[qq] * q[o];
        r[o] = ri;
        acc[qq] += ri * ri;
      }
  block_sum_cols(acc, k, part);
}

__global__ void __launch_bounds__(BT) update_d_k_kernel(double* __restrict__ d, const double* __restrict__ s,
                                                        const double* __restrict__ sc, int n, int k) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double be[2] = {0.0, 0.0};
  for (int qq = 0; qq < 2; ++qq)
    if (lane + 32 * qq < k) be[qq] = sc[(size_t)(lane + 32 * qq) * S_COUNT + S_BETA];
  for (int row = blockIdx.x * (BT / 32) + warp; row < n; row += gridDim.x * (BT / 32))
    for (int qq = 0; qq < 2; ++qq)
      if (lane + 32 * qq < k) {
        const size_t o = (size_t)row * k + lane + 32 * qq;
        d[o] = s[o] + be[qq] * d[o];
      }
}

__global__ void __launch_bounds__(BT) residual_k_kernel(const double* __restrict__ b, const double* __restrict__ q,
                                                        int n, int k, double* __restrict__ part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double acc[2] = {0.0, 0.0};
  for (int row = blockIdx.x * (BT / 32) + warp; row < n; row += gridDim.x * (BT / 32))
    for (int qq = 0; qq < 2; ++qq)
      if (lane + 32 * qq < k) {
        const size_t o = (size_t)row * k + lane + 32 * qq;
        const double e = b[o] - q[o];
        acc[qq] += e * e;
      }
  block_sum_cols(acc, k, part);
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
  dot_k_kernel<<<BBLOCKS, BT, 0, st>>>(B, B, n, k, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_BNORM);
  RSCHOL_CUDA(cudaMemcpyAsync(s, r, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
  apply(s);
  dot_k_kernel<<<BBLOCKS, BT, 0, st>>>(r, s, n, k, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_DELTA0);
  RSCHOL_CUDA(cudaMemcpyAsync(d, s, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
  RSCHOL_LAUNCH_CHECK();
  launches += 4;
  std::vector<char> active(k, 1);
  int nActive = k, i = 0;
  while (i < maxit && nActive > 0) {
    spmv_k_kernel<<<BBLOCKS, BT, 0, st>>>(n, k, rp, ci, v, d, q, part);
    finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_ALPHA);
    update_xr_k_kernel<<<BBLOCKS, BT, 0, st>>>(X, r, d, q, sc, n, k, part);
    finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_RNORM);
    RSCHOL_CUDA(cudaMemcpyAsync(s, r, sizeof(double) * nk, cudaMemcpyDeviceToDevice, st));
    apply(s);
    dot_k_kernel<<<BBLOCKS, BT, 0, st>>>(r, s, n, k, part);
    finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_BETA);
    update_d_k_kernel<<<BBLOCKS, BT, 0, st>>>(d, s, sc, n, k);
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
  spmv_k_kernel<<<BBLOCKS, BT, 0, st>>>(n, k, rp, ci, v, X, q, part);
  residual_k_kernel<<<BBLOCKS, BT, 0, st>>>(B, q, n, k, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_TRUE);
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
                       std::function<void(double*, int)> apply, std::function<int()> applyError)
    : pcg_(pcg), kmax_(kmax), perm_(dPerm), apply_(std::move(apply)), applyError_(std::move(applyError)) {
  if (kmax < 1 || kmax > KMAX) throw std::runtime_error("PcgSession: 1..64 columns");
  part_.alloc(sizeof(double) * BBLOCKS * kmax);
  sc_.alloc(sizeof(double) * S_COUNT * kmax);
  RSCHOL_CUDA(cudaMallocHost((void**)&hsc_, sizeof(double) * S_COUNT * kmax));
  hscNew_.assign((size_t)S_COUNT * kmax, 0.0);
}

PcgSession::~PcgSession() {
  if (hsc_) cudaFreeHost(hsc_);
}

// The column blocks grow (doubling, up to kmax) when more columns are active
// than they hold; they never shrink while the session lives.
void PcgSession::reserve_set(int set, int k) {
  if (cap_[set] >= k) return;
  const size_t nk = sizeof(double) * std::max<size_t>(1, (size_t)pcg_.n * k);
  for (auto* v : {&x_[set], &r_[set], &d_[set], &b_[set]}) v->alloc(nk);
  cap_[set] = k;
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
        dot_k_kernel<<<BBLOCKS, BT, 0, st>>>(b_[cur_].as<double>(), b_[cur_].as<double>(), n, k, part_.as<double>());
        finish_k_kernel<<<1, KMAX, 0, st>>>(part_.as<double>(), BBLOCKS, k, sc_.as<double>(), F_BNORM);
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
  // 2. s = M^{-1} r; t = r.s; d = s + beta d
  RSCHOL_CUDA(cudaMemcpyAsync(S, R, nkBytes, cudaMemcpyDeviceToDevice, st));
  apply_(S, k);
  dot_k_kernel<<<BBLOCKS, BT, 0, st>>>(R, S, n, k, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_SLOT);
  update_d_k_kernel<<<BBLOCKS, BT, 0, st>>>(D, S, sc, n, k);
  // 3. q = A d; alpha; x += alpha d; r -= alpha q; ||r|| / ||b||
  spmv_k_kernel<<<BBLOCKS, BT, 0, st>>>(n, k, rp, ci, v, D, Q, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_ALPHA);
  update_xr_k_kernel<<<BBLOCKS, BT, 0, st>>>(X, R, D, Q, sc, n, k, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_RNORM);
  RSCHOL_LAUNCH_CHECK();
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
  spmv_k_kernel<<<BBLOCKS, BT, 0, st>>>(n, k, rp, ci, v, X, Q, part);
  residual_k_kernel<<<BBLOCKS, BT, 0, st>>>(B, Q, n, k, part);
  finish_k_kernel<<<1, KMAX, 0, st>>>(part, BBLOCKS, k, sc, F_TRUE);
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
