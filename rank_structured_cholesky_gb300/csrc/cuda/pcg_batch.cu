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

enum { S_DELTA = 0, S_ALPHA, S_BETA, S_RREL, S_BNORM, S_DQ, S_ACTIVE, S_BREAK, S_COUNT };
enum { F_ALPHA = 0, F_RNORM, F_BETA, F_DELTA0, F_BNORM, F_TRUE };

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

}  // namespace rschol
