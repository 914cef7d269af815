// Batched dense kernels (FP64 and FP32 instantiations).
#include <cfloat>
#include <climits>

#include "common.cuh"
#include "dense.cuh"

namespace rschol {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, GEMM_THREADS = 256;

template <class T>
__global__ void __launch_bounds__(GEMM_THREADS) gemm_kernel(const GemmTask<T>* __restrict__ tasks, int nTasks) {
  int lo = 0, hi = nTasks - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].tileBase <= b) lo = mid;
    else hi = mid - 1;
  }
  const GemmTask<T> t = tasks[lo];
  const int local = b - t.tileBase;
  const int ti = local / t.tilesN, tj = local - ti * t.tilesN;
  const int row0 = ti * BM, col0 = tj * BN;
  if (t.lower && row0 + BM - 1 < col0) return;

  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);

  for (int k0 = 0; k0 < t.K; k0 += BK) {
    if (!t.tA) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int i = (tid >> 4) + 16 * q, k = tid & 15;
        int gi = row0 + i, gk = k0 + k;
        As[k][i] = (gi < t.M && gk < t.K) ? t.A[(size_t)gi * t.lda + gk] : T(0);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int i = tid & 63, k = (tid >> 6) + 4 * q;
        int gi = row0 + i, gk = k0 + k;
        As[k][i] = (gi < t.M && gk < t.K) ? t.A[(size_t)gk * t.lda + gi] : T(0);
      }
    }
    if (!t.tB) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int j = tid & 63, k = (tid >> 6) + 4 * q;
        int gj = col0 + j, gk = k0 + k;
        Bs[k][j] = (gj < t.N && gk < t.K) ? t.B[(size_t)gk * t.ldb + gj] : T(0);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        int j = (tid >> 4) + 16 * q, k = tid & 15;
        int gj = col0 + j, gk = k0 + k;
        Bs[k][j] = (gj < t.N && gk < t.K) ? t.B[(size_t)gj * t.ldb + gk] : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gi = row0 + ty + 16 * i;
    if (gi >= t.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gj = col0 + tx + 16 * j;
      if (gj >= t.N) continue;
      T* c = t.C + (size_t)gi * t.ldc + gj;
      T v = t.alpha * acc[i][j];
      if (t.beta != T(0)) v = fma(t.beta, *c, v);
      *c = v;
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256) potrf_kernel(const PotrfTask<T>* __restrict__ tasks, int* flag) {
  const PotrfTask<T> t = tasks[blockIdx.x];
  __shared__ T a[64][65];
  __shared__ int bad;
  const int n = t.n, tid = threadIdx.x;
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    int i = idx / n, j = idx - i * n;
    a[i][j] = (j <= i) ? t.A[(size_t)i * t.ld + j] : T(0);
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {
      T d = a[j][j];
      if (!(d > T(0))) {   // not positive definite (or NaN): keep going, report
        bad = 1;
        d = T(1);
      }
      a[j][j] = sqrt(d);
    }
    __syncthreads();
    const T djj = a[j][j];
    for (int i = j + 1 + tid; i < n; i += blockDim.x) a[i][j] /= djj;
    __syncthreads();
    const int m = n - j - 1;
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      int ii = idx / m, kk = idx - ii * m;
      if (kk <= ii) a[j + 1 + ii][j + 1 + kk] -= a[j + 1 + ii][j] * a[j + 1 + kk][j];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    int i = idx / n, j = idx - i * n;
    if (j <= i) t.A[(size_t)i * t.ld + j] = a[i][j];
  }
  if (tid == 0 && bad) atomicMin(flag, t.code);
}

template <class T>
__global__ void __launch_bounds__(256) trsm_kernel(const TrsmTask<T>* __restrict__ tasks, int nTasks) {
  int lo = 0, hi = nTasks - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].chunkBase <= b) lo = mid;
    else hi = mid - 1;
  }
  const TrsmTask<T> t = tasks[lo];
  const int r0 = (b - t.chunkBase) * 64;
  const int nr = min(64, t.rows - r0);
  const int w = t.w, tid = threadIdx.x;
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  T (*L)[65] = reinterpret_cast<T (*)[65]>(trsm_smem);
  T (*X)[65] = reinterpret_cast<T (*)[65]>(trsm_smem + sizeof(T) * 64 * 65);
  for (int idx = tid; idx < w * w; idx += blockDim.x) {
    int i = idx / w, j = idx - i * w;
    L[i][j] = (j <= i) ? t.L[(size_t)i * t.ldl + j] : T(0);
  }
  for (int idx = tid; idx < nr * w; idx += blockDim.x) {
    int i = idx / w, j = idx - i * w;
    X[i][j] = t.B[(size_t)(r0 + i) * t.ldb + j];
  }
  __syncthreads();
  for (int j = 0; j < w; ++j) {
    const T d = L[j][j];
    for (int i = tid; i < nr; i += blockDim.x) X[i][j] /= d;
    __syncthreads();
    const int rem = w - j - 1;
    for (int idx = tid; idx < nr * rem; idx += blockDim.x) {
      int i = idx / rem, k = j + 1 + (idx - i * rem);
      X[i][k] -= X[i][j] * L[k][j];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < nr * w; idx += blockDim.x) {
    int i = idx / w, j = idx - i * w;
    t.B[(size_t)(r0 + i) * t.ldb + j] = X[i][j];
  }
}

template <class T>
__global__ void __launch_bounds__(256) extadd_kernel(const ExtAddTarget<T>* __restrict__ tg, int nT,
                                                     const ExtAddSource<T>* __restrict__ src) {
  int lo = 0, hi = nT - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tg[mid].colBase <= b) lo = mid;
    else hi = mid - 1;
  }
  const ExtAddTarget<T> t = tg[lo];
  const int col = b - t.colBase;
  for (int s = t.srcBegin; s < t.srcEnd; ++s) {
    const ExtAddSource<T> S = src[s];
    const int sb = S.colInv[col];
    if (sb < 0) continue;   // uniform across the block
    const int a0 = S.lowerOnly ? sb : 0;
    for (int a = a0 + threadIdx.x; a < S.nrows; a += blockDim.x) {
      T* dst = t.F + (size_t)S.rowRel[a] * t.ld + col;
      *dst = fma(S.sign, S.D[(size_t)a * S.ld + sb], *dst);
    }
    __syncthreads();   // the next source may hit the same target rows
  }
}

template <class T>
__global__ void scatter_kernel(const double* __restrict__ Avals, const long long* __restrict__ srcIdx,
                               const long long* __restrict__ dstIdx, long long count, T* __restrict__ dst) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x)
    dst[dstIdx[k]] = (T)Avals[srcIdx[k]];
}

constexpr int QR_THREADS = 512;

template <class R>
__device__ __forceinline__ R warp_sum_d(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum, broadcast to every thread.
template <class R>
__device__ R block_sum_bcast(R v, R* red) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    R t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : R(0);
    t = warp_sum_d(t);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// Householder QR (LAPACK dgeqr2: dlarfg reflectors with v_0 = 1) followed by
// the explicit thin Q (dorg2r), on a column-major copy of Y.
template <class T>
__global__ void __launch_bounds__(QR_THREADS) householder_qr_kernel(const QrTask<T>* __restrict__ tasks) {
  const QrTask<T> t = tasks[blockIdx.x];
  const int n = t.n, r = t.r;
  T* W = t.W;
  T* tau = W + (size_t)r * n;
  __shared__ T red[33];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (long long idx = tid; idx < (long long)n * r; idx += blockDim.x) {
    const int i = (int)(idx / r), j = (int)(idx - (long long)i * r);
    W[(size_t)j * n + i] = t.Y[idx];
  }
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    T* ck = W + (size_t)k * n;
    T s = T(0);
    for (int i = k + 1 + tid; i < n; i += blockDim.x) s += ck[i] * ck[i];
    const T xnorm2 = block_sum_bcast<T>(s, red);
    const T alpha = ck[k];
    T tk = T(0), beta = alpha, scal = T(0);
    if (xnorm2 > T(0)) {
      beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
      tk = (beta - alpha) / beta;
      scal = T(1) / (alpha - beta);
    }
    __syncthreads();
    if (xnorm2 > T(0))
      for (int i = k + 1 + tid; i < n; i += blockDim.x) ck[i] = ck[i] * scal;
    if (tid == 0) {
      ck[k] = beta;
      tau[k] = tk;
    }
    __syncthreads();
    if (tk != T(0)) {
      for (int j = k + 1 + warp; j < r; j += nw) {
        T* cj = W + (size_t)j * n;
        T w = T(0);
        for (int i = k + 1 + lane; i < n; i += 32) w += ck[i] * cj[i];
        w = warp_sum_d<T>(w);
        const T cjk = cj[k];
        __syncwarp();
        w = tk * (w + cjk);
        if (lane == 0) cj[k] = cjk - w;
        for (int i = k + 1 + lane; i < n; i += 32) cj[i] = cj[i] - w * ck[i];
      }
    }
    __syncthreads();
  }
  for (int k = r - 1; k >= 0; --k) {
    T* ck = W + (size_t)k * n;
    const T tk = tau[k];
    if (tk != T(0)) {
      for (int j = k + 1 + warp; j < r; j += nw) {
        T* cj = W + (size_t)j * n;
        T w = T(0);
        for (int i = k + 1 + lane; i < n; i += 32) w += ck[i] * cj[i];
        w = warp_sum_d<T>(w);
        const T cjk = cj[k];
        __syncwarp();
        w = tk * (w + cjk);
        if (lane == 0) cj[k] = cjk - w;
        for (int i = k + 1 + lane; i < n; i += 32) cj[i] = cj[i] - w * ck[i];
      }
    }
    __syncthreads();
    for (int i = k + 1 + tid; i < n; i += blockDim.x) ck[i] = -tk * ck[i];
    for (int i = tid; i < k; i += blockDim.x) ck[i] = T(0);
    if (tid == 0) ck[k] = T(1) - tk;
    __syncthreads();
  }
  for (long long idx = tid; idx < (long long)n * r; idx += blockDim.x) {
    const int i = (int)(idx / r), j = (int)(idx - (long long)i * r);
    t.Y[idx] = W[(size_t)j * n + i];
  }
}

template <class T>
__global__ void set_identity_kernel(const IdentTask<T>* __restrict__ tasks) {
  const IdentTask<T> t = tasks[blockIdx.y];
  T* U = t.U;
  const int n = t.n, ld = t.ld;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < (long long)n * n;
       k += (long long)gridDim.x * blockDim.x) {
    int i = (int)(k / n), j = (int)(k - (long long)i * n);
    U[(size_t)i * ld + j] = (i == j) ? T(1) : T(0);
  }
}

template <class T>
__global__ void box_muller_kernel(const uint32_t* __restrict__ raw, long long count, T* __restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x) {
    const double u1 = ((double)raw[2 * k] + 0.5) * (1.0 / 4294967296.0);
    const double u2 = (double)raw[2 * k + 1] * (1.0 / 4294967296.0);
    const double r = sqrt(-2.0 * log(1.0 - u1));
    const double phi = 2.0 * 3.14159265358979323846264338328 * u2;
    out[k] = (T)(r * cos(phi));
  }
}

int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g > 152LL * 32) g = 152LL * 32;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

template <class T> void launch_gemm(const GemmTask<T>* d, int n, int tiles, cudaStream_t s) {
  if (n <= 0 || tiles <= 0) return;
  gemm_kernel<T><<<tiles, GEMM_THREADS, 0, s>>>(d, n);
  RSCHOL_LAUNCH_CHECK();
}
template <class T> void launch_potrf(const PotrfTask<T>* d, int n, int* flag, cudaStream_t s) {
  if (n <= 0) return;
  potrf_kernel<T><<<n, 256, 0, s>>>(d, flag);
  RSCHOL_LAUNCH_CHECK();
}
template <class T> void launch_trsm(const TrsmTask<T>* d, int n, int chunks, cudaStream_t s) {
  if (n <= 0 || chunks <= 0) return;
  const int smem = (int)(2 * sizeof(T) * 64 * 65);
  static bool configured = false;   // per instantiation
  if (!configured) {
    RSCHOL_CUDA(cudaFuncSetAttribute(trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    configured = true;
  }
  trsm_kernel<T><<<chunks, 256, smem, s>>>(d, n);
  RSCHOL_LAUNCH_CHECK();
}
template <class T>
void launch_extadd(const ExtAddTarget<T>* tg, int nT, const ExtAddSource<T>* src, int cols, cudaStream_t s) {
  if (nT <= 0 || cols <= 0) return;
  extadd_kernel<T><<<cols, 128, 0, s>>>(tg, nT, src);
  RSCHOL_LAUNCH_CHECK();
}
template <class T>
void launch_scatter(const double* A, const long long* si, const long long* di, long long count, T* dst,
                    cudaStream_t s) {
  if (count <= 0) return;
  scatter_kernel<T><<<grid_for(count, 256), 256, 0, s>>>(A, si, di, count, dst);
  RSCHOL_LAUNCH_CHECK();
}
template <class T> void launch_householder_qr(const QrTask<T>* d, int n, cudaStream_t s) {
  if (n <= 0) return;
  householder_qr_kernel<T><<<n, QR_THREADS, 0, s>>>(d);
  RSCHOL_LAUNCH_CHECK();
}
template <class T> void launch_set_identity(const IdentTask<T>* d, int n, cudaStream_t s) {
  if (n <= 0) return;
  set_identity_kernel<T><<<dim3(64, n), 256, 0, s>>>(d);
  RSCHOL_LAUNCH_CHECK();
}
template <class T> void launch_box_muller(const uint32_t* raw, long long count, T* out, cudaStream_t s) {
  if (count <= 0) return;
  box_muller_kernel<T><<<grid_for(count, 256), 256, 0, s>>>(raw, count, out);
  RSCHOL_LAUNCH_CHECK();
}

#define RSCHOL_INST(T)                                                                                   \
  template void launch_gemm<T>(const GemmTask<T>*, int, int, cudaStream_t);                              \
  template void launch_potrf<T>(const PotrfTask<T>*, int, int*, cudaStream_t);                           \
  template void launch_trsm<T>(const TrsmTask<T>*, int, int, cudaStream_t);                              \
  template void launch_extadd<T>(const ExtAddTarget<T>*, int, const ExtAddSource<T>*, int, cudaStream_t); \
  template void launch_scatter<T>(const double*, const long long*, const long long*, long long, T*,      \
                                  cudaStream_t);                                                         \
  template void launch_householder_qr<T>(const QrTask<T>*, int, cudaStream_t);                           \
  template void launch_set_identity<T>(const IdentTask<T>*, int, cudaStream_t);                          \
  template void launch_box_muller<T>(const uint32_t*, long long, T*, cudaStream_t);
RSCHOL_INST(double)
RSCHOL_INST(float)

}  // namespace rschol
