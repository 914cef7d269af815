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
  __shared__ T L[64][65];
  __shared__ T X[64][65];
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

template <class T> struct Unit;
template <> struct Unit<double> { static __device__ double v() { return 1.1102230246251565e-16; } };
template <> struct Unit<float> { static __device__ float v() { return 5.9604645e-08f; } };

template <class T>
__global__ void shift_diag_kernel(const ShiftTask<T>* __restrict__ tasks) {
  const ShiftTask<T> t = tasks[blockIdx.x];
  T* G = t.G;
  const int r = t.r, ld = t.ld, rows = t.rows;
  __shared__ double part[256];
  double s = 0;
  for (int i = threadIdx.x; i < r; i += blockDim.x) s += (double)G[(size_t)i * ld + i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  const double shift = 11.0 * ((double)rows * r + (double)r * (r + 1)) * (double)Unit<T>::v() * part[0];
  for (int i = threadIdx.x; i < r; i += blockDim.x) G[(size_t)i * ld + i] += (T)shift;
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
  trsm_kernel<T><<<chunks, 256, 0, s>>>(d, n);
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
template <class T> void launch_shift_diag(const ShiftTask<T>* d, int n, cudaStream_t s) {
  if (n <= 0) return;
  shift_diag_kernel<T><<<n, 256, 0, s>>>(d);
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
  template void launch_shift_diag<T>(const ShiftTask<T>*, int, cudaStream_t);                            \
  template void launch_set_identity<T>(const IdentTask<T>*, int, cudaStream_t);                          \
  template void launch_box_muller<T>(const uint32_t*, long long, T*, cudaStream_t);
RSCHOL_INST(double)
RSCHOL_INST(float)

}  // namespace rschol
