// Batched dense kernels (FP64 and FP32 instantiations).
#include <algorithm>
#include <cfloat>
#include <climits>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "dense.cuh"
#include "solve_dev.cuh"

namespace rschol {

namespace {

using solvedev::st_release;
using solvedev::wait_geq;
using solvedev::wait_geq_lim;

constexpr int BM = 64, BN = 64, BK = 16, GEMM_THREADS = 256;

// One 64 x 64 tile of C = alpha op(A) op(B) + beta C at (row0, col0), by
// the 256 threads of the block.  Two shared stages: the next K slice is
// loaded into registers while the current one is multiplied (one barrier per
// slice); C is fetched before the K loop.  Each C entry's K order is the
// plain ascending one.
template <class T>
__device__ void gemm_tile(const GemmTask<T>& t, int row0, int col0, T (*As)[BK][BM + 1], T (*Bs)[BK][BN + 1]) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
  T cpre[4][4];
  if (t.beta != T(0)) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int gi = row0 + ty + 16 * i, gj = col0 + tx + 16 * j;
        cpre[i][j] = (gi < t.M && gj < t.N) ? __ldcg(t.C + (size_t)gi * t.ldc + gj) : T(0);
      }
  }
  T ra[4], rb[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int i, k;
      if (!t.tA) { i = (tid >> 4) + 16 * q; k = tid & 15; }
      else { i = tid & 63; k = (tid >> 6) + 4 * q; }
      const int gi = row0 + i, gk = k0 + k;
      ra[q] = (gi < t.M && gk < t.K) ? __ldcg(t.tA ? t.A + (size_t)gk * t.lda + gi : t.A + (size_t)gi * t.lda + gk)
                                       : T(0);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int j, k;
      if (!t.tB) { j = tid & 63; k = (tid >> 6) + 4 * q; }
      else { j = (tid >> 4) + 16 * q; k = tid & 15; }
      const int gj = col0 + j, gk = k0 + k;
      rb[q] = (gj < t.N && gk < t.K) ? __ldcg(t.tB ? t.B + (size_t)gj * t.ldb + gk : t.B + (size_t)gk * t.ldb + gj)
                                       : T(0);
    }
  };
  auto store = [&](int st) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int i, k;
      if (!t.tA) { i = (tid >> 4) + 16 * q; k = tid & 15; }
      else { i = tid & 63; k = (tid >> 6) + 4 * q; }
      As[st][k][i] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int j, k;
      if (!t.tB) { j = tid & 63; k = (tid >> 6) + 4 * q; }
      else { j = (tid >> 4) + 16 * q; k = tid & 15; }
      Bs[st][k][j] = rb[q];
    }
  };
  if (t.K > 0) {
    load(0);
    store(0);
  }
  __syncthreads();
  int st = 0;
  for (int k0 = 0; k0 < t.K; k0 += BK) {
    const bool more = k0 + BK < t.K;
    if (more) load(k0 + BK);
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[st][k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = Bs[st][k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
    }
    if (more) store(st ^ 1);
    __syncthreads();
    st ^= 1;
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
      if (t.beta != T(0)) v = fma(t.beta, cpre[i][j], v);
      *c = v;
    }
  }
}

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
  __shared__ T As[2][BK][BM + 1];
  __shared__ T Bs[2][BK][BN + 1];
  gemm_tile<T>(t, row0, col0, As, Bs);
}

template <class T>
__global__ void __launch_bounds__(256) potrf_kernel(const PotrfTask<T>* __restrict__ tasks, int* flag) {
  // Right-looking Cholesky of one <= 64 x 64 tile in 16-column panels: one
  // warp factors the panel's diagonal block, every thread solves a row of
  // the panel below it, then all threads update the trailing triangle.
  const PotrfTask<T> t = tasks[blockIdx.x];
  __shared__ T a[64][65];
  __shared__ int bad;
  const int n = t.n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    a[i][j] = (j <= i) ? t.A[(size_t)i * t.ld + j] : T(0);
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int p0 = 0; p0 < n; p0 += 16) {
    const int pw = min(16, n - p0);
    if (warp == 0) {
      for (int j = 0; j < pw; ++j) {
        const int jj = p0 + j;
        if (lane == 0) {
          T d = a[jj][jj];
          if (!(d > T(0))) {   // not positive definite (or NaN): keep going, report
            bad = 1;
            d = T(1);
          }
          a[jj][jj] = sqrt(d);
        }
        __syncwarp();
        if (lane > j && lane < pw) a[p0 + lane][jj] /= a[jj][jj];
        __syncwarp();
        if (lane > j && lane < pw) {
          const T lij = a[p0 + lane][jj];
          for (int k = j + 1; k <= lane; ++k) a[p0 + lane][p0 + k] -= lij * a[p0 + k][jj];
        }
        __syncwarp();
      }
    }
    __syncthreads();
    for (int i = p0 + pw + tid; i < n; i += blockDim.x)
      for (int j = 0; j < pw; ++j) {
        T s = a[i][p0 + j];
        for (int k = 0; k < j; ++k) s -= a[i][p0 + k] * a[p0 + j][p0 + k];
        a[i][p0 + j] = s / a[p0 + j][p0 + j];
      }
    __syncthreads();
    const int q0 = p0 + pw, m = n - q0;
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      const int ii = idx / m, kk = idx - ii * m;
      if (kk <= ii) {
        T s = T(0);
        for (int c = 0; c < pw; ++c) s += a[q0 + ii][p0 + c] * a[q0 + kk][p0 + c];
        a[q0 + ii][q0 + kk] -= s;
      }
    }
    __syncthreads();
  }
  for (int idx = tid; idx < n * n; idx += blockDim.x) {
    const int i = idx / n, j = idx - i * n;
    if (j <= i) t.A[(size_t)i * t.ld + j] = a[i][j];
  }
  if (tid == 0 && bad) atomicMin(flag, t.code);
}

template <class T>
__global__ void __launch_bounds__(256) trsm_kernel(const TrsmTask<T>* __restrict__ tasks, int nTasks) {
  // B (64-row chunk x w) := B L^{-T} in 16-column panels: each row solves
  // with the panel's diagonal block (16 steps), then all threads update the
  // columns to the right.
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
    const int i = idx / w, j = idx - i * w;
    L[i][j] = (j <= i) ? t.L[(size_t)i * t.ldl + j] : T(0);
  }
  for (int idx = tid; idx < nr * w; idx += blockDim.x) {
    const int i = idx / w, j = idx - i * w;
    X[i][j] = t.B[(size_t)(r0 + i) * t.ldb + j];
  }
  __syncthreads();
  for (int p0 = 0; p0 < w; p0 += 16) {
    const int pw = min(16, w - p0);
    if (tid < nr)
      for (int j = 0; j < pw; ++j) {
        T s = X[tid][p0 + j];
        for (int k = 0; k < j; ++k) s -= X[tid][p0 + k] * L[p0 + j][p0 + k];
        X[tid][p0 + j] = s / L[p0 + j][p0 + j];
      }
    __syncthreads();
    const int q0 = p0 + pw, wq = w - q0;
    for (int idx = tid; idx < nr * wq; idx += blockDim.x) {
      const int i = idx / wq, q = q0 + (idx - i * wq);
      T s = T(0);
      for (int c = 0; c < pw; ++c) s += X[i][p0 + c] * L[q][p0 + c];
      X[i][q] -= s;
    }
    __syncthreads();
  }
  for (int idx = tid; idx < nr * w; idx += blockDim.x) {
    const int i = idx / w, j = idx - i * w;
    t.B[(size_t)(r0 + i) * t.ldb + j] = X[i][j];
  }
}

// FP32 variants: a register-resident POTRF (thread (i, g) keeps row i,
// columns g, g + 4, ... of the tile) and a TRSM that inverts the tile in
// every block and multiplies; they beat the panel-blocked kernels above in
// FP32, while FP64 prefers the blocked ones.  The tile bodies are device
// functions shared with the fused level kernel below.

// Right-looking Cholesky of one n x n (n <= 64) tile at A (row-major, ld) by
// the block's 256 threads as a 16 x 16 grid: thread (ti, tk) keeps the 4 x 4
// entries (ti + 16 a, tk + 16 b) in registers.  Column j is published
// unscaled (u_i = a_ij for i > j, zeros at rows <= j; the pivot p = a_jj
// apart) through a double-buffered shared vector laid out by (i % 16, i / 16),
// so one barrier per column suffices and a thread reads its four row values
// and its four column values as two 16-byte loads; every thread then runs
// the same 16 unpredicated FMAs a_ik -= (u_i / p) u_k (the zeros leave
// finished entries unchanged; entries right of the diagonal are never
// stored).  Finally L_jj = sqrt(p_j), L_ij = a_ij / sqrt(p_j).  A
// non-positive pivot is replaced by 1 and reported as atomicMin(flag, code).
// 1 / p on a POTRF's critical path: the fast reciprocal (MUFU-based,
// __fdividef, within 2 ulp) in FP32, whose factor carries larger rounding
// errors anyway; exact division in FP64.
__device__ __forceinline__ float pivot_recip(float p) { return __fdividef(1.0f, p); }
__device__ __forceinline__ double pivot_recip(double p) { return 1.0 / p; }

template <class T>
__device__ void potrf_tile_reg(T* A, int ld, int n, int code, int* flag) {
  __shared__ __align__(16) T col[2][64];
  __shared__ T piv[64];
  __shared__ int bad;
  const int tid = threadIdx.x, ti = tid >> 4, tk = tid & 15;
  T v[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = ti + 16 * a, k = tk + 16 * b;
      v[a][b] = (i < n && k <= i) ? __ldcg(A + (size_t)i * ld + k) : T(0);
    }
  if (tid == 0) bad = 0;
  __syncthreads();
#pragma unroll
  for (int b0 = 0; b0 < 4; ++b0) {
#pragma unroll 1
    for (int jj = 0; jj < 16; ++jj) {
      const int j = 16 * b0 + jj;
      if (j >= n) break;
      T* cj = col[j & 1];
      if (tk == jj) {   // the owners of column j: rows ti + 16 a
        T u[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const int i = ti + 16 * a;
          u[a] = v[a][b0];
          if (i == j) {
            T p = u[a];
            if (!(p > T(0))) {   // not positive definite (or NaN): keep going, report
              bad = 1;
              p = T(1);
            }
            piv[j] = p;
          }
          if (i <= j) u[a] = T(0);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) cj[4 * ti + a] = u[a];
      }
      __syncthreads();
      const T rp = pivot_recip(piv[j]);
      T ur[4], uc[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        ur[a] = cj[4 * ti + a] * rp;
        uc[a] = cj[4 * tk + a];
      }
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) v[a][b] -= ur[a] * uc[b];
    }
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = ti + 16 * a, k = tk + 16 * b;
      if (i < n && k <= i) {
        const T d = sqrt(piv[k]);
        A[(size_t)i * ld + k] = (k == i) ? d : v[a][b] / d;
      }
    }
  if (tid == 0 && bad) atomicMin(flag, code);
  __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(256) potrf_reg_kernel(const PotrfTask<T>* __restrict__ tasks, int* flag) {
  const PotrfTask<T> t = tasks[blockIdx.x];
  potrf_tile_reg<T>(t.A, t.ld, t.n, t.code, flag);
}

// Li := L^{-1}, L the w x w lower tile at Lg (ld ldl) padded to 64 with a
// unit diagonal (so the leading w x w block of Li is the inverse; only the
// 16 x 16 blocks that cover it are formed).  Blocked: the 16 x 16 diagonal
// inverses by forward substitution (warp b inverts block b, lane c keeps
// column c in registers, the diagonal reciprocals formed up front), then the
// off-diagonal blocks by distance from the diagonal,
// Li[R][C] = -Li[R][R] sum_{K=C}^{R-1} L[R][K] Li[K][C], with unrolled
// fixed-length inner products.  L, Li: 64 x 65 shared; Tm: 3 x 16 x 17
// shared.  256 threads.
template <class T>
__device__ void tile_inverse(const T* Lg, int ldl, int w, T (*L)[65], T (*Li)[65], T (*Tm)[16][17]) {
  const int tid = threadIdx.x;
  // tile loads unrolled: all 16 loads of a thread in flight at once
#pragma unroll
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int i = idx >> 6, j = idx & 63;
    L[i][j] = (i < w && j <= i) ? __ldcg(Lg + (size_t)i * ldl + j) : (i == j ? T(1) : T(0));
    Li[i][j] = T(0);
  }
  __syncthreads();
  const int nb = (w + 15) >> 4;   // 16 x 16 blocks that cover the w x w inverse
  {
    const int wb = tid >> 5, c = tid & 15;
    if (wb < nb && (tid & 31) < 16) {
      const int o = 16 * wb;
      T d[16], x[16];
#pragma unroll
      for (int r = 0; r < 16; ++r) d[r] = T(1) / L[o + r][o + r];
      // x = column c of the block inverse: x_r = (delta_rc - sum_{k<r} L_rk x_k) / L_rr;
      // rows above c come out zero by themselves
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        T s = (r == c) ? T(1) : T(0);
#pragma unroll
        for (int k = 0; k < r; ++k) s -= L[o + r][o + k] * x[k];
        x[r] = s * d[r];
      }
#pragma unroll
      for (int r = 0; r < 16; ++r) Li[o + r][o + c] = x[r];
    }
  }
  __syncthreads();
#pragma unroll
  for (int d = 1; d < 4; ++d) {
    if (d >= nb) break;
    const int np = nb - d;   // block pairs (R, C = R - d)
    for (int e = tid; e < np * 256; e += 256) {
      const int pr = e >> 8, i = (e >> 4) & 15, j = e & 15;
      const int C = pr, R = pr + d;
      T s = T(0);
#pragma unroll
      for (int k = 0; k < 16 * d; ++k) s += L[16 * R + i][16 * C + k] * Li[16 * C + k][16 * C + j];
      Tm[pr][i][j] = s;
    }
    __syncthreads();
    for (int e = tid; e < np * 256; e += 256) {
      const int pr = e >> 8, i = (e >> 4) & 15, j = e & 15;
      const int C = pr, R = pr + d;
      T s = T(0);
#pragma unroll
      for (int k = 0; k < 16; ++k) s += Li[16 * R + i][16 * R + k] * Tm[pr][k][j];   // Li[R][R] is lower
      Li[16 * R + i][16 * C + j] = -s;
    }
    __syncthreads();
  }
}

// B (nr <= 64 rows x w) := B Li^T with Li = L^{-1} (64 x 65 shared, zero
// above the diagonal); X: 64 x 65 shared staging.  256 threads.
template <class T>
__device__ void trsm_chunk_mul(T* B, int ldb, int nr, int w, T (*X)[65], T (*Li)[65]) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int idx = tid; idx < 64 * 64; idx += 256) {
    const int i = idx >> 6, j = idx & 63;
    X[i][j] = (i < nr && j < w) ? __ldcg(B + (size_t)i * ldb + j) : T(0);
  }
  __syncthreads();
  // out[i][j] = sum_{k <= j} X[i][k] Li[j][k]; thread: rows ty + 16 a, columns tx + 16 c
  const int tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[a][c] = T(0);
#pragma unroll 4
  for (int k = 0; k < w; ++k) {
    T xa[4], lb[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) xa[a] = X[ty + 16 * a][k];
#pragma unroll
    for (int c = 0; c < 4; ++c) lb[c] = Li[tx + 16 * c][k];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[a][c] = fma(xa[a], lb[c], acc[a][c]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = ty + 16 * a;
    if (i >= nr) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = tx + 16 * c;
      if (j < w) B[(size_t)i * ldb + j] = acc[a][c];
    }
  }
  __syncthreads();
}

// One FP32 tile product of the fused Cholesky, 256 threads:
//   C := C - A B^T (sub) or C := A B^T,
// C (M x N), A (M x K), B (N x K) row-major, M, N, K <= 64.  Every global
// load of a thread is issued before the first use (one latency round instead
// of one per K slice); a warp's load instruction covers 4 rows x 8 columns
// (four full 32-byte sectors).  A and B land k-major in shared memory with a
// pitch of 68 floats -- conflict-free stores, and a thread's four rows (four
// columns) are one 16-byte shared load -- so a K step is 2 shared loads for
// 16 FMAs (the 64 x 65 layout took 8).  Each thread owns rows 4 ty + a and
// columns 4 tx + b; the products are summed in ascending k and subtracted
// from C at the end.  A and C may alias (the TRSM items overwrite their
// input): all of A is read before the barrier that precedes the stores.
__device__ void tile_abt_f32(const float* A, int lda, const float* B, int ldb, float* C, int ldc, int M, int N,
                             int K, bool sub, float* smem) {
  constexpr int PITCH = 68;
  float (*As)[PITCH] = reinterpret_cast<float (*)[PITCH]>(smem);
  float (*Bs)[PITCH] = reinterpret_cast<float (*)[PITCH]>(smem + 64 * PITCH);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tx = tid & 15, ty = tid >> 4;
  float ra[16], rb[16], c[4][4];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int pr = q * 8 + warp, i = 4 * (pr & 15) + (lane & 3), k = 8 * (pr >> 4) + (lane >> 2);
    ra[q] = (i < M && k < K) ? __ldcg(A + (size_t)i * lda + k) : 0.f;
    rb[q] = (i < N && k < K) ? __ldcg(B + (size_t)i * ldb + k) : 0.f;
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int i = 4 * ty + a, j = 4 * tx + b;
      c[a][b] = (sub && i < M && j < N) ? __ldcg(C + (size_t)i * ldc + j) : 0.f;
    }
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int pr = q * 8 + warp, i = 4 * (pr & 15) + (lane & 3), k = 8 * (pr >> 4) + (lane >> 2);
    As[k][i] = ra[q];
    Bs[k][i] = rb[q];
  }
  __syncthreads();
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    const float4 av = *reinterpret_cast<const float4*>(&As[k][4 * ty]);
    const float4 bv = *reinterpret_cast<const float4*>(&Bs[k][4 * tx]);
    const float ar[4] = {av.x, av.y, av.z, av.w}, br[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = fmaf(ar[a], br[b], acc[a][b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = 4 * ty + a;
    if (i >= M) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = 4 * tx + b;
      if (j < N) C[(size_t)i * ldc + j] = sub ? c[a][b] - acc[a][b] : acc[a][b];
    }
  }
  __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(256) trsm_inv_kernel(const TrsmTask<T>* __restrict__ tasks, int nTasks) {
  // B (64-row chunk x w) := B L^{-T}: the block inverts its w x w tile and
  // multiplies.
  int lo = 0, hi = nTasks - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].chunkBase <= b) lo = mid;
    else hi = mid - 1;
  }
  const TrsmTask<T> t = tasks[lo];
  const int rb0 = (b - t.chunkBase) * TRSM_ROWS_F32;
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  T (*L)[65] = reinterpret_cast<T (*)[65]>(trsm_smem);
  T (*Li)[65] = reinterpret_cast<T (*)[65]>(trsm_smem + sizeof(T) * 64 * 65);
  T (*X)[65] = reinterpret_cast<T (*)[65]>(trsm_smem + 2 * sizeof(T) * 64 * 65);
  T (*Tm)[16][17] = reinterpret_cast<T (*)[16][17]>(trsm_smem + 3 * sizeof(T) * 64 * 65);   // 3 blocks
  tile_inverse<T>(t.L, t.ldl, t.w, L, Li, Tm);
  for (int sub = 0; sub < TRSM_ROWS_F32 / 64; ++sub) {
    const int r0 = rb0 + 64 * sub;
    if (r0 >= t.rows) break;
    trsm_chunk_mul<T>(t.B + (size_t)r0 * t.ldb, t.ldb, min(64, t.rows - r0), t.w, X, Li);
  }
}

// Blocked partial Cholesky of every front of a level in one launch.  A job
// factors the first nDiag columns of a front F (rows x rows, lower, row-major)
// in panels: the first w0 = nDiag - 64 (P - 1) wide, the others 64, so that
// every later panel and every trailing block is aligned to the tile grid
// b(0) = 0, b(t) = w0 + 64 (t - 1).  Panel p is one POTRF of tile (p, p)
// (which also stores the tile's inverse), one TRSM per row tile a > p, and
// one update C(a, b) -= X(a) X(b)^T (K = panel width) per lower tile of the
// trailing block with column tile b below nUpd.  Each piece is a work item;
// a block takes the next item from a ticket counter (the items are listed in
// a topological order, so a block only waits on items taken before its own) and
// waits, bounded, on per-tile completion counters:
//   POTRF(p)       tile (p, p) updated by the p earlier panels
//   TRSM(p, a)     POTRF(p) done; tile (a, p) updated by the p earlier panels
//   GEMM(p, a, b)  TRSM(p, a) and TRSM(p, b) done; tile (a, b) updated by the p earlier panels
// sync[0] is the ticket, the counters follow (zeroed before every launch);
// a wait that gives up sets flag[1].  Data written by other blocks is read
// through L2 (ld.global.cg).
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned smid() {
  unsigned r;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(r));
  return r;
}

// (Four blocks per SM -- 64 registers, small spills -- measured slower: the
// c2 factor 27.3 vs 27.0 ms; the critical POTRF chain pays for the spills.)
template <class T>
__global__ void __launch_bounds__(256) chol_fused_kernel(const CholFusedJob<T>* __restrict__ jobs,
                                                         const CholItem* __restrict__ items, int nItems,
                                                         int* __restrict__ sync, T* __restrict__ ws, int* flag,
                                                         unsigned long long* __restrict__ trace) {
  extern __shared__ __align__(16) unsigned char cf_smem[];
  __shared__ int sTicket, sOk;
  __shared__ unsigned long long tStart, tReady;
  int* err = flag + 1;
  if (threadIdx.x == 0) {
    sTicket = atomicAdd(sync, 1);
    if (trace) tStart = globaltimer_ns();
  }
  __syncthreads();
  if (sTicket >= nItems) {   // counters not reset: report, touch nothing
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const CholItem it = items[sTicket];
  const CholFusedJob<T> j = jobs[it.job];
  int* cnt = sync + 1 + j.cnt;     // TR x TU: panels applied to tile (a, b)
  int* tdone = cnt + j.TR * j.TU;  // TR: panels whose TRSM of row tile a is done
  int* pdone = tdone + j.TR;       // P: POTRF of panel p done
  const int p = it.p, a = it.a, b = it.b;
  const int* lim = flag + 2;   // polls before a wait gives up (set with the flags before the factorisation)
  auto bnd = [&](int t) { return t == 0 ? 0 : j.w0 + 64 * (t - 1); };      // columns (and Cholesky rows)
  auto rbnd = [&](int t) { return t == 0 ? 0 : j.r1 + 64 * (t - 1); };     // rows
  const int c0 = bnd(p), wp = bnd(p + 1) - c0;
  if ((threadIdx.x >> 5) == 0) {
    bool ok;
    if (it.kind == CHOL_POTRF) ok = j.L ? true : wait_geq_lim(cnt + p * j.TU + p, p, err, lim);
    else if (it.kind == CHOL_TRSM)
      ok = wait_geq_lim(pdone + p, 1, err, lim) && wait_geq_lim(cnt + a * j.TU + p, p, err, lim);
    else
      ok = wait_geq_lim(tdone + a, p + 1, err, lim) && (j.L || wait_geq_lim(tdone + b, p + 1, err, lim)) &&
           wait_geq_lim(cnt + a * j.TU + b, p, err, lim);
    if (threadIdx.x == 0) {
      sOk = ok;
      if (trace) tReady = globaltimer_ns();
    }
  }
  __syncthreads();
  if (!sOk) return;
  T* F = j.F;
  const int ld = j.ld;
  int* done;
  int doneVal;
  if (it.kind == CHOL_POTRF) {
    // Cholesky job: factor the diagonal tile; TRSM job: L is factored already
    T* A = j.L ? const_cast<T*>(j.L) + (size_t)c0 * j.ldl + c0 : F + (size_t)c0 * ld + c0;
    const int lda = j.L ? j.ldl : ld;
    if (!j.L) potrf_tile_reg<T>(A, ld, wp, j.code, flag);
    if (j.L || c0 + wp < j.nRows) {   // rows below: the TRSM items multiply by the inverse
      T (*L)[65] = reinterpret_cast<T (*)[65]>(cf_smem);
      T (*Li)[65] = reinterpret_cast<T (*)[65]>(cf_smem + sizeof(T) * 64 * 65);
      T (*Tm)[16][17] = reinterpret_cast<T (*)[16][17]>(cf_smem + 2 * sizeof(T) * 64 * 65);
      tile_inverse<T>(A, lda, wp, L, Li, Tm);
      T* out = ws + j.inv + (size_t)p * 4096;
#pragma unroll
      for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) out[idx] = Li[idx >> 6][idx & 63];
    }
    done = pdone + p;
    doneVal = 1;
  } else if (it.kind == CHOL_TRSM && std::is_same<T, float>::value) {
    // X(a) := X(a) Li(p)^T with the panel's inverse tile straight from the workspace
    const int r0 = rbnd(a), nr = min(rbnd(a + 1), j.nRows) - r0;
    float* X = reinterpret_cast<float*>(F) + (size_t)r0 * ld + c0;
    const float* Li = reinterpret_cast<const float*>(ws) + j.inv + (size_t)p * 4096;
    tile_abt_f32(X, ld, Li, 64, X, ld, nr, wp, wp, false, reinterpret_cast<float*>(cf_smem));
    done = tdone + a;
    doneVal = p + 1;
  } else if (it.kind == CHOL_TRSM) {
    T (*X)[65] = reinterpret_cast<T (*)[65]>(cf_smem);
    T (*Li)[65] = reinterpret_cast<T (*)[65]>(cf_smem + sizeof(T) * 64 * 65);
    const T* in = ws + j.inv + (size_t)p * 4096;
#pragma unroll
    for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) Li[idx >> 6][idx & 63] = __ldcg(in + idx);
    __syncthreads();
    const int r0 = rbnd(a);
    trsm_chunk_mul<T>(F + (size_t)r0 * ld + c0, ld, min(rbnd(a + 1), j.nRows) - r0, wp, X, Li);
    done = tdone + a;
    doneVal = p + 1;
  } else if (std::is_same<T, float>::value) {   // update of tile (a, b) by panel p
    const int r0 = rbnd(a), q0 = bnd(b);
    float* Ff = reinterpret_cast<float*>(F);
    const float* Bp = j.L ? reinterpret_cast<const float*>(j.L) + (size_t)q0 * j.ldl + c0 : Ff + (size_t)q0 * ld + c0;
    const int m = min(rbnd(a + 1), j.nRows) - r0, n = min(bnd(b + 1), j.nUpd) - q0, ldb = j.L ? j.ldl : ld;
    tile_abt_f32(Ff + (size_t)r0 * ld + c0, ld, Bp, ldb, Ff + (size_t)r0 * ld + q0, ld, m, n, wp, true,
                 reinterpret_cast<float*>(cf_smem));
    done = cnt + a * j.TU + b;
    doneVal = p + 1;
  } else {
    const int r0 = rbnd(a), q0 = bnd(b);
    GemmTask<T> g;
    g.A = F + (size_t)r0 * ld + c0;
    g.B = j.L ? j.L + (size_t)q0 * j.ldl + c0 : F + (size_t)q0 * ld + c0;   // TRSM job: X(a) L(b, p)^T
    g.C = F + (size_t)r0 * ld + q0;
    g.M = min(rbnd(a + 1), j.nRows) - r0;
    g.N = min(bnd(b + 1), j.nUpd) - q0;
    g.K = wp;
    g.lda = g.ldc = ld;
    g.ldb = j.L ? j.ldl : ld;
    g.tA = 0;
    g.tB = 1;
    g.lower = 0;
    g.alpha = T(-1);
    g.beta = T(1);
    T (*As)[BK][BM + 1] = reinterpret_cast<T (*)[BK][BM + 1]>(cf_smem);
    T (*Bs)[BK][BN + 1] = reinterpret_cast<T (*)[BK][BN + 1]>(cf_smem + 2 * sizeof(T) * BK * (BM + 1));
    gemm_tile<T>(g, 0, 0, As, Bs);
    done = cnt + a * j.TU + b;
    doneVal = p + 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(done, doneVal);
    if (trace) {   // diagnostics: when the item started, was ready, ended (ns), and its SM
      unsigned long long* r = trace + 4 * (size_t)sTicket;
      r[0] = tStart;
      r[1] = tReady;
      r[2] = globaltimer_ns();
      r[3] = smid();
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256) extadd_kernel(const ExtAddRow<T>* __restrict__ rows, int nRows,
                                                     const ExtAddSeg* __restrict__ segs,
                                                     const ExtAddSource<T>* __restrict__ src) {
  const int lane = threadIdx.x & 31;
  const int rw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (rw >= nRows) return;
  const ExtAddRow<T> R = rows[rw];
  for (int g = R.segBegin; g < R.segEnd; ++g) {
    const ExtAddSeg sg = segs[g];
    const ExtAddSource<T>& S = src[sg.src];
    const T* drow = S.D + (size_t)sg.a * S.ld;
    const int b1 = min(S.b1, sg.a + 1);
    for (int b = S.b0 + lane; b < b1; b += 32) {
      T* dst = R.Frow + S.rowRel[b];
      *dst = fma(S.sign, drow[b], *dst);
    }
    __syncwarp();   // the next source may hit the same target entries
  }
}

template <class T>
__global__ void scatter_kernel(const double* __restrict__ Avals, const long long* __restrict__ srcIdx,
                               const long long* __restrict__ dstIdx, long long count, T* __restrict__ dst) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x)
    dst[dstIdx[k]] = (T)Avals[srcIdx[k]];
}

// ---------------------------------------------------------------------------
// Blocked Householder QR of the sketches (LAPACK dgeqrf + dorgqr: dlarfg
// reflectors with v_0 = 1, compact-WY panels of QR_PB columns, dlarft's
// forward column-wise T).  Per panel: one block per matrix factors the panel
// (in shared memory when it fits), then many blocks apply the panel's block
// reflector to the trailing columns.  Q = H_0 ... H_{r-1} [I; 0] is formed by
// applying the block reflectors to [I; 0] in reverse order.
constexpr int QR_PB = 16;          // panel width
constexpr int QRP_THREADS = 512;   // panel kernel
constexpr int QA_ROWS = 64;        // apply kernel: row chunk
constexpr int QA_CW = 16;          // apply kernel: columns per block
constexpr int QR_SMEM_MAX = 200 * 1024;

template <class R>
__device__ __forceinline__ R warp_sum_d(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum of v[0..15] over the 32 lanes of a warp; lane l (l < 16) returns the
// total of v[l] (31 shuffles, fixed order).
template <class R>
__device__ __forceinline__ R warp_transpose_sum16(R (&v)[QR_PB]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], 16);
#pragma unroll
  for (int w = 8; w >= 1; w >>= 1) {
    const bool up = (lane & w) != 0;
#pragma unroll
    for (int i = 0; i < w; ++i) {
      const R send = up ? v[i] : v[i + w];
      const R keep = up ? v[i + w] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, w);
    }
  }
  return v[0];
}

// Y (row-major n x r) -> W (column-major, ld n), 32 x 32 tiles.
template <class T>
__global__ void __launch_bounds__(256) qr_to_colmajor(const QrTask<T>* __restrict__ tasks) {
  __shared__ T tile[32][33];
  const QrTask<T> t = tasks[blockIdx.y];
  const int n = t.n, r = t.r;
  const int tr = (n + 31) / 32, tc = (r + 31) / 32;
  const int lx = threadIdx.x & 31, ly = threadIdx.x >> 5;
  for (int tl = blockIdx.x; tl < tr * tc; tl += gridDim.x) {
    const int i0 = (tl / tc) * 32, j0 = (tl % tc) * 32;
    for (int y = ly; y < 32; y += 8)
      if (i0 + y < n && j0 + lx < r) tile[y][lx] = t.Y[(size_t)(i0 + y) * r + j0 + lx];
    __syncthreads();
    for (int y = ly; y < 32; y += 8)
      if (j0 + y < r && i0 + lx < n) t.W[(size_t)(j0 + y) * n + i0 + lx] = tile[lx][y];
    __syncthreads();
  }
}

// Y (row-major n x r) := [I; 0]
template <class T>
__global__ void qr_set_e(const QrTask<T>* __restrict__ tasks) {
  const QrTask<T> t = tasks[blockIdx.y];
  const long long tot = (long long)t.n * t.r;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < tot; k += (long long)gridDim.x * blockDim.x) {
    const long long i = k / t.r, j = k - i * t.r;
    t.Y[k] = (i == j) ? T(1) : T(0);
  }
}

// Factor columns j0 .. j0+pw-1 of W (rows j0 .. n-1).  On return the panel
// holds V below its diagonal and T (pw x pw, upper) in place of the upper
// triangle of its diagonal block (R is not needed: only Q is used).
template <class T>
__global__ void __launch_bounds__(QRP_THREADS) qr_panel_kernel(const QrTask<T>* __restrict__ tasks, int j0,
                                                               long long smemElems) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr int NW = QRP_THREADS / 32;
  __shared__ T redA[NW];
  __shared__ T redC[NW][QR_PB];
  __shared__ T sred[QR_PB], sfin[QR_PB];
  __shared__ T Ts[QR_PB][QR_PB + 1];
  const QrTask<T> t = tasks[blockIdx.x];
  const int n = t.n, r = t.r;
  if (j0 >= r) return;
  const int pw = min(QR_PB, r - j0), nr = n - j0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* Wg = t.W + (size_t)j0 * n + j0;   // panel element (i, c) at Wg[c * n + i]
  T* P = Wg;
  long long lp = n;
  const bool inSmem = (long long)nr * pw <= smemElems;
  if (inSmem) {   // a thread's loads of all panel columns in flight at once
    P = reinterpret_cast<T*>(smraw);
    lp = nr;
    for (int i = tid; i < nr; i += QRP_THREADS) {
      T tmp[QR_PB];
#pragma unroll
      for (int c = 0; c < QR_PB; ++c)
        if (c < pw) tmp[c] = Wg[(size_t)c * n + i];
#pragma unroll
      for (int c = 0; c < QR_PB; ++c)
        if (c < pw) P[c * lp + i] = tmp[c];
    }
  }
  for (int idx = tid; idx < QR_PB * (QR_PB + 1); idx += QRP_THREADS) (&Ts[0][0])[idx] = T(0);
  __syncthreads();
  for (int kk = 0; kk < pw; ++kk) {
    T* pk = P + kk * lp;
    // dlarfg on column kk
    T x2 = T(0);
    for (int i = kk + 1 + tid; i < nr; i += QRP_THREADS) x2 += pk[i] * pk[i];
    x2 = warp_sum_d(x2);
    if (lane == 0) redA[warp] = x2;
    __syncthreads();
    x2 = T(0);
#pragma unroll
    for (int q = 0; q < NW; ++q) x2 += redA[q];
    const T alpha = pk[kk];
    T tau = T(0), scal = T(1);
    if (x2 > T(0)) {
      const T beta = -copysign(sqrt(alpha * alpha + x2), alpha);
      tau = (beta - alpha) / beta;
      scal = T(1) / (alpha - beta);
      for (int i = kk + 1 + tid; i < nr; i += QRP_THREADS) pk[i] *= scal;
    }
    // s_c = P[kk][c] + sum_{i>kk} v_i P[i][c] for every panel column c
    T part[QR_PB];
#pragma unroll
    for (int c = 0; c < QR_PB; ++c) part[c] = T(0);
    for (int i = kk + 1 + tid; i < nr; i += QRP_THREADS) {
      const T vi = pk[i];
#pragma unroll
      for (int c = 0; c < QR_PB; ++c)
        if (c < pw) part[c] += P[c * lp + i] * vi;
    }
    const T ws = warp_transpose_sum16(part);
    if (lane < QR_PB) redC[warp][lane] = ws;
    __syncthreads();
    if (tid < pw) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < NW; ++q) s += redC[q][tid];
      sred[tid] = s + P[tid * lp + kk];
    }
    __syncthreads();
    // T column kk (dlarft): T[p][kk] = -tau sum_{q=p}^{kk-1} T[p][q] y_q, T[kk][kk] = tau
    if (tid < kk) {
      T s = T(0);
      for (int q = tid; q < kk; ++q) s += Ts[tid][q] * sred[q];
      Ts[tid][kk] = -tau * s;
    }
    if (tid == kk) Ts[kk][kk] = tau;
    if (tid < pw) sfin[tid] = tau * sred[tid];
    __syncthreads();
    // apply H_kk to the remaining panel columns
    if (tau != T(0)) {
      for (int c = kk + 1; c < pw; ++c) {
        const T w = sfin[c];
        T* pc = P + c * lp;
        for (int i = kk + 1 + tid; i < nr; i += QRP_THREADS) pc[i] -= w * pk[i];
        if (tid == 0) pc[kk] -= w;
      }
    }
    __syncthreads();
  }
  if (inSmem)
    for (int c = 0; c < pw; ++c)
      for (int i = tid; i < nr; i += QRP_THREADS) Wg[(size_t)c * n + i] = P[c * lp + i];
  __syncthreads();
  // T over the upper triangle of the diagonal block
  for (int idx = tid; idx < pw * pw; idx += QRP_THREADS) {
    const int a = idx / pw, b = idx - a * pw;
    if (a <= b) Wg[(size_t)b * n + a] = Ts[a][b];
  }
}

// The same panel factorisation with the panel in registers (FP32, at most
// 512 R rows): thread t keeps rows t + 512 q (q < R) of the 16 panel
// columns, so a column step touches shared memory only for its three block
// reductions (|x|^2 below the diagonal with row kk, the 16 dot products
// s_c = v^T P[:, c], the T column) -- three barriers per column.  Reflectors,
// T factor and layout as qr_panel_kernel (the sums run in another fixed order).
template <int R>
__global__ void __launch_bounds__(QRP_THREADS, 1) qr_panel_reg_kernel(const QrTask<float>* __restrict__ tasks,
                                                                      int j0) {
  constexpr int NW = QRP_THREADS / 32;
  __shared__ float redA[2][NW];
  __shared__ float redC[NW][QR_PB];
  __shared__ float rowk[QR_PB], sred[QR_PB];
  __shared__ float Ts[QR_PB][QR_PB + 1];
  const QrTask<float> t = tasks[blockIdx.x];
  const int n = t.n, r = t.r;
  if (j0 >= r) return;
  const int pw = min(QR_PB, r - j0), nr = n - j0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float* Wg = t.W + (size_t)j0 * n + j0;   // panel element (i, c) at Wg[c * n + i]
  float a[R][QR_PB];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int i = tid + QRP_THREADS * q;
#pragma unroll
    for (int c = 0; c < QR_PB; ++c) a[q][c] = (i < nr && c < pw) ? Wg[(size_t)c * n + i] : 0.f;
  }
  for (int idx = tid; idx < QR_PB * (QR_PB + 1); idx += QRP_THREADS) (&Ts[0][0])[idx] = 0.f;
  if (tid < QR_PB) sred[tid] = 0.f;   // columns beyond pw keep s = 0
#pragma unroll
  for (int kk = 0; kk < QR_PB; ++kk) {
    if (kk >= pw) break;
    // |x|^2 below the diagonal; row kk published (alpha and the unit row of the reflector)
    float x2 = 0.f;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int i = tid + QRP_THREADS * q;
      if (i > kk && i < nr) x2 += a[q][kk] * a[q][kk];
    }
    x2 = warp_sum_d(x2);
    if (lane == 0) redA[kk & 1][warp] = x2;
    if (tid == kk)
#pragma unroll
      for (int c = 0; c < QR_PB; ++c) rowk[c] = a[0][c];
    __syncthreads();
    x2 = 0.f;
#pragma unroll
    for (int q = 0; q < NW; ++q) x2 += redA[kk & 1][q];
    const float alpha = rowk[kk];
    float tau = 0.f, scal = 1.f;
    if (x2 > 0.f) {
      const float beta = -copysignf(sqrtf(alpha * alpha + x2), alpha);
      tau = (beta - alpha) / beta;
      scal = 1.f / (alpha - beta);
    }
    float v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int i = tid + QRP_THREADS * q;
      v[q] = (i > kk && i < nr) ? a[q][kk] * scal : 0.f;
      if (i > kk && i < nr) a[q][kk] = v[q];
    }
    // s_c = P[kk][c] + sum_{i > kk} v_i P[i][c]
    float part[QR_PB];
#pragma unroll
    for (int c = 0; c < QR_PB; ++c) {
      part[c] = 0.f;
#pragma unroll
      for (int q = 0; q < R; ++q) part[c] += v[q] * a[q][c];
    }
    const float ws = warp_transpose_sum16(part);
    if (lane < QR_PB) redC[warp][lane] = ws;
    __syncthreads();
    if (tid < pw) {
      float sum = 0.f;
#pragma unroll
      for (int q = 0; q < NW; ++q) sum += redC[q][tid];
      sred[tid] = sum + rowk[tid];
    }
    __syncthreads();
    // T column kk (dlarft): T[p][kk] = -tau sum_{q=p}^{kk-1} T[p][q] s_q, T[kk][kk] = tau
    if (tid < kk) {
      float sum = 0.f;
      for (int q = tid; q < kk; ++q) sum += Ts[tid][q] * sred[q];
      Ts[tid][kk] = -tau * sum;
    }
    if (tid == kk) Ts[kk][kk] = tau;
    // apply H_kk to the columns right of kk
    if (tau != 0.f) {
#pragma unroll
      for (int c = kk + 1; c < QR_PB; ++c) {
        const float w = tau * sred[c];
#pragma unroll
        for (int q = 0; q < R; ++q) a[q][c] -= w * v[q];
        if (tid == kk) a[0][c] -= w;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int i = tid + QRP_THREADS * q;
    if (i < nr)
#pragma unroll
      for (int c = 0; c < QR_PB; ++c)
        if (c < pw) Wg[(size_t)c * n + i] = a[q][c];
  }
  __syncthreads();
  // T over the upper triangle of the diagonal block
  for (int idx = tid; idx < pw * pw; idx += QRP_THREADS) {
    const int ra = idx / pw, cb = idx - ra * pw;
    if (ra <= cb) Wg[(size_t)cb * n + ra] = Ts[ra][cb];
  }
}

// Apply the block reflector of panel j0 to the other columns, in parallel
// over (row block of QA_RB rows, group of QA_CW columns):
//   mode 0 (factor): W[j0:n, c] := (I - V T^T V^T) W[j0:n, c], c >= j0 + pw
//   mode 1 (form Q): Y[j0:n, c] := (I - V T V^T) Y[j0:n, c],   c >= j0
// in two launches: Zpart = V^T A per row block; then per row block Z = the
// row-block partials added in order, M = T^T Z (or T Z), A -= V M (every block
// of a column group forms the same small M instead of a launch of its own).
// ws holds Zpart (tasks x cgMax x rbMax x 16 x 16).
// Rows per block of the apply: one 64-row chunk, so a QR of few tall panels
// still spreads over many blocks (c2 factor 21.65 ms at 64 rows, 22.00 at
// 128, 22.85 at 256, 24.51 at 512).
constexpr int QA_RB = 64;

template <class T>
struct QrApplyView {
  const T* V;   // panel reflectors, column-major (ld n), V[p][i] at V[p * n + i], unit diagonal implied
  T* A;
  int n, r, nr, pw, c0, cw;
  int mode;
  __device__ size_t aidx(int j0, int i, int c) const {
    return mode == 0 ? (size_t)(c0 + c) * n + j0 + i : (size_t)(j0 + i) * r + c0 + c;
  }
  __device__ T v(int i, int p) const {   // reflector p at panel row i (i counted from j0)
    if (p >= pw) return T(0);
    return i == p ? T(1) : (i > p ? V[(size_t)p * n + i] : T(0));
  }
};

template <class T>
__device__ __forceinline__ bool qr_view(const QrTask<T>& t, int j0, int mode, int cg, QrApplyView<T>& w) {
  const int n = t.n, r = t.r;
  if (j0 >= r) return false;
  w.n = n;
  w.r = r;
  w.pw = min(QR_PB, r - j0);
  w.nr = n - j0;
  w.mode = mode;
  w.c0 = (mode == 0 ? j0 + w.pw : j0) + cg * QA_CW;
  if (w.c0 >= r) return false;
  w.cw = min(QA_CW, r - w.c0);
  w.V = t.W + (size_t)j0 * n + j0;
  w.A = mode == 0 ? t.W : t.Y;
  return true;
}

template <class T>
__global__ void __launch_bounds__(256) qr_zpart_kernel(const QrTask<T>* __restrict__ tasks, int j0, int mode,
                                                       T* __restrict__ ws, int cgMax, int rbMax) {
  __shared__ T Vs[QA_ROWS][QR_PB + 1];
  __shared__ T As[QA_ROWS][QA_CW + 1];
  const QrTask<T> t = tasks[blockIdx.y];
  const int cg = blockIdx.x % cgMax, rb = blockIdx.x / cgMax;
  QrApplyView<T> w;
  if (!qr_view(t, j0, mode, cg, w)) return;
  const int r0 = rb * QA_RB;
  if (r0 >= w.nr) return;
  const int r1 = min(w.nr, r0 + QA_RB);
  const int tid = threadIdx.x, zp = tid % QR_PB, zc = tid / QR_PB;
  T z = T(0);
  for (int i0 = r0; i0 < r1; i0 += QA_ROWS) {
    const int h = min(QA_ROWS, r1 - i0);
    for (int idx = tid; idx < QA_ROWS * QR_PB; idx += blockDim.x) {
      const int p = idx / QA_ROWS, i = idx - p * QA_ROWS;
      Vs[i][p] = i < h ? w.v(i0 + i, p) : T(0);
    }
    for (int idx = tid; idx < QA_ROWS * QA_CW; idx += blockDim.x) {
      int i, c;
      if (mode == 0) { c = idx / QA_ROWS; i = idx - c * QA_ROWS; }
      else { i = idx / QA_CW; c = idx - i * QA_CW; }
      As[i][c] = (i < h && c < w.cw) ? w.A[w.aidx(j0, i0 + i, c)] : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int i = 0; i < QA_ROWS; ++i) z += Vs[i][zp] * As[i][zc];
    __syncthreads();
  }
  ws[(((size_t)blockIdx.y * cgMax + cg) * rbMax + rb) * (QR_PB * QA_CW) + zp * QA_CW + zc] = z;
}

template <class T>
__global__ void __launch_bounds__(256) qr_update_kernel(const QrTask<T>* __restrict__ tasks, int j0, int mode,
                                                        const T* __restrict__ ws, int cgMax, int rbMax) {
  __shared__ T Vs[QA_ROWS][QR_PB + 1];
  __shared__ T As[QA_ROWS][QA_CW + 1];
  __shared__ T M[QR_PB][QA_CW + 1];
  __shared__ T Z[QR_PB][QA_CW + 1];
  __shared__ T Ts[QR_PB][QR_PB + 1];
  const QrTask<T> t = tasks[blockIdx.y];
  const int cg = blockIdx.x % cgMax, rb = blockIdx.x / cgMax;
  QrApplyView<T> w;
  if (!qr_view(t, j0, mode, cg, w)) return;
  const int r0 = rb * QA_RB;
  if (r0 >= w.nr) return;
  const int r1 = min(w.nr, r0 + QA_RB);
  const int tid = threadIdx.x;
  {
    // M = T^T Z (mode 0) or T Z (mode 1), Z = V^T A summed over the row blocks'
    // partials in row-block order: every block of the column group forms the
    // same M (a 16 x 16 reduction, cheaper than a launch of its own)
    const int zp = tid % QR_PB, zc = tid / QR_PB;
    const int a = tid / QR_PB, b = tid - a * QR_PB;   // T over the upper triangle of the diagonal block
    Ts[a][b] = (a <= b && b < w.pw) ? w.V[(size_t)b * w.n + a] : T(0);
    const int nrb = (w.nr + QA_RB - 1) / QA_RB;
    const T* zpart = ws + ((size_t)blockIdx.y * cgMax + cg) * rbMax * (QR_PB * QA_CW) + zp * QA_CW + zc;
    T z = T(0);
    for (int q = 0; q < nrb; ++q) z += zpart[(size_t)q * (QR_PB * QA_CW)];
    Z[zp][zc] = z;
    __syncthreads();
    T m = T(0);
    if (mode == 0) {
      for (int q = 0; q <= zp; ++q) m += Ts[q][zp] * Z[q][zc];   // T^T Z
    } else {
      for (int q = zp; q < QR_PB; ++q) m += Ts[zp][q] * Z[q][zc];   // T Z
    }
    M[zp][zc] = m;
  }
  const int ai = tid % QA_ROWS, aq = (tid / QA_ROWS) * 4;
  for (int i0 = r0; i0 < r1; i0 += QA_ROWS) {
    const int h = min(QA_ROWS, r1 - i0);
    for (int idx = tid; idx < QA_ROWS * QR_PB; idx += blockDim.x) {
      const int p = idx / QA_ROWS, i = idx - p * QA_ROWS;
      Vs[i][p] = i < h ? w.v(i0 + i, p) : T(0);
    }
    for (int idx = tid; idx < QA_ROWS * QA_CW; idx += blockDim.x) {
      int i, c;
      if (mode == 0) { c = idx / QA_ROWS; i = idx - c * QA_ROWS; }
      else { i = idx / QA_CW; c = idx - i * QA_CW; }
      As[i][c] = (i < h && c < w.cw) ? w.A[w.aidx(j0, i0 + i, c)] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) {
      T s = T(0);
#pragma unroll
      for (int p = 0; p < QR_PB; ++p) s += Vs[ai][p] * M[p][aq + cc];
      As[ai][aq + cc] -= s;
    }
    __syncthreads();
    for (int idx = tid; idx < QA_ROWS * QA_CW; idx += blockDim.x) {
      int i, c;
      if (mode == 0) { c = idx / QA_ROWS; i = idx - c * QA_ROWS; }
      else { i = idx / QA_CW; c = idx - i * QA_CW; }
      if (i < h && c < w.cw) w.A[w.aidx(j0, i0 + i, c)] = As[i][c];
    }
    __syncthreads();
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
  if constexpr (std::is_same<T, float>::value) potrf_reg_kernel<T><<<n, 256, 0, s>>>(d, flag);
  else potrf_kernel<T><<<n, 256, 0, s>>>(d, flag);
  RSCHOL_LAUNCH_CHECK();
}
template <class T> void launch_trsm(const TrsmTask<T>* d, int n, int chunks, cudaStream_t s) {
  if (n <= 0 || chunks <= 0) return;
  static std::once_flag once;   // per instantiation; callers may be on several threads
  if constexpr (std::is_same<T, float>::value) {
    const int smem = (int)(3 * sizeof(T) * 64 * 65 + 3 * sizeof(T) * 16 * 17);
    std::call_once(once, [&] {
      RSCHOL_CUDA(cudaFuncSetAttribute(trsm_inv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    });
    trsm_inv_kernel<T><<<chunks, 256, smem, s>>>(d, n);
  } else {
    const int smem = (int)(2 * sizeof(T) * 64 * 65);
    std::call_once(once, [&] {
      RSCHOL_CUDA(cudaFuncSetAttribute(trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    });
    trsm_kernel<T><<<chunks, 256, smem, s>>>(d, n);
  }
  RSCHOL_LAUNCH_CHECK();
}
template <class T>
void launch_chol_fused(const CholFusedJob<T>* jobs, const CholItem* items, int nItems, int* sync, long long syncInts,
                       T* ws, int* flag, unsigned long long* trace, cudaStream_t s) {
  if (nItems <= 0) return;
  RSCHOL_CUDA(cudaMemsetAsync(sync, 0, sizeof(int) * (size_t)syncInts, s));
  const int smem = (int)(sizeof(T) * (3 * 64 * 65 + 3 * 16 * 17));
  static std::once_flag once;
  std::call_once(once, [&] {
    RSCHOL_CUDA(cudaFuncSetAttribute(chol_fused_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  });
  chol_fused_kernel<T><<<nItems, 256, smem, s>>>(jobs, items, nItems, sync, ws, flag, trace);
  RSCHOL_LAUNCH_CHECK();
}
template <class T>
void launch_extadd(const ExtAddRow<T>* rows, int nRows, const ExtAddSeg* segs, const ExtAddSource<T>* src,
                   cudaStream_t s) {
  if (nRows <= 0) return;
  extadd_kernel<T><<<(nRows + 7) / 8, 256, 0, s>>>(rows, nRows, segs, src);
  RSCHOL_LAUNCH_CHECK();
}
// a block of 256 threads per (task, 64-row slab)
__global__ void block_convert_kernel(const CvtTask* __restrict__ tasks, int toDouble) {
  const CvtTask t = tasks[blockIdx.y];
  const int r0 = blockIdx.x * 64;
  if (r0 >= t.n) return;
  const int r1 = min(t.n, r0 + 64);
  for (int i = r0 + (threadIdx.x >> 5); i < r1; i += 8)
    for (int j = threadIdx.x & 31; j <= i; j += 32) {
      if (toDouble) t.D[(size_t)i * t.ldd + j] = (double)t.F[(size_t)i * t.ld + j];
      else t.F[(size_t)i * t.ld + j] = (float)t.D[(size_t)i * t.ldd + j];
    }
}

void launch_block_convert(const CvtTask* d, int nTasks, int maxN, int toDouble, cudaStream_t s) {
  if (nTasks <= 0 || maxN <= 0) return;
  block_convert_kernel<<<dim3((maxN + 63) / 64, nTasks), 256, 0, s>>>(d, toDouble);
  RSCHOL_LAUNCH_CHECK();
}

__global__ void init_flags_kernel(int* flag, int waitLimit) {
  flag[0] = INT_MAX;
  flag[1] = 0;
  flag[2] = waitLimit;
}

void launch_init_flags(int* flag, int waitLimit, cudaStream_t s) {
  init_flags_kernel<<<1, 1, 0, s>>>(flag, waitLimit);
  RSCHOL_LAUNCH_CHECK();
}

template <class T>
void launch_scatter(const double* A, const long long* si, const long long* di, long long count, T* dst,
                    cudaStream_t s) {
  if (count <= 0) return;
  scatter_kernel<T><<<grid_for(count, 256), 256, 0, s>>>(A, si, di, count, dst);
  RSCHOL_LAUNCH_CHECK();
}
long long householder_qr_workspace(int nTasks, int maxRows, int maxR) {
  const long long cgMax = (maxR + QA_CW - 1) / QA_CW, rbMax = (maxRows + QA_RB - 1) / QA_RB;
  return (long long)nTasks * cgMax * rbMax * (QR_PB * QA_CW);
}

template <class T>
int launch_householder_qr(const QrTask<T>* d, int n, int maxRows, int maxR, T* ws, cudaStream_t s) {
  if (n <= 0 || maxR <= 0) return 0;
  const int cgMax = (maxR + QA_CW - 1) / QA_CW, rbMax = (maxRows + QA_RB - 1) / QA_RB;
  int launches = 0;
  auto apply = [&](int j0, int mode) {
    qr_zpart_kernel<T><<<dim3(cgMax * rbMax, n), 256, 0, s>>>(d, j0, mode, ws, cgMax, rbMax);
    qr_update_kernel<T><<<dim3(cgMax * rbMax, n), 256, 0, s>>>(d, j0, mode, ws, cgMax, rbMax);
    RSCHOL_LAUNCH_CHECK();
    launches += 2;
  };
  static std::once_flag once;
  std::call_once(once, [] {
    RSCHOL_CUDA(cudaFuncSetAttribute(qr_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, QR_SMEM_MAX));
  });
  const long long tiles = (long long)((maxRows + 31) / 32) * ((maxR + 31) / 32);
  qr_to_colmajor<T><<<dim3((unsigned)std::min<long long>(tiles, 64), n), 256, 0, s>>>(d);
  RSCHOL_LAUNCH_CHECK();
  launches += 1;
  const size_t smem = std::min<size_t>((size_t)QR_SMEM_MAX, sizeof(T) * (size_t)maxRows * QR_PB);
  const long long smemElems = (long long)(smem / sizeof(T));
  const int panels = (maxR + QR_PB - 1) / QR_PB;
  for (int p = 0; p < panels; ++p) {
    const int j0 = p * QR_PB;
    if constexpr (std::is_same<T, float>::value) {
      if (maxRows <= QRP_THREADS) qr_panel_reg_kernel<1><<<n, QRP_THREADS, 0, s>>>(d, j0);
      else if (maxRows <= 2 * QRP_THREADS) qr_panel_reg_kernel<2><<<n, QRP_THREADS, 0, s>>>(d, j0);
      else if (maxRows <= 4 * QRP_THREADS) qr_panel_reg_kernel<4><<<n, QRP_THREADS, 0, s>>>(d, j0);
      else qr_panel_kernel<T><<<n, QRP_THREADS, smem, s>>>(d, j0, smemElems);
    } else {
      qr_panel_kernel<T><<<n, QRP_THREADS, smem, s>>>(d, j0, smemElems);
    }
    RSCHOL_LAUNCH_CHECK();
    ++launches;
    if (maxR - j0 - QR_PB > 0) apply(j0, 0);
  }
  const long long ecount = (long long)maxRows * maxR;
  qr_set_e<T><<<dim3((unsigned)std::max<long long>(1, std::min<long long>((ecount + 255) / 256, 256)), n), 256, 0, s>>>(d);
  RSCHOL_LAUNCH_CHECK();
  ++launches;
  for (int p = panels - 1; p >= 0; --p) apply(p * QR_PB, 1);
  return launches;
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
  template void launch_chol_fused<T>(const CholFusedJob<T>*, const CholItem*, int, int*, long long, T*, int*,  \
                                     unsigned long long*, cudaStream_t);                                 \
  template void launch_extadd<T>(const ExtAddRow<T>*, int, const ExtAddSeg*, const ExtAddSource<T>*,      \
                                 cudaStream_t);                                                          \
  template void launch_scatter<T>(const double*, const long long*, const long long*, long long, T*,      \
                                  cudaStream_t);                                                         \
  template int launch_householder_qr<T>(const QrTask<T>*, int, int, int, T*, cudaStream_t);                  \
  template void launch_set_identity<T>(const IdentTask<T>*, int, cudaStream_t);                          \
  template void launch_box_muller<T>(const uint32_t*, long long, T*, cudaStream_t);
RSCHOL_INST(double)
RSCHOL_INST(float)

}  // namespace rschol
