// Batched preconditioner apply: W (n x k, row-major, the k right-hand sides
// of a row contiguous) := M^{-1} W with one pass over the factor.
//
// Same operator and schedule as SolveEngine::apply_inplace, with every vector
// widened to k columns: the interior supernodes run in one ticketed launch
// per direction (a thread per (row, right-hand side) pair), and the
// compressed levels become batched GEMMs on the factor's GEMM kernels:
//   forward   Y = X F (row blocks of X stop at the diagonal), Z = U^T Y,
//             U_c = -V Z;
//   backward  S = V^T X_R, G = Y - U S, X = X^T G (column blocks of X start at
//             the diagonal).
// Factor bytes are read once per apply whatever k is; vector bytes scale
// with k.
#include <algorithm>
#include <mutex>
#include <stdexcept>
#include <type_traits>

#include "solve.cuh"
#include "solve_dev.cuh"

namespace rschol {

namespace {

using namespace solvedev;

// Every (row, right-hand side) pair of the interior solves is a dot product
// formed serially in a fixed order, so each column's arithmetic is the same
// whatever k is.  pair_dots runs such a family: for r < rows, c < k,
// acc = init(r, c), then for j = lo(r) .. hi(r) - 1 in order
// acc += a(r, j) * F(j, c) (acc -= ... when SUB), then out(r, c, acc).  A
// thread takes a tile of RA rows x RC columns (consecutive threads take
// consecutive column tiles): 1 x 1 spreads the pairs over all threads at
// small k, 4 x 4 reuses every load of A and F four times at large k.  The
// tiling only changes which thread forms a pair, not its arithmetic.
template <class T, int RA, int RC, bool SUB, class AE, class FV, class Init, class Lo, class Hi, class Out>
__device__ __forceinline__ void pair_dots(int rows, int k, AE a, FV fv, Init init, Lo lo, Hi hi, Out out) {
  const int ct = (k + RC - 1) / RC, rt = (rows + RA - 1) / RA;
  for (int tile = threadIdx.x; tile < rt * ct; tile += blockDim.x) {
    const int tr = tile / ct;
    const int r0 = tr * RA, c0 = (tile - tr * ct) * RC;
    T acc[RA][RC];
    int l[RA], h[RA];
    int jlo = 0x7fffffff, jhi = -0x7fffffff;
#pragma unroll
    for (int r = 0; r < RA; ++r) {
      const bool rv = r0 + r < rows;
      l[r] = rv ? lo(r0 + r) : 0;
      h[r] = rv ? hi(r0 + r) : 0;
#pragma unroll
      for (int q = 0; q < RC; ++q) acc[r][q] = (rv && c0 + q < k) ? init(r0 + r, c0 + q) : T(0);
      if (rv) {
        jlo = min(jlo, l[r]);
        jhi = max(jhi, h[r]);
      }
    }
    bool same = true;   // every row of the tile runs over [jlo, jhi)
#pragma unroll
    for (int r = 0; r < RA; ++r) same = same && (r0 + r >= rows || (l[r] == jlo && h[r] == jhi));
    if (same) {
      for (int j = jlo; j < jhi; ++j) {
        T f[RC];
#pragma unroll
        for (int q = 0; q < RC; ++q) f[q] = (RC == 1 || c0 + q < k) ? fv(j, c0 + q) : T(0);
#pragma unroll
        for (int r = 0; r < RA; ++r) {
          const T av = (RA == 1 || r0 + r < rows) ? a(r0 + r, j) : T(0);
#pragma unroll
          for (int q = 0; q < RC; ++q) {
            if (SUB) acc[r][q] -= av * f[q];
            else acc[r][q] += av * f[q];
          }
        }
      }
    } else {
      for (int j = jlo; j < jhi; ++j) {
        T f[RC];
#pragma unroll
        for (int q = 0; q < RC; ++q) f[q] = (RC == 1 || c0 + q < k) ? fv(j, c0 + q) : T(0);
#pragma unroll
        for (int r = 0; r < RA; ++r)
          if (j >= l[r] && j < h[r]) {
            const T av = a(r0 + r, j);
#pragma unroll
            for (int q = 0; q < RC; ++q) {
              if (SUB) acc[r][q] -= av * f[q];
              else acc[r][q] += av * f[q];
            }
          }
      }
    }
#pragma unroll
    for (int r = 0; r < RA; ++r)
#pragma unroll
      for (int q = 0; q < RC; ++q)
        if (r0 + r < rows && c0 + q < k) out(r0 + r, c0 + q, acc[r][q]);
  }
}

// f := L^{-1} f for k right-hand sides (f: n x k in shared memory, row
// stride k) with the inverted 64 x 64 diagonal blocks of L; t: 64 x k
// shared.
template <class T, int RA, int RC>
__device__ void trsv_dinv_k(const T* __restrict__ L, int ld, int n, const T* __restrict__ D, T* f, T* t, int k) {
  for (int i0 = 0; i0 < n; i0 += 64) {
    const int h = min(64, n - i0);
    pair_dots<T, RA, RC, true>(
        h, k, [&](int i, int j) { return L[(size_t)(i0 + i) * ld + j]; },
        [&](int j, int c) { return f[(size_t)j * k + c]; }, [&](int i, int c) { return f[(size_t)(i0 + i) * k + c]; },
        [](int) { return 0; }, [&](int) { return i0; }, [&](int i, int c, T v) { t[(size_t)i * k + c] = v; });
    __syncthreads();
    const T* Db = D + (size_t)i0 * 64;
    pair_dots<T, RA, RC, false>(
        h, k, [&](int i, int j) { return Db[(size_t)i * h + j]; }, [&](int j, int c) { return t[(size_t)j * k + c]; },
        [](int, int) { return T(0); }, [](int) { return 0; }, [](int i) { return i + 1; },
        [&](int i, int c, T v) { f[(size_t)(i0 + i) * k + c] = v; });
    __syncthreads();
  }
}

// f := L^{-T} f for k right-hand sides, same blocks.
template <class T, int RA, int RC>
__device__ void trsv_dinv_t_k(const T* __restrict__ L, int ld, int n, const T* __restrict__ D, T* f, T* t, int k) {
  if (n <= 0) return;
  for (int i0 = ((n - 1) / 64) * 64; i0 >= 0; i0 -= 64) {
    const int h = min(64, n - i0);
    pair_dots<T, RA, RC, true>(
        h, k, [&](int j, int i) { return L[(size_t)i * ld + i0 + j]; },
        [&](int i, int c) { return f[(size_t)i * k + c]; }, [&](int j, int c) { return f[(size_t)(i0 + j) * k + c]; },
        [&](int) { return i0 + h; }, [&](int) { return n; }, [&](int j, int c, T v) { t[(size_t)j * k + c] = v; });
    __syncthreads();
    const T* Db = D + (size_t)i0 * 64;
    pair_dots<T, RA, RC, false>(
        h, k, [&](int j, int i) { return Db[(size_t)i * h + j]; }, [&](int i, int c) { return t[(size_t)i * k + c]; },
        [](int, int) { return T(0); }, [](int j) { return j; }, [&](int) { return h; },
        [&](int j, int c, T v) { f[(size_t)(i0 + j) * k + c] = v; });
    __syncthreads();
  }
}

template <class T, int RA, int RC>
__global__ void __launch_bounds__(256) interior_forward_k(const SNode<T>* __restrict__ nodes,
                                                          const RowBlock* __restrict__ work,
                                                          const int* __restrict__ rel, const int* __restrict__ child,
                                                          int* __restrict__ sync, int epoch, int k,
                                                          const T* __restrict__ w, T* __restrict__ yout,
                                                          T* __restrict__ wu) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int sTicket;
  int* err = sync;
  if (threadIdx.x == 0) sTicket = atomicAdd(&sync[SYNC_TICK_F], 1);
  __syncthreads();
  if (sTicket >= (int)gridDim.x) {   // counters not reset: report, touch nothing
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const RowBlock wk = work[sTicket];
  const SNode<T>& nd = nodes[wk.node];
  const int n = nd.n, a0 = wk.b * ICH, a1 = min(nd.m, a0 + ICH);
  const int warp = threadIdx.x >> 5;
  T* f = reinterpret_cast<T*>(smraw);   // n x k
  T* t = f + (size_t)n * k;             // 64 x k
  T* wud = wu + nd.wuOff * k;
  if (warp == 0)
    for (int c = nd.childBegin; c < nd.childEnd; ++c) {
      const SNode<T>& cn = nodes[child[c]];
      if (!wait_geq(sync + cn.syncOff + 1, epoch * max(1, cn.nch), err)) break;
    }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n * k; idx += blockDim.x) f[idx] = w[(size_t)nd.c0 * k + idx];
  for (int idx = a0 * k + threadIdx.x; idx < a1 * k; idx += blockDim.x) wud[idx] = T(0);
  __syncthreads();
  for (int c = nd.childBegin; c < nd.childEnd; ++c) {
    const SNode<T>& cn = nodes[child[c]];
    const T* wuc = wu + cn.wuOff * k;
    const int* rl = rel + cn.relOff;
    for (int idx = threadIdx.x; idx < cn.m * k; idx += blockDim.x) {
      const int a = idx / k, q = idx - a * k;
      const int tr = rl[a];
      const T v = __ldcg(wuc + idx);
      if (tr < n) f[(size_t)tr * k + q] += v;
      else if (tr - n >= a0 && tr - n < a1) wud[(size_t)(tr - n) * k + q] += v;
    }
    __syncthreads();
  }
  trsv_dinv_k<T, RA, RC>(nd.L, nd.ld, n, nd.Dinv, f, t, k);
  if (wk.b == 0)
    for (int idx = threadIdx.x; idx < n * k; idx += blockDim.x) yout[(size_t)nd.c0 * k + idx] = f[idx];
  // wud[a][c] -= L21[a] . y[:, c]
  {
    const T* L21 = nd.L + (size_t)(n + a0) * nd.ld;
    const int ld = nd.ld;
    pair_dots<T, RA, RC, false>(
        a1 - a0, k, [&](int a, int j) { return L21[(size_t)a * ld + j]; },
        [&](int j, int c) { return f[(size_t)j * k + c]; }, [](int, int) { return T(0); }, [](int) { return 0; },
        [&](int) { return n; }, [&](int a, int c, T v) { wud[(size_t)(a0 + a) * k + c] -= v; });
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(sync + nd.syncOff + 1, 1);
  }
  launch_done(&sync[SYNC_TICK_F], &sync[SYNC_DONE_F]);
}

template <class T, int RA, int RC>
__global__ void __launch_bounds__(256) interior_backward_k(const SNode<T>* __restrict__ nodes,
                                                           const RowBlock* __restrict__ work,
                                                           const int* __restrict__ rows, int* __restrict__ sync,
                                                           int epoch, int k, T* __restrict__ ipart,
                                                           const T* __restrict__ yin, T* __restrict__ w) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int sLast, sTicket;
  int* err = sync;
  if (threadIdx.x == 0) sTicket = atomicAdd(&sync[SYNC_TICK_B], 1);
  __syncthreads();
  if (sTicket >= (int)gridDim.x) {
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const RowBlock wk = work[sTicket];
  const SNode<T>& nd = nodes[wk.node];
  if (nd.parentI >= 0 && (threadIdx.x >> 5) == 0) wait_geq(sync + nodes[nd.parentI].syncOff + 2, epoch, err);
  __syncthreads();
  const int n = nd.n, a0 = wk.b * ICH, a1 = min(nd.m, a0 + ICH);
  T* f = reinterpret_cast<T*>(smraw);   // n x k
  T* t = f + (size_t)n * k;             // 64 x k
  const int nch = (nd.m + ICH - 1) / ICH;
  if (nch > 0) {
    // part[j][c] = sum_{a in chunk} L21[a][j] x_{rows[a]}[c] (x written by
    // other blocks of this launch: loads bypass L1)
    const int* rw = rows + nd.rowsOff;
    const T* L21 = nd.L + (size_t)n * nd.ld;
    const int ld = nd.ld;
    T* part = ipart + (nd.zpOff + (size_t)wk.b * n) * k;
    pair_dots<T, RA, RC, false>(
        n, k, [&](int j, int a) { return L21[(size_t)a * ld + j]; },
        [&](int a, int c) { return __ldcg(w + (size_t)rw[a] * k + c); }, [](int, int) { return T(0); },
        [&](int) { return a0; }, [&](int) { return a1; }, [&](int j, int c, T v) { part[(size_t)j * k + c] = v; });
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      sLast = (atomicAdd(sync + nd.syncOff, 1) == nch - 1);
      __threadfence();
    }
    __syncthreads();
    if (!sLast) {
      launch_done(&sync[SYNC_TICK_B], &sync[SYNC_DONE_B]);
      return;
    }
  }
  for (int idx = threadIdx.x; idx < n * k; idx += blockDim.x) {
    T s = T(0);
    for (int c = 0; c < nch; ++c) s += __ldcg(ipart + (nd.zpOff + (size_t)c * n) * k + idx);
    f[idx] = yin[(size_t)nd.c0 * k + idx] - s;
  }
  __syncthreads();
  trsv_dinv_t_k<T, RA, RC>(nd.L, nd.ld, n, nd.Dinv, f, t, k);
  for (int idx = threadIdx.x; idx < n * k; idx += blockDim.x) w[(size_t)nd.c0 * k + idx] = f[idx];
  __syncthreads();
  if (threadIdx.x == 0) {
    if (nch > 0) sync[nd.syncOff] = 0;
    st_release(sync + nd.syncOff + 2, epoch);
  }
  launch_done(&sync[SYNC_TICK_B], &sync[SYNC_DONE_B]);
}

// w[c0 + i][c] += fixed-order sum of row i's contributions (a warp per row).
template <class T>
__global__ void __launch_bounds__(256) compressed_gather_k(const SNode<T>* __restrict__ nodes,
                                                           const int* __restrict__ lvl,
                                                           const long long* __restrict__ cstart,
                                                           const long long* __restrict__ ent, int k,
                                                           const T* __restrict__ wu, T* __restrict__ w) {
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= nd.n) return;
  const long long* cs = cstart + nd.cOff;
  for (int c = lane; c < k; c += 32) {
    T acc = T(0);
    for (long long e = cs[i]; e < cs[i + 1]; ++e) acc += wu[ent[e] * k + c];
    w[(size_t)(nd.c0 + i) * k + c] += acc;
  }
}

// X_R (m x k) of every compressed supernode of a level into its u region.
template <class T>
__global__ void __launch_bounds__(256) compressed_gather_xr_k(const SNode<T>* __restrict__ nodes,
                                                              const int* __restrict__ lvl,
                                                              const int* __restrict__ rows, int k,
                                                              const T* __restrict__ w, T* __restrict__ wu) {
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int lane = threadIdx.x & 31;
  const int a = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (a >= nd.m || nd.r == 0) return;
  const int g = rows[nd.rowsOff + a];
  T* dst = wu + (nd.wuOff + 2 * nd.r + a) * k;
  for (int c = lane; c < k; c += 32) dst[c] = w[(size_t)g * k + c];
}

// Products of the compressed levels: C (M x k) = alpha op(A) B + beta C
// with B (K x k, row stride ldb) the block of right-hand sides.  With k <= 64
// these are streaming products over the factor's X, U and V, so they run on
// SIMT kernels that read A once, coalesced.  Each output column's sum has a
// fixed order that depends on K alone (not on k); tasks are cut into units
// (one block each) of a row group and a group of CW columns (skinny_cw),
// numbered from each task's unitBase.
template <class T>
struct SkinnyTask {
  const T* A;
  const T* B;
  T* C;
  int M, K, lda, ldb, ldc;
  T alpha, beta;
  int unitBase;
};

template <class T>
__device__ __forceinline__ int find_skinny(const SkinnyTask<T>* __restrict__ tasks, int count, int u) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].unitBase <= u) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Row form, A row-major M x K.  A block per (16 rows, column group), a warp
// per two rows; lane l adds kk = l, l + 32, ... in order (zeros past K),
// then the lanes meet in a fixed butterfly.  Chunks of 256 rows of B are
// staged in shared memory transposed, so lane l reads its kk without bank
// conflicts, and each staged value serves both rows of the warp.
constexpr int SK_CHUNK = 256;   // kk per staged chunk of B (8 per lane)

template <class T, int CW>
__global__ void __launch_bounds__(256) skinny_rows_kernel(const SkinnyTask<T>* __restrict__ tasks, int count, int k) {
  __shared__ T Bs[CW][SK_CHUNK + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int u = blockIdx.x;
  const SkinnyTask<T> t = tasks[find_skinny(tasks, count, u)];
  const int cg = (k + CW - 1) / CW;
  const int local = u - t.unitBase, rb = local / cg, c0 = (local - rb * cg) * CW;
  const int i0 = rb * 16 + warp * 2;
  T acc[2][CW];
#pragma unroll
  for (int q = 0; q < CW; ++q) acc[0][q] = acc[1][q] = T(0);
  const T* a0 = t.A + (size_t)min(i0, t.M - 1) * t.lda;
  const T* a1 = t.A + (size_t)min(i0 + 1, t.M - 1) * t.lda;
  for (int kk0 = 0; kk0 < t.K; kk0 += SK_CHUNK) {
    T av[2][SK_CHUNK / 32];
#pragma unroll
    for (int s = 0; s < SK_CHUNK / 32; ++s) {
      const int kk = kk0 + lane + 32 * s;
      av[0][s] = kk < t.K ? a0[kk] : T(0);
      av[1][s] = kk < t.K ? a1[kk] : T(0);
    }
    for (int e = threadIdx.x; e < SK_CHUNK * CW; e += blockDim.x) {
      const int l = e / CW, q = e - l * CW;
      Bs[q][l] = (kk0 + l < t.K && c0 + q < k) ? t.B[(size_t)(kk0 + l) * t.ldb + c0 + q] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < SK_CHUNK / 32; ++s)
#pragma unroll
      for (int q = 0; q < CW; ++q) {
        const T b = Bs[q][lane + 32 * s];
        acc[0][q] += av[0][s] * b;
        acc[1][q] += av[1][s] * b;
      }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    const int i = i0 + r;
#pragma unroll
    for (int q = 0; q < CW; ++q) {
      const T v = warp_sum(acc[r][q]);
      if (lane == q && i < t.M && c0 + q < k) {
        T* c = t.C + (size_t)i * t.ldc + c0 + q;
        T o = t.alpha * v;
        if (t.beta != T(0)) o += t.beta * *c;
        *c = o;
      }
    }
  }
}

// Transposed form, A stored K x M (op(A)[i][kk] = A[kk][i]).  A block per
// (64 rows, column group): lanes take rows i0 + lane and i0 + lane + 32
// (coalesced along A's rows), warp w adds kk = w, w + 8, ... in order, and
// the 8 warp partials are added in warp order.
template <class T, int CW>
__global__ void __launch_bounds__(256) skinny_cols_kernel(const SkinnyTask<T>* __restrict__ tasks, int count, int k) {
  // warp partials go through shared memory QB columns at a time (<= 32 KB)
  constexpr int QB = sizeof(T) * 8 * 64 * CW > 32768 ? CW / 2 : CW;
  __shared__ T red[8][64][QB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int u = blockIdx.x;
  const SkinnyTask<T> t = tasks[find_skinny(tasks, count, u)];
  const int cg = (k + CW - 1) / CW;
  const int local = u - t.unitBase, rb = local / cg, c0 = (local - rb * cg) * CW;
  const int i0 = rb * 64;
  const bool v0 = i0 + lane < t.M, v1 = i0 + lane + 32 < t.M;
  T acc[2][CW];
#pragma unroll
  for (int q = 0; q < CW; ++q) acc[0][q] = acc[1][q] = T(0);
#pragma unroll 8
  for (int kk = warp; kk < t.K; kk += 8) {
    const T* arow = t.A + (size_t)kk * t.lda + i0;
    const T a0 = v0 ? arow[lane] : T(0), a1 = v1 ? arow[lane + 32] : T(0);
    const T* b = t.B + (size_t)kk * t.ldb + c0;
#pragma unroll
    for (int q = 0; q < CW; ++q) {
      const T bv = c0 + q < k ? b[q] : T(0);
      acc[0][q] += a0 * bv;
      acc[1][q] += a1 * bv;
    }
  }
#pragma unroll
  for (int qb = 0; qb < CW; qb += QB) {
#pragma unroll
    for (int q = 0; q < QB; ++q) {
      red[warp][lane][q] = acc[0][qb + q];
      red[warp][lane + 32][q] = acc[1][qb + q];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * QB; e += blockDim.x) {
      const int r = e / QB, q = e - r * QB;
      if (i0 + r >= t.M || c0 + qb + q >= k) continue;
      T v = T(0);
#pragma unroll
      for (int w = 0; w < 8; ++w) v += red[w][r][q];
      T* c = t.C + (size_t)(i0 + r) * t.ldc + c0 + qb + q;
      T o = t.alpha * v;
      if (t.beta != T(0)) o += t.beta * *c;
      *c = o;
    }
    __syncthreads();
  }
}

// Long-K products of the batched apply run as K slices (each slice's product
// to its own block of a workspace, so many more tiles are in flight at small
// k); this kernel then forms C = alpha * (slice 0 + slice 1 + ...) + beta * C,
// slices added in order.  The slicing depends on K alone, so the arithmetic of
// a column does not depend on how many columns the block has.
template <class T>
struct SliceSum {
  T* C;
  const T* ws;   // slices x M x N, row stride N
  int ldc, M, N, slices;
  T alpha, beta;
};

template <class T>
__global__ void __launch_bounds__(256) slice_sum_kernel(const SliceSum<T>* __restrict__ sums) {
  const SliceSum<T> t = sums[blockIdx.y];
  const long long mn = (long long)t.M * t.N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < mn; e += (long long)gridDim.x * blockDim.x) {
    T s = T(0);
    for (int q = 0; q < t.slices; ++q) s += t.ws[q * mn + e];
    const int i = (int)(e / t.N), j = (int)(e - (long long)i * t.N);
    T* c = t.C + (size_t)i * t.ldc + j;
    T v = t.alpha * s;
    if (t.beta != T(0)) v += t.beta * *c;
    *c = v;
  }
}

template <class A, class B>
__global__ void convert_k_kernel(const A* __restrict__ src, B* __restrict__ dst, long long count,
                                 int* __restrict__ clr = nullptr, int nClr = 0) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (B)src[i];
  // the last kernel of a batched apply also zeroes the interior completion
  // counters (their last reader, the backward launch, has finished)
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nClr; i += gridDim.x * blockDim.x) clr[i] = 0;
}

int skinny_width(int k) {
  int p = 1;
  while (p < k) p <<= 1;
  return p;
}

// columns per unit: k rounded up to a power of two, at most 16 (row form) or
// 8 (transposed form, whose B values are broadcast loads)
int skinny_cw(int k, bool cols) { return std::min(cols ? 8 : 16, skinny_width(k)); }

}  // namespace

template <class T>
int SolveEngine<T>::batch_capacity() const {
  const size_t per = sizeof(T) * (size_t)(maxNI_ + 64);
  const int bySmem = (int)std::min<size_t>(64, (200 * 1024) / std::max<size_t>(per, 1));
  return std::max(1, bySmem);
}

template <class T>
void SolveEngine<T>::plan_batch(int k, int cwR, int cwC) {
  const int key = k * 256 + cwR * 16 + cwC;   // cwR <= 16, cwC <= 8
  if (key == kB_) return;
  const Symbolic& S = F_.S;
  cudaStream_t st = F_.stream;
  if (k > kAllocB_) {
    dWuB_.alloc(sizeof(T) * std::max(1LL, wuTotal_ * k));
    dYB_.alloc(sizeof(T) * std::max<long long>(1, (long long)S.n * k));
    dIpB_.alloc(sizeof(T) * std::max(1LL, ipTotal_ * k));
    if (!dSyncB_.p) {
      dSyncB_.alloc(sizeof(int) * syncInts_);
      RSCHOL_CUDA(cudaMemsetAsync(dSyncB_.p, 0, sizeof(int) * syncInts_, st));
    }
    dWB_.alloc(sizeof(T) * std::max<long long>(1, (long long)S.n * k));   // the working copy of W
    kAllocB_ = k;
    ++batchGen_;
    bPlans_.clear();   // the task lists point into the old buffers
  }
  auto found = bPlans_.find(key);
  if (found != bPlans_.end()) {
    bPlan_ = &found->second;
    kB_ = key;
    return;
  }
  BatchPlan& plan = bPlans_[key];
  // products of the compressed levels (skinny SIMT kernels)
  std::vector<SkinnyTask<T>> tasks;
  auto& steps = plan.steps;
  steps.assign(6 * cLevels_.size(), {});
  T* wu = dWuB_.as<T>();
  T* yb = dYB_.as<T>();
  T* w = dWB_.as<T>();
  // column groups of the two product forms
  const int cgR = (k + cwR - 1) / cwR;
  const int cgC = (k + cwC - 1) / cwC;
  struct Prod {   // one product before it is cut into units
    const T* A;
    const T* B;
    T* C;
    int M, K, lda, ldb, ldc;
    bool tA;
    T alpha, beta;
  };
  auto mk = [&](const T* A, int lda, bool tA, const T* B, int ldb, T* C, int ldc, int M, int, int K, T alpha,
                T beta) { return Prod{A, B, C, M, K, lda, ldb, ldc, tA, alpha, beta}; };
  // K slicing of the transposed form (a thread runs down K): tasks with K
  // above kSliceMin run as slices of kSlice into a workspace, then a
  // fixed-order sum; the slicing depends on K alone
  constexpr int kSlice = 512, kSliceMin = 768;
  std::vector<SliceSum<T>> sums;
  std::vector<std::pair<size_t, long long>> taskWs;   // (task, workspace offset) to patch
  std::vector<std::pair<size_t, long long>> sumWs;    // (sum, workspace offset) to patch
  long long wsTotal = 0;
  auto flush = [&](std::vector<Prod>& batch, int slot) {
    if (batch.empty()) return;
    const bool cols = batch[0].tA;   // a flush holds one form
    std::vector<SkinnyTask<T>> run;
    const long long sum0 = (long long)sums.size();
    long long maxMN = 0, wsStep = 0;
    auto add = [&](const Prod& g, T* C, int ldc, T alpha, T beta) {
      run.push_back(SkinnyTask<T>{g.A, g.B, C, g.M, g.K, g.lda, g.ldb, ldc, alpha, beta, 0});
    };
    for (const Prod& g : batch) {
      if (!cols || g.K <= kSliceMin) {
        add(g, g.C, g.ldc, g.alpha, g.beta);
        continue;
      }
      const int ns = (g.K + kSlice - 1) / kSlice;
      const long long mn = (long long)g.M * k;
      sumWs.push_back({sums.size(), wsStep});
      sums.push_back(SliceSum<T>{g.C, nullptr, g.ldc, g.M, k, ns, g.alpha, g.beta});
      for (int q = 0; q < ns; ++q) {
        Prod t = g;
        t.K = std::min(kSlice, g.K - q * kSlice);
        t.A = g.A + (size_t)q * kSlice * g.lda;
        t.B = g.B + (size_t)q * kSlice * g.ldb;
        taskWs.push_back({tasks.size() + run.size(), wsStep + q * mn});
        add(t, nullptr, k, T(1), T(0));
      }
      wsStep += ns * mn;
      maxMN = std::max(maxMN, mn);
    }
    wsTotal = std::max(wsTotal, wsStep);   // every step's slices start at the workspace base
    int units = 0;   // one block per unit: (16 rows | 64 rows, column group)
    for (auto& t : run) {
      t.unitBase = units;
      units += cols ? (t.M + 63) / 64 * cgC : (t.M + 15) / 16 * cgR;
    }
    XStep xs{(long long)tasks.size(), (int)run.size(), units, cols ? 1 : 0};
    xs.redOff = sum0;
    xs.redCount = (int)(sums.size() - sum0);
    xs.redGrid = (int)std::min<long long>(64, (maxMN + 255) / 256);
    steps[slot].push_back(xs);
    tasks.insert(tasks.end(), run.begin(), run.end());
    batch.clear();
  };
  const int L = (int)cLevels_.size();
  for (int l = 0; l < L; ++l) {
    std::vector<Prod> gy, gz, gu, gs, gg, gx;
    for (int q = 0; q < cLevels_[l].second; ++q) {
      const int j = F_.compressedLevels[l][q];
      const SNode<T>& nd = nodes_[j];
      const int n = nd.n, m = nd.m, r = nd.r;
      T* z = wu + nd.wuOff * k;
      T* sv = wu + (nd.wuOff + r) * k;
      T* u = wu + (nd.wuOff + 2 * r) * k;
      T* yj = yb + (size_t)nd.c0 * k;
      T* wj = w + (size_t)nd.c0 * k;
      for (int ib = 0; ib < nd.nb; ++ib) {   // Y = X F by row blocks
        const int h = std::min(64, n - ib * 64), K = std::min(n, (ib + 1) * 64);
        gy.push_back(mk(nd.X + (size_t)ib * 64 * n, n, false, wj, k, yj + (size_t)ib * 64 * k, k, h, k, K, T(1),
                        T(0)));
      }
      if (r > 0) {
        gz.push_back(mk(nd.U, r, true, yj, k, z, k, r, k, n, T(1), T(0)));
        if (m > 0 && l + 1 < L) gu.push_back(mk(nd.V, r, false, z, k, u, k, m, k, r, T(-1), T(0)));
        if (m > 0) {
          gs.push_back(mk(nd.V, r, true, u, k, sv, k, r, k, m, T(1), T(0)));
          gg.push_back(mk(nd.U, r, false, sv, k, yj, k, n, k, r, T(-1), T(1)));
        }
      }
      for (int jb = 0; jb < nd.nb; ++jb) {   // X = X^T G by column blocks
        const int h = std::min(64, n - jb * 64), K = n - jb * 64;
        gx.push_back(mk(nd.X + (size_t)jb * 64 * n + jb * 64, n, true, yj + (size_t)jb * 64 * k, k,
                        wj + (size_t)jb * 64 * k, k, h, k, K, T(1), T(0)));
      }
    }
    flush(gy, 6 * l + 0);
    flush(gz, 6 * l + 1);
    flush(gu, 6 * l + 2);
    flush(gs, 6 * l + 3);
    flush(gg, 6 * l + 4);
    flush(gx, 6 * l + 5);
  }
  plan.ws.alloc(sizeof(T) * std::max(1LL, wsTotal));
  T* ws = plan.ws.template as<T>();
  for (auto& tw : taskWs) tasks[tw.first].C = ws + tw.second;
  for (auto& sw : sumWs) sums[sw.first].ws = ws + sw.second;
  plan.sums.alloc(std::max<size_t>(16, sums.size() * sizeof(SliceSum<T>)));
  if (!sums.empty())
    RSCHOL_CUDA(cudaMemcpyAsync(plan.sums.p, sums.data(), sums.size() * sizeof(SliceSum<T>), cudaMemcpyHostToDevice,
                                st));
  plan.tasks.alloc(std::max<size_t>(16, tasks.size() * sizeof(SkinnyTask<T>)));
  if (!tasks.empty())
    RSCHOL_CUDA(cudaMemcpyAsync(plan.tasks.p, tasks.data(), tasks.size() * sizeof(SkinnyTask<T>),
                                cudaMemcpyHostToDevice, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  bPlan_ = &plan;
  kB_ = key;
}

template <class T>
typename SolveEngine<T>::BatchCfg SolveEngine<T>::heuristic_cfg(int kp) const {
  // what the tuner picks on 2D and 3D diffusion factors of 0.26 - 1 M
  // unknowns: 1 x 1 pair tiles up to 16 columns, 2 x 4 above; row-form groups
  // of up to 16 columns; transposed-form groups of 4, 8 from 16 columns on
  BatchCfg c;
  if (kp >= 32) c.ra = 2, c.rc = 4;
  c.cwR = std::min(16, skinny_width(kp));
  c.cwC = std::min(kp >= 16 ? 8 : 4, skinny_width(kp));
  return c;
}

// The width class of k is kp = k rounded up to a power of two (<= the batch
// capacity); its shapes are timed once, at k = kp, on a zero block: first the
// interior pair tile, then the row-form and the transposed-form column
// groups, each over a handful of candidates, the fastest of two timed
// applies after one warm-up.
template <class T>
int SolveEngine<T>::width_class(int k) const {
  return std::min(skinny_width(k), std::max(k, batch_capacity()));
}

template <class T>
const typename SolveEngine<T>::BatchCfg& SolveEngine<T>::config_for(int k, cudaStream_t st, bool tune) {
  const int kp = width_class(k);
  auto it = tuned_.find(kp);
  if (it != tuned_.end() && (it->second.ms > 0 || !tune)) return it->second;
  BatchCfg best = heuristic_cfg(kp);
  if (tune) {
    const size_t bytes = sizeof(double) * (size_t)std::max(1, F_.S.n) * kp;
    DevBuf zero;
    zero.alloc(bytes);
    RSCHOL_CUDA(cudaMemsetAsync(zero.p, 0, bytes, st));
    cudaEvent_t e0, e1;
    RSCHOL_CUDA(cudaEventCreate(&e0));
    RSCHOL_CUDA(cudaEventCreate(&e1));
    auto time_cfg = [&](const BatchCfg& c) {
      apply_batch_cfg(zero.as<double>(), kp, st, c);   // warm-up (plans this shape)
      float bestMs = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        RSCHOL_CUDA(cudaEventRecord(e0, st));
        apply_batch_cfg(zero.as<double>(), kp, st, c);
        RSCHOL_CUDA(cudaEventRecord(e1, st));
        RSCHOL_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        RSCHOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        bestMs = std::min(bestMs, ms);
      }
      return (double)bestMs;
    };
    best.ms = time_cfg(best);
    auto consider = [&](BatchCfg c) {
      if (c.ra == best.ra && c.rc == best.rc && c.cwR == best.cwR && c.cwC == best.cwC) return;
      c.ms = time_cfg(c);
      if (c.ms < best.ms) best = c;
    };
    const int tiles[4][2] = {{1, 1}, {1, 4}, {2, 4}, {4, 4}};
    for (auto& tl : tiles) {
      BatchCfg c = best;
      c.ra = tl[0];
      c.rc = tl[1];
      consider(c);
    }
    for (int cw = 4; cw <= std::min(16, kp); cw *= 2) {
      BatchCfg c = best;
      c.cwR = cw;
      consider(c);
    }
    for (int cw = 2; cw <= std::min(8, kp); cw *= 2) {
      BatchCfg c = best;
      c.cwC = cw;
      consider(c);
    }
    RSCHOL_CUDA(cudaEventDestroy(e0));
    RSCHOL_CUDA(cudaEventDestroy(e1));
  }
  ++batchGen_;   // new tile shapes: a captured apply would use the old ones
  return tuned_[kp] = best;
}

template <class T>
void SolveEngine<T>::autotune_batch(int kmax, cudaStream_t st) {
  kmax = std::min(kmax, batch_capacity());
  for (int k = 1; k <= kmax; k = width_class(k) + 1) config_for(k, st, true);
}

template <class T>
std::vector<std::array<double, 6>> SolveEngine<T>::batch_tuning() const {
  std::vector<std::array<double, 6>> out;
  for (const auto& kv : tuned_)
    out.push_back({(double)kv.first, (double)kv.second.ra, (double)kv.second.rc, (double)kv.second.cwR,
                   (double)kv.second.cwC, kv.second.ms});
  return out;
}

template <class T>
void SolveEngine<T>::apply_batch(double* W64, int k, cudaStream_t st) {
  if (k <= 0) return;
  if (k > batch_capacity()) throw std::runtime_error("apply_batch: more right-hand sides than one pass handles");
  apply_batch_cfg(W64, k, st, config_for(k, st, autotune_));
}

template <class T>
void SolveEngine<T>::apply_batch_cfg(double* W64, int k, cudaStream_t st, const BatchCfg& cfg) {
  plan_batch(k, cfg.cwR, cfg.cwC);
  const int n = F_.S.n;
  const long long nk = (long long)n * k;
  T* w = dWB_.as<T>();
  convert_k_kernel<double, T><<<(unsigned)std::min<long long>((nk + 255) / 256, 4096), 256, 0, st>>>(W64, w, nk);
  RSCHOL_LAUNCH_CHECK();
  // completion targets: every apply starts its counters at zero (they are
  // cleared by its last kernel), so the apply keeps no host state and replays
  // inside CUDA graphs
  const int epoch = 1;
  int* sync = dSyncB_.as<int>();
  const size_t smem = sizeof(T) * (size_t)(maxNI_ + 64) * k;
  static std::once_flag once;
  std::call_once(once, [] {
    const int sm = 200 * 1024;
#define RSCHOL_SMEM_ATTR(RA, RC)                                                                                \
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_forward_k<T, RA, RC>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm)); \
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_backward_k<T, RA, RC>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))
    RSCHOL_SMEM_ATTR(1, 1);
    RSCHOL_SMEM_ATTR(1, 4);
    RSCHOL_SMEM_ATTR(2, 4);
    RSCHOL_SMEM_ATTR(4, 4);
#undef RSCHOL_SMEM_ATTR
  });
  // register tiles of (row, column) pairs (BatchCfg)
  using IF = decltype(&interior_forward_k<T, 1, 1>);
  using IB = decltype(&interior_backward_k<T, 1, 1>);
  IF fwd = interior_forward_k<T, 1, 1>;
  IB bwd = interior_backward_k<T, 1, 1>;
  if (cfg.ra == 4) {
    fwd = interior_forward_k<T, 4, 4>;
    bwd = interior_backward_k<T, 4, 4>;
  } else if (cfg.ra == 2) {
    fwd = interior_forward_k<T, 2, 4>;
    bwd = interior_backward_k<T, 2, 4>;
  } else if (cfg.rc == 4) {
    fwd = interior_forward_k<T, 1, 4>;
    bwd = interior_backward_k<T, 1, 4>;
  }
  if (nIWork_ > 0) {
    fwd<<<nIWork_, 256, smem, st>>>(dNodes_.as<SNode<T>>(), dIWork_.as<RowBlock>(), dRel_.as<int>(), dChild_.as<int>(),
                                    sync, epoch, k, w, dYB_.as<T>(), dWuB_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  const int* lvl = dLevelNodes_.as<int>();
  const SkinnyTask<T>* bg = bPlan_->tasks.template as<SkinnyTask<T>>();
  auto gemm = [&](int slot) {
    for (const XStep& x : bPlan_->steps[slot]) {
      const SkinnyTask<T>* tk = bg + x.off;
      const int cw = x.tc ? cfg.cwC : cfg.cwR;
#define RSCHOL_SKINNY(CW)                                                     \
  if (x.tc) skinny_cols_kernel<T, CW><<<x.tiles, 256, 0, st>>>(tk, x.count, k); \
  else skinny_rows_kernel<T, CW><<<x.tiles, 256, 0, st>>>(tk, x.count, k)
      switch (cw) {
        case 1: RSCHOL_SKINNY(1); break;
        case 2: RSCHOL_SKINNY(2); break;
        case 4: RSCHOL_SKINNY(4); break;
        case 8: RSCHOL_SKINNY(8); break;
        default: RSCHOL_SKINNY(16); break;
      }
#undef RSCHOL_SKINNY
      RSCHOL_LAUNCH_CHECK();
      if (x.redCount > 0) {
        slice_sum_kernel<T><<<dim3(x.redGrid, x.redCount), 256, 0, st>>>(bPlan_->sums.template as<SliceSum<T>>() +
                                                                         x.redOff);
        RSCHOL_LAUNCH_CHECK();
      }
    }
  };
  const int L = (int)cLevels_.size();
  for (int l = 0; l < L; ++l) {
    const int* lv = lvl + cLevels_[l].first;
    compressed_gather_k<T><<<dim3(cRowGrid_[l], cLevels_[l].second), 256, 0, st>>>(
        dNodes_.as<SNode<T>>(), lv, dCStart_.as<long long>(), dCEnt_.as<long long>(), k, dWuB_.as<T>(), w);
    RSCHOL_LAUNCH_CHECK();
    gemm(6 * l + 0);
    gemm(6 * l + 1);
    gemm(6 * l + 2);
  }
  for (int l = L - 1; l >= 0; --l) {
    const int* lv = lvl + cLevels_[l].first;
    compressed_gather_xr_k<T><<<dim3(cMRowGrid_[l], cLevels_[l].second), 256, 0, st>>>(
        dNodes_.as<SNode<T>>(), lv, dRows_.as<int>(), k, w, dWuB_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    gemm(6 * l + 3);
    gemm(6 * l + 4);
    gemm(6 * l + 5);
  }
  if (nIWork_ > 0) {
    bwd<<<nIWork_, 256, smem, st>>>(dNodes_.as<SNode<T>>(), dIWorkB_.as<RowBlock>(), dRows_.as<int>(), sync, epoch,
                                    k, dIpB_.as<T>(), dYB_.as<T>(), w);
    RSCHOL_LAUNCH_CHECK();
  }
  convert_k_kernel<T, double><<<(unsigned)std::min<long long>((nk + 255) / 256, 4096), 256, 0, st>>>(
      w, W64, nk, nIWork_ > 0 ? sync + SYNC_GLOBAL : nullptr, nIWork_ > 0 ? syncInts_ - SYNC_GLOBAL : 0);
  RSCHOL_LAUNCH_CHECK();
}

template <class T>
int SolveEngine<T>::take_error_batch(cudaStream_t st) {
  int e = 0;
  if (!dSyncB_.p) return 0;
  RSCHOL_CUDA(cudaMemcpyAsync(&e, dSyncB_.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  if (e) {
    RSCHOL_CUDA(cudaMemsetAsync(dSyncB_.p, 0, sizeof(int) * syncInts_, st));
    RSCHOL_CUDA(cudaStreamSynchronize(st));
  }
  return e;
}

template int SolveEngine<double>::batch_capacity() const;
template int SolveEngine<float>::batch_capacity() const;
template void SolveEngine<double>::plan_batch(int, int, int);
template void SolveEngine<float>::plan_batch(int, int, int);
template SolveEngine<double>::BatchCfg SolveEngine<double>::heuristic_cfg(int) const;
template SolveEngine<float>::BatchCfg SolveEngine<float>::heuristic_cfg(int) const;
template const SolveEngine<double>::BatchCfg& SolveEngine<double>::config_for(int, cudaStream_t, bool);
template const SolveEngine<float>::BatchCfg& SolveEngine<float>::config_for(int, cudaStream_t, bool);
template int SolveEngine<double>::width_class(int) const;
template int SolveEngine<float>::width_class(int) const;
template void SolveEngine<double>::autotune_batch(int, cudaStream_t);
template void SolveEngine<float>::autotune_batch(int, cudaStream_t);
template void SolveEngine<double>::apply_batch_cfg(double*, int, cudaStream_t, const BatchCfg&);
template void SolveEngine<float>::apply_batch_cfg(double*, int, cudaStream_t, const BatchCfg&);
template std::vector<std::array<double, 6>> SolveEngine<double>::batch_tuning() const;
template std::vector<std::array<double, 6>> SolveEngine<float>::batch_tuning() const;
template void SolveEngine<double>::apply_batch(double*, int, cudaStream_t);
template void SolveEngine<float>::apply_batch(double*, int, cudaStream_t);
template int SolveEngine<double>::take_error_batch(cudaStream_t);
template int SolveEngine<float>::take_error_batch(cudaStream_t);

}  // namespace rschol
