#include <algorithm>
#include <type_traits>

#include "solve.cuh"

namespace rschol {

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <class V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

// f := L^{-1} f for a dense lower L (n x n, leading dimension ld); f in
// shared memory.  32-wide tiles: warp 0 solves the diagonal tile, then every
// thread updates its own rows below with a 32-term dot product whose 32
// loads are independent (memory-level parallelism instead of one
// latency-bound warp reduction per row).
template <class T>
__device__ void trsv_lower(const T* __restrict__ L, int ld, int n, T* f, T (*tile)[33]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int tw = min(32, n - t0);
    for (int idx = threadIdx.x; idx < tw * tw; idx += blockDim.x) {
      int i = idx / tw, j = idx - i * tw;
      tile[i][j] = (j <= i) ? L[(size_t)(t0 + i) * ld + t0 + j] : T(0);
    }
    __syncthreads();
    if (warp == 0) {
      T v = (lane < tw) ? f[t0 + lane] : T(0);
      for (int j = 0; j < tw; ++j) {
        const T yj = __shfl_sync(FULL, v, j) / tile[j][j];
        if (lane == j) v = yj;
        else if (lane > j && lane < tw) v -= tile[lane][j] * yj;
      }
      if (lane < tw) f[t0 + lane] = v;
    }
    __syncthreads();
    for (int i = t0 + tw + threadIdx.x; i < n; i += blockDim.x) {
      const T* row = L + (size_t)i * ld + t0;
      T s = T(0);
      if (tw == 32) {
#pragma unroll
        for (int k = 0; k < 32; ++k) s += row[k] * f[t0 + k];
      } else {
        for (int k = 0; k < tw; ++k) s += row[k] * f[t0 + k];
      }
      f[i] -= s;
    }
    __syncthreads();
  }
}

// out[k] = sum_{i < rows} M[i][k] * v(i) for k < cols (M row-major, ld),
// computed by nGroups groups of threads that split the rows, then a
// fixed-order reduction of the group partials in shared memory.
// scratch: nGroups * cols doubles of shared memory.
template <class T, class VecFn>
__device__ void gemv_t_split(const T* __restrict__ M, int ld, int rows, int cols, VecFn v, T* out,
                             T* scratch) {
  const int groups = max(1, (int)blockDim.x / max(cols, 1));
  const int g = threadIdx.x / max(cols, 1), k = threadIdx.x - g * max(cols, 1);
  if (cols <= (int)blockDim.x) {
    if (g < groups) {
      T s = T(0);
      for (int i = g; i < rows; i += groups) s += M[(size_t)i * ld + k] * v(i);
      scratch[g * cols + k] = s;
    }
    __syncthreads();
    for (int kk = threadIdx.x; kk < cols; kk += blockDim.x) {
      T s = T(0);
      for (int q = 0; q < groups; ++q) s += scratch[q * cols + kk];
      out[kk] = s;
    }
  } else {
    for (int kk = threadIdx.x; kk < cols; kk += blockDim.x) {
      T s = T(0);
      for (int i = 0; i < rows; ++i) s += M[(size_t)i * ld + kk] * v(i);
      out[kk] = s;
    }
  }
  __syncthreads();
}

// f := L^{-T} f.
template <class T>
__device__ void trsv_lower_t(const T* __restrict__ L, int ld, int n, T* f, T (*tile)[33]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (n <= 0) return;
  for (int t0 = ((n - 1) / 32) * 32; t0 >= 0; t0 -= 32) {
    const int tw = min(32, n - t0);
    for (int idx = threadIdx.x; idx < tw * tw; idx += blockDim.x) {
      int i = idx / tw, j = idx - i * tw;
      tile[i][j] = (j <= i) ? L[(size_t)(t0 + i) * ld + t0 + j] : T(0);
    }
    __syncthreads();
    if (warp == 0) {
      T v = (lane < tw) ? f[t0 + lane] : T(0);
      for (int j = tw - 1; j >= 0; --j) {
        const T xj = __shfl_sync(FULL, v, j) / tile[j][j];
        if (lane == j) v = xj;
        else if (lane < j) v -= tile[j][lane] * xj;
      }
      if (lane < tw) f[t0 + lane] = v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < t0; i += blockDim.x) {
      T s = T(0);
      for (int k = 0; k < tw; ++k) s += L[(size_t)(t0 + k) * ld + i] * f[t0 + k];
      f[i] -= s;
    }
    __syncthreads();
  }
}

template <class T>
__global__ void __launch_bounds__(256) interior_forward_kernel(const SNode<T>* __restrict__ nodes,
                                                               const int* __restrict__ lvl,
                                                               const int* __restrict__ rows,
                                                               const int* __restrict__ rel,
                                                               const int* __restrict__ child,
                                                               T* __restrict__ w, T* __restrict__ wu) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* f = reinterpret_cast<T*>(smraw);
  __shared__ T tile[32][33];
  const SNode<T> nd = nodes[lvl[blockIdx.x]];
  T* wud = wu + nd.wuOff;
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) f[i] = w[nd.c0 + i];
  for (int a = threadIdx.x; a < nd.m; a += blockDim.x) wud[a] = 0.0;
  __syncthreads();
  for (int c = nd.childBegin; c < nd.childEnd; ++c) {
    const SNode<T> cn = nodes[child[c]];
    const T* wuc = wu + cn.wuOff;
    const int* rl = rel + cn.relOff;
    for (int a = threadIdx.x; a < cn.m; a += blockDim.x) {
      const int t = rl[a];
      if (t < nd.n) f[t] += wuc[a];
      else wud[t - nd.n] += wuc[a];
    }
    __syncthreads();
  }
  trsv_lower<T>(nd.L, nd.ld, nd.n, f, tile);
  // update vector: wud -= L21 y, one thread per row (independent loads)
  for (int a = threadIdx.x; a < nd.m; a += blockDim.x) {
    const T* row = nd.L + (size_t)(nd.n + a) * nd.ld;
    T s = T(0);
    for (int j = 0; j < nd.n; ++j) s += row[j] * f[j];
    wud[a] -= s;
  }
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) w[nd.c0 + i] = f[i];
}

template <class T>
__global__ void __launch_bounds__(256) interior_backward_kernel(const SNode<T>* __restrict__ nodes,
                                                                const int* __restrict__ lvl,
                                                                const int* __restrict__ rows,
                                                                T* __restrict__ w) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  __shared__ T tile[32][33];
  __shared__ T scratch[256];
  const SNode<T> nd = nodes[lvl[blockIdx.x]];
  T* f = sm;
  T* t = sm + nd.n;
  T* xr = sm + 2 * nd.n;
  const int* rw = rows + nd.rowsOff;
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) f[i] = w[nd.c0 + i];
  for (int a = threadIdx.x; a < nd.m; a += blockDim.x) xr[a] = w[rw[a]];
  __syncthreads();
  if (nd.m > 0) {
    // t = L21^T x_R with the rows split over thread groups
    gemv_t_split<T>(nd.L + (size_t)nd.n * nd.ld, nd.ld, nd.m, nd.n, [&](int a) { return xr[a]; }, t, scratch);
    for (int i = threadIdx.x; i < nd.n; i += blockDim.x) f[i] -= t[i];
    __syncthreads();
  }
  trsv_lower_t<T>(nd.L, nd.ld, nd.n, f, tile);
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) w[nd.c0 + i] = f[i];
}

// ---------------------------------------------------------------------------
// Compressed supernodes: 64-row blocks, one thread block (256 threads, warp w
// owning rows 8w..8w+7 of the block) per row block.

constexpr int SPIN_LIMIT = 1 << 22;   // polls (with a short sleep) before a wait gives up

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *(const volatile int*)p; }

// Warp-uniform bounded wait for *flag != 0.  Returns false when the wait gave
// up (after SPIN_LIMIT polls, or as soon as another block reported an error);
// the error word is then set.
__device__ __forceinline__ bool wait_ready(const int* flag, int* err) {
  if (__all_sync(FULL, ld_acquire(flag) != 0)) return true;
  for (int it = 1; it <= SPIN_LIMIT; ++it) {
    __nanosleep(64);
    if (__all_sync(FULL, ld_acquire(flag) != 0)) return true;
    if ((it & 63) == 0 && __any_sync(FULL, ld_volatile(err) != 0)) return false;
  }
  if ((threadIdx.x & 31) == 0) atomicExch(err, 1);
  return false;
}

// After the block's own results are stored: publish them (ready flag), and
// let the last block of the supernode and the last block of the launch reset
// the counters for the next apply.  Returns true in the supernode's last block
// (all of its blocks have stored their partials and left their waits).
__device__ __forceinline__ bool finish_row_block(int* flag, int* nodeDone, int nb, int* levelTick, int* levelDone, int* sLast) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    st_release(flag, 1);
    const int d = atomicAdd(nodeDone, 1);
    *sLast = (d == nb - 1);
    if (atomicAdd(levelDone, 1) == (int)gridDim.x - 1) {
      atomicExch(levelTick, 0);
      atomicExch(levelDone, 0);
    }
    __threadfence();
  }
  __syncthreads();
  return *sLast != 0;
}

// acc[rr] (row 8w+rr of the block) += P[row][2l] v0 + P[row][2l+1] v1 for a
// 64-column tile P (row-major, ld), rows limited to h.
template <class T>
__device__ __forceinline__ void tile_rows(const T* __restrict__ P, int ld, int h, T v0, T v1, T (&acc)[8]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int rr = 0; rr < 8; ++rr) {
    const int i = warp * 8 + rr;
    if (i < h) {
      const T* p = P + (size_t)i * ld + 2 * lane;
      acc[rr] += p[0] * v0 + p[1] * v1;
    }
  }
}

// Forward row block: f_b = w_b + contributions - sum_{k<b} L[b,k] y_k,
// y_b = Dinv_b f_b, partial z_b = U_b^T y_b.
template <class T>
__global__ void __launch_bounds__(256) compressed_forward_blocks(const SNode<T>* __restrict__ nodes,
                                                                 const RowBlock* __restrict__ tickets,
                                                                 const long long* __restrict__ cstart,
                                                                 const CEntry<T>* __restrict__ ent,
                                                                 int* __restrict__ sync, int levelSync,
                                                                 T* __restrict__ zpart, T* __restrict__ w,
                                                                 T* __restrict__ wu) {
  __shared__ int sTicket, sLast;
  __shared__ T fb[SOLVE_RB], yb[SOLVE_RB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* err = sync;
  if (threadIdx.x == 0) sTicket = atomicAdd(&sync[levelSync], 1);
  __syncthreads();
  if (sTicket >= (int)gridDim.x) {   // counters not reset: report, touch nothing
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const RowBlock tk = tickets[sTicket];
  const SNode<T>& nd = nodes[tk.node];
  const int n = nd.n, i0 = tk.b * SOLVE_RB, h = min(SOLVE_RB, n - i0);
  T* wn = w + nd.c0;
  int* flags = sync + nd.syncOff;
  // 1. right-hand side rows with their contribution lists (warp per row)
  const long long* cs = cstart + nd.cOff;
  for (int rr = 0; rr < 8; ++rr) {
    const int i = warp * 8 + rr;
    T acc = T(0);
    if (i < h) {
      for (long long e = cs[i0 + i]; e < cs[i0 + i + 1]; ++e) {
        const CEntry<T> E = ent[e];
        if (E.r == 0) {
          if (lane == 0) acc += *E.v;
        } else {
          T s = T(0);
          for (int k = lane; k < E.r; k += 32) s += E.v[k] * E.z[k];
          acc -= s;
        }
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) fb[i] = (i < h) ? wn[i0 + i] + acc : T(0);
  }
  // 2. earlier row blocks, as they become ready
  T acc[8];
#pragma unroll
  for (int rr = 0; rr < 8; ++rr) acc[rr] = T(0);
  bool ok = true;
  for (int kb = 0; kb < tk.b && ok; ++kb) {
    ok = wait_ready(flags + kb, err);
    const T y0 = __ldcg(wn + kb * SOLVE_RB + 2 * lane), y1 = __ldcg(wn + kb * SOLVE_RB + 2 * lane + 1);
    tile_rows<T>(nd.L + (size_t)i0 * nd.ld + kb * SOLVE_RB, nd.ld, h, y0, y1, acc);
  }
  __syncwarp();
#pragma unroll
  for (int rr = 0; rr < 8; ++rr) {
    const T s = warp_sum(acc[rr]);
    if (lane == 0) fb[warp * 8 + rr] -= s;
  }
  __syncthreads();
  // 3. y_b = Dinv_b f_b
  {
    T d[8];
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) d[rr] = T(0);
    tile_rows<T>(nd.Dinv + (size_t)tk.b * SOLVE_RB * SOLVE_RB, SOLVE_RB, h, fb[2 * lane], fb[2 * lane + 1], d);
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      const T s = warp_sum(d[rr]);
      const int i = warp * 8 + rr;
      if (lane == 0) {
        yb[i] = (i < h) ? s : T(0);
        if (i < h) wn[i0 + i] = s;
      }
    }
  }
  __syncthreads();
  // 4. partial z_b = U_b^T y_b
  const int r = nd.r;
  for (int k = threadIdx.x; k < r; k += blockDim.x) {
    T s = T(0);
    for (int i = 0; i < h; ++i) s += nd.U[(size_t)(i0 + i) * r + k] * yb[i];
    zpart[nd.zpOff + (size_t)tk.b * r + k] = s;
  }
  const int nb = nd.nb;
  if (finish_row_block(flags + tk.b, flags + nb, nb, &sync[levelSync], &sync[levelSync + 1], &sLast)) {
    // last row block of this supernode: z in fixed order, then reset the flags
    for (int k = threadIdx.x; k < r; k += blockDim.x) {
      T s = T(0);
      for (int b = 0; b < nb; ++b) s += __ldcg(zpart + nd.zpOff + (size_t)b * r + k);
      wu[nd.wuOff + k] = s;
    }
    for (int b = threadIdx.x; b < nb; b += blockDim.x) flags[b] = 0;
    if (threadIdx.x == 0) flags[nb] = 0;
  }
}

// s = V^T x_R of every compressed supernode of a level: 128-row chunks, then
// the last chunk to finish sums the chunk partials in fixed order.
template <class T>
__global__ void __launch_bounds__(256) compressed_vtx_kernel(const SNode<T>* __restrict__ nodes,
                                                             const int* __restrict__ lvl,
                                                             const int* __restrict__ rows,
                                                             int* __restrict__ sync, T* __restrict__ spart,
                                                             const T* __restrict__ w, T* __restrict__ sv) {
  __shared__ T xs[128];
  __shared__ int sLast;
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int ch = blockIdx.x;
  if (ch >= nd.nch) return;
  const int r = nd.r, a0 = ch * 128, ah = min(128, nd.m - a0);
  const int* rw = rows + nd.rowsOff + a0;
  for (int a = threadIdx.x; a < ah; a += blockDim.x) xs[a] = w[rw[a]];
  __syncthreads();
  for (int k = threadIdx.x; k < r; k += blockDim.x) {
    T s = T(0);
    for (int a = 0; a < ah; ++a) s += nd.V[(size_t)(a0 + a) * r + k] * xs[a];
    spart[nd.spOff + (size_t)ch * r + k] = s;
  }
  __syncthreads();
  int* done = sync + nd.syncOff + nd.nb + 2;
  if (threadIdx.x == 0) {
    __threadfence();
    sLast = (atomicAdd(done, 1) == nd.nch - 1);
    __threadfence();
  }
  __syncthreads();
  if (!sLast) return;
  for (int k = threadIdx.x; k < r; k += blockDim.x) {
    T s = T(0);
    for (int c = 0; c < nd.nch; ++c) s += __ldcg(spart + nd.spOff + (size_t)c * r + k);
    sv[nd.wuOff + r + k] = s;
  }
  if (threadIdx.x == 0) *done = 0;
}

// Backward row block (row blocks in reverse order): g_b = w_b - U_b s,
// v = g_b - sum_{k>b} L[k,b]^T x_k, x_b = Dinv_b^T v.
template <class T>
__global__ void __launch_bounds__(256) compressed_backward_blocks(const SNode<T>* __restrict__ nodes,
                                                                  const RowBlock* __restrict__ tickets,
                                                                  int* __restrict__ sync, int levelSync,
                                                                  const T* __restrict__ sv, T* __restrict__ w) {
  __shared__ int sTicket, sLast;
  __shared__ T gb[SOLVE_RB], vb[SOLVE_RB];
  __shared__ T red[8][SOLVE_RB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int* err = sync;
  if (threadIdx.x == 0) sTicket = atomicAdd(&sync[levelSync], 1);
  __syncthreads();
  if (sTicket >= (int)gridDim.x) {   // counters not reset: report, touch nothing
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const RowBlock tk = tickets[sTicket];
  const SNode<T>& nd = nodes[tk.node];
  const int n = nd.n, nb = nd.nb, i0 = tk.b * SOLVE_RB, h = min(SOLVE_RB, n - i0), r = nd.r;
  T* wn = w + nd.c0;
  int* flags = sync + nd.syncOff;
  // 1. g_b = w_b - U_b s (warp per row)
  const bool offd = r > 0 && nd.m > 0;
  const T* s = sv + nd.wuOff + r;
  for (int rr = 0; rr < 8; ++rr) {
    const int i = warp * 8 + rr;
    T acc = T(0);
    if (offd && i < h)
      for (int k = lane; k < r; k += 32) acc += nd.U[(size_t)(i0 + i) * r + k] * s[k];
    acc = warp_sum(acc);
    if (lane == 0) gb[i] = (i < h) ? wn[i0 + i] - acc : T(0);
  }
  // 2. later row blocks: column block b of L below the diagonal, transposed
  T p0 = T(0), p1 = T(0);
  bool ok = true;
  for (int kb = nb - 1; kb > tk.b && ok; --kb) {
    ok = wait_ready(flags + kb, err);
    const int k0 = kb * SOLVE_RB, kh = min(SOLVE_RB, n - k0);
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      const int i = warp * 8 + rr;
      if (i < kh) {
        const T xi = __ldcg(wn + k0 + i);
        const T* p = nd.L + (size_t)(k0 + i) * nd.ld + i0 + 2 * lane;
        p0 += p[0] * xi;
        p1 += p[1] * xi;
      }
    }
  }
  red[warp][2 * lane] = p0;
  red[warp][2 * lane + 1] = p1;
  __syncthreads();
  if (threadIdx.x < SOLVE_RB) {
    T t = T(0);
#pragma unroll
    for (int q = 0; q < 8; ++q) t += red[q][threadIdx.x];
    vb[threadIdx.x] = gb[threadIdx.x] - t;
  }
  __syncthreads();
  // 3. x_b = Dinv_b^T v (rows of Dinv split over the warps)
  {
    const T* D = nd.Dinv + (size_t)tk.b * SOLVE_RB * SOLVE_RB;
    T q0 = T(0), q1 = T(0);
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      const int i = warp * 8 + rr;
      const T vi = vb[i];
      q0 += D[(size_t)i * SOLVE_RB + 2 * lane] * vi;
      q1 += D[(size_t)i * SOLVE_RB + 2 * lane + 1] * vi;
    }
    __syncthreads();
    red[warp][2 * lane] = q0;
    red[warp][2 * lane + 1] = q1;
    __syncthreads();
    if (threadIdx.x < h) {
      T t = T(0);
#pragma unroll
      for (int q = 0; q < 8; ++q) t += red[q][threadIdx.x];
      wn[i0 + threadIdx.x] = t;
    }
  }
  if (finish_row_block(flags + tk.b, flags + nb + 1, nb, &sync[levelSync], &sync[levelSync + 1], &sLast)) {
    for (int b = threadIdx.x; b < nb; b += blockDim.x) flags[b] = 0;
    if (threadIdx.x == 0) flags[nb + 1] = 0;
  }
}

// Inverse of each lower-triangular diagonal block (column c by thread c,
// forward substitution), zero-padded to 64 x 64.
template <class T>
__global__ void __launch_bounds__(64) invert_diag_blocks(const DinvTask<T>* __restrict__ tasks) {
  __shared__ T Ls[SOLVE_RB][SOLVE_RB + 1];
  const DinvTask<T> t = tasks[blockIdx.x];
  const int h = t.h, c = threadIdx.x;
  for (int idx = threadIdx.x; idx < h * h; idx += blockDim.x) {
    const int i = idx / h, j = idx - i * h;
    Ls[i][j] = (j <= i) ? t.L[(size_t)i * t.ld + j] : T(0);
  }
  T* D = t.D;
  for (int i = 0; i < SOLVE_RB; ++i) D[i * SOLVE_RB + c] = T(0);
  __syncthreads();
  if (c < h) {
    for (int i = c; i < h; ++i) {
      T s = (i == c) ? T(1) : T(0);
      for (int k = c; k < i; ++k) s -= Ls[i][k] * D[k * SOLVE_RB + c];
      D[i * SOLVE_RB + c] = s / Ls[i][i];
    }
  }
}

template <class A, class B>
__global__ void convert_kernel(const A* __restrict__ src, B* __restrict__ dst, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (B)src[i];
}

}  // namespace

template <class T>
SolveEngine<T>::SolveEngine(FactorEngine<T>& F) : F_(F) {}

template <class T>
void SolveEngine<T>::plan() {
  const Symbolic& S = F_.S;
  const int nn = (int)S.nodes.size();
  nodes_.assign(nn, SNode<T>{});
  std::vector<int> rowsAll, rel, child, lvlNodes;
  long long wuCur = 0, dinvCur = 0, zpCur = 0, spCur = 0;
  int syncCur = 1 + 4 * (int)F_.compressedLevels.size();   // error word, per-level tickets
  bytesPerApply_ = 0;
  std::vector<int> pos(S.n, -1);
  std::vector<DinvTask<T>> dinvTasks;
  std::vector<long long> dinvTaskOff, dinvNodeOff(nn, 0);
  for (int s = 0; s < nn; ++s) {
    const Node& nd = S.nodes[s];
    SNode<T>& sn = nodes_[s];
    sn.ld = F_.ld[s];
    sn.n = nd.n;
    sn.m = nd.m();
    sn.c0 = nd.c0;
    sn.rowsOff = (long long)rowsAll.size();
    rowsAll.insert(rowsAll.end(), nd.rows.begin(), nd.rows.end());
    if (!nd.compressed) {
      sn.L = F_.interior() + F_.frontOff[s];
      sn.r = 0;
      sn.wuOff = wuCur;
      wuCur += nd.m();
      bytesPerApply_ += 2.0 * sizeof(T) * (double)(nd.n * (nd.n + 1) / 2 + (double)nd.m() * nd.n);
    } else {
      sn.L = F_.compressed() + F_.frontOff[s];
      sn.r = F_.rank[s];
      sn.V = sn.r ? F_.vu() + F_.vOff[s] : nullptr;
      sn.U = sn.r ? F_.vu() + F_.uOff[s] : nullptr;
      sn.wuOff = wuCur;
      wuCur += 2LL * sn.r;
      sn.nb = (nd.n + SOLVE_RB - 1) / SOLVE_RB;
      sn.nch = (sn.r > 0 && sn.m > 0) ? (sn.m + 127) / 128 : 0;
      sn.syncOff = syncCur;
      syncCur += sn.nb + 3;
      sn.zpOff = zpCur;
      zpCur += (long long)sn.nb * sn.r;
      sn.spOff = spCur;
      spCur += (long long)sn.nch * sn.r;
      for (int b = 0; b < sn.nb; ++b) {
        DinvTask<T> t{};
        t.L = sn.L + (size_t)b * SOLVE_RB * sn.ld + (size_t)b * SOLVE_RB;
        t.ld = sn.ld;
        t.h = std::min(SOLVE_RB, nd.n - b * SOLVE_RB);
        dinvTasks.push_back(t);
        dinvTaskOff.push_back(dinvCur + (long long)b * SOLVE_RB * SOLVE_RB);
      }
      dinvNodeOff[s] = dinvCur;
      dinvCur += (long long)sn.nb * SOLVE_RB * SOLVE_RB;
      bytesPerApply_ += 2.0 * sizeof(T) * ((double)nd.n * (nd.n + 1) / 2 + (double)sn.r * (nd.m() + nd.n));
    }
  }
  // interior children and rel maps (target index of each row in the parent front)
  for (int s = 0; s < nn; ++s) {
    const Node& nd = S.nodes[s];
    if (nd.compressed) continue;
    nodes_[s].childBegin = (int)child.size();
    for (int c : S.children[s]) child.push_back(c);
    nodes_[s].childEnd = (int)child.size();
    for (int a = 0; a < nd.m(); ++a) pos[nd.rows[a]] = a;
    for (int c : S.children[s]) {
      const Node& cn = S.nodes[c];
      nodes_[c].relOff = (long long)rel.size();
      for (int a = 0; a < cn.m(); ++a) {
        int g = cn.rows[a];
        rel.push_back(g <= nd.c1 ? g - nd.c0 : nd.n + pos[g]);
      }
    }
    for (int a = 0; a < nd.m(); ++a) pos[nd.rows[a]] = -1;
  }
  // contribution sources of compressed supernodes: interior roots' update
  // vectors first, then compressed descendants' V z
  std::vector<std::vector<SPull>> pl(nn);
  for (int c = 0; c < nn; ++c) {
    const Node& cn = S.nodes[c];
    bool isRoot = !cn.compressed && (cn.parent < 0 || S.nodes[cn.parent].compressed);
    if (!cn.compressed && !isRoot) continue;
    for (size_t q = 0; q < cn.interNode.size(); ++q)
      pl[cn.interNode[q]].push_back(SPull{c, cn.interStart[q], cn.interStart[q + 1], cn.compressed ? 1 : 0});
  }
  for (int s = 0; s < nn; ++s)
    if (S.nodes[s].compressed)
      std::stable_sort(pl[s].begin(), pl[s].end(), [](const SPull& a, const SPull& b) { return a.kind < b.kind; });
  iLevels_.clear();
  cLevels_.clear();
  smemIF_.clear();
  smemIB_.clear();
  for (auto& lv : F_.interiorLevels) {
    iLevels_.push_back({(long long)lvlNodes.size(), (int)lv.size()});
    lvlNodes.insert(lvlNodes.end(), lv.begin(), lv.end());
    size_t f = 8, b = 8;
    for (int d : lv) {
      f = std::max(f, sizeof(T) * S.nodes[d].n);
      b = std::max(b, sizeof(T) * (2 * S.nodes[d].n + S.nodes[d].m()));
    }
    smemIF_.push_back(f);
    smemIB_.push_back(b);
  }
  for (size_t v : smemIB_)
    if (v > 200 * 1024) throw std::runtime_error("interior front too large for the shared-memory solve");
  // compressed levels: row-block tickets (forward: block 0 of every node, then
  // block 1, ...; backward: last blocks first), so that a thread block only
  // waits on blocks with smaller tickets
  std::vector<RowBlock> tickF, tickB;
  tickOff_.clear();
  cBlocks_.clear();
  cMaxCh_.clear();
  for (auto& lv : F_.compressedLevels) {
    cLevels_.push_back({(long long)lvlNodes.size(), (int)lv.size()});
    lvlNodes.insert(lvlNodes.end(), lv.begin(), lv.end());
    tickOff_.push_back((long long)tickF.size());
    int maxNb = 0, maxCh = 1, blocks = 0;
    for (int j : lv) {
      maxNb = std::max(maxNb, nodes_[j].nb);
      maxCh = std::max(maxCh, nodes_[j].nch);
      blocks += nodes_[j].nb;
    }
    for (int d = 0; d < maxNb; ++d)
      for (int j : lv)
        if (d < nodes_[j].nb) {
          tickF.push_back(RowBlock{j, d});
          tickB.push_back(RowBlock{j, nodes_[j].nb - 1 - d});
        }
    cBlocks_.push_back(blocks);
    cMaxCh_.push_back(maxCh);
  }
  cudaStream_t st = F_.stream;
  auto up = [&](DevBuf& b, const void* src, size_t bytes) {
    b.alloc(std::max<size_t>(bytes, 16));
    if (bytes) RSCHOL_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, st));
  };
  dWu_.alloc(sizeof(T) * std::max(1LL, wuCur));
  dDinv_.alloc(sizeof(T) * std::max(1LL, dinvCur));
  dZp_.alloc(sizeof(T) * std::max(1LL, zpCur));
  dSp_.alloc(sizeof(T) * std::max(1LL, spCur));
  for (size_t q = 0; q < dinvTasks.size(); ++q) dinvTasks[q].D = dDinv_.as<T>() + dinvTaskOff[q];
  for (int s = 0; s < nn; ++s)
    if (S.nodes[s].compressed) nodes_[s].Dinv = dDinv_.as<T>() + dinvNodeOff[s];
  nDinv_ = (int)dinvTasks.size();
  // per-row contribution lists of the compressed supernodes (in source order)
  {
    std::vector<long long> cstart;
    std::vector<CEntry<T>> ents;
    const T* wuBase = dWu_.as<T>();
    for (int s = 0; s < nn; ++s) {
      const Node& nd = S.nodes[s];
      if (!nd.compressed) continue;
      std::vector<int> cnt(nd.n + 1, 0);
      for (const SPull& P : pl[s])
        for (int a = P.a0; a < P.a1; ++a) cnt[S.nodes[P.src].rows[a] - nd.c0 + 1]++;
      for (int t = 0; t < nd.n; ++t) cnt[t + 1] += cnt[t];
      const long long base = (long long)ents.size();
      nodes_[s].cOff = (long long)cstart.size();
      for (int t = 0; t <= nd.n; ++t) cstart.push_back(base + cnt[t]);
      ents.resize(ents.size() + cnt[nd.n]);
      std::vector<int> fill(cnt.begin(), cnt.end() - 1);
      for (const SPull& P : pl[s]) {
        const SNode<T>& src = nodes_[P.src];
        for (int a = P.a0; a < P.a1; ++a) {
          CEntry<T> e{};
          if (P.kind == 0) {
            e.v = wuBase + src.wuOff + a;
            e.r = 0;
          } else {
            e.v = src.V + (size_t)a * src.r;
            e.z = wuBase + src.wuOff;
            e.r = src.r;
          }
          ents[base + fill[S.nodes[P.src].rows[a] - nd.c0]++] = e;
        }
      }
    }
    up(dCStart_, cstart.data(), cstart.size() * sizeof(long long));
    up(dCEnt_, ents.data(), ents.size() * sizeof(CEntry<T>));
  }
  up(dNodes_, nodes_.data(), nodes_.size() * sizeof(SNode<T>));
  up(dRows_, rowsAll.data(), rowsAll.size() * sizeof(int));
  up(dRel_, rel.data(), rel.size() * sizeof(int));
  up(dChild_, child.data(), child.size() * sizeof(int));
  up(dLevelNodes_, lvlNodes.data(), lvlNodes.size() * sizeof(int));
  up(dTickF_, tickF.data(), tickF.size() * sizeof(RowBlock));
  up(dTickB_, tickB.data(), tickB.size() * sizeof(RowBlock));
  up(dDinvTasks_, dinvTasks.data(), dinvTasks.size() * sizeof(DinvTask<T>));
  syncInts_ = syncCur;
  dSync_.alloc(sizeof(int) * syncCur);
  RSCHOL_CUDA(cudaMemsetAsync(dSync_.p, 0, sizeof(int) * syncCur, st));
  if (!std::is_same<T, double>::value) dW_.alloc(sizeof(T) * std::max(1, S.n));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  const int maxSmem = 200 * 1024;
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_backward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  launchesPerApply_ = 2 * (long long)iLevels_.size() + 3 * (long long)cLevels_.size() +
                      (std::is_same<T, double>::value ? 0 : 2);
  bytesPerApply_ += 8.0 * 4 * S.n;
}

template <class T>
int SolveEngine<T>::prepare(cudaStream_t st) {
  if (nDinv_ == 0) return 0;
  invert_diag_blocks<T><<<nDinv_, SOLVE_RB, 0, st>>>(dDinvTasks_.as<DinvTask<T>>());
  RSCHOL_LAUNCH_CHECK();
  return 1;
}

template <class T>
int SolveEngine<T>::take_error(cudaStream_t st) {
  int e = 0;
  if (!dSync_.p) return 0;
  RSCHOL_CUDA(cudaMemcpyAsync(&e, dSync_.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  if (e) {
    // a wait gave up: counters and flags are in an unknown state
    RSCHOL_CUDA(cudaMemsetAsync(dSync_.p, 0, sizeof(int) * syncInts_, st));
    RSCHOL_CUDA(cudaStreamSynchronize(st));
  }
  return e;
}

template <class T>
void SolveEngine<T>::apply_inplace(double* w64, cudaStream_t st) {
  // FP32 factors are applied in FP32 (the PCG recurrences stay FP64)
  T* w = std::is_same<T, double>::value ? reinterpret_cast<T*>(w64) : dW_.as<T>();
  const int n = F_.S.n;
  if (!std::is_same<T, double>::value) {
    convert_kernel<double, T><<<(n + 255) / 256, 256, 0, st>>>(w64, w, n);
    RSCHOL_LAUNCH_CHECK();
  }
  const int* lvl = dLevelNodes_.as<int>();
  int* sync = dSync_.as<int>();
  for (size_t l = 0; l < iLevels_.size(); ++l) {
    interior_forward_kernel<T><<<iLevels_[l].second, 256, smemIF_[l], st>>>(
        dNodes_.as<SNode<T>>(), lvl + iLevels_[l].first, dRows_.as<int>(), dRel_.as<int>(), dChild_.as<int>(), w,
        dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  for (size_t l = 0; l < cLevels_.size(); ++l) {
    compressed_forward_blocks<T><<<cBlocks_[l], 256, 0, st>>>(
        dNodes_.as<SNode<T>>(), dTickF_.as<RowBlock>() + tickOff_[l], dCStart_.as<long long>(),
        dCEnt_.as<CEntry<T>>(), sync, 1 + 4 * (int)l, dZp_.as<T>(), w, dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  for (int l = (int)cLevels_.size() - 1; l >= 0; --l) {
    compressed_vtx_kernel<T><<<dim3(cMaxCh_[l], cLevels_[l].second), 256, 0, st>>>(
        dNodes_.as<SNode<T>>(), lvl + cLevels_[l].first, dRows_.as<int>(), sync, dSp_.as<T>(), w, dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    compressed_backward_blocks<T><<<cBlocks_[l], 256, 0, st>>>(
        dNodes_.as<SNode<T>>(), dTickB_.as<RowBlock>() + tickOff_[l], sync, 1 + 4 * l + 2, dWu_.as<T>(), w);
    RSCHOL_LAUNCH_CHECK();
  }
  for (int l = (int)iLevels_.size() - 1; l >= 0; --l) {
    interior_backward_kernel<T><<<iLevels_[l].second, 256, smemIB_[l], st>>>(
        dNodes_.as<SNode<T>>(), lvl + iLevels_[l].first, dRows_.as<int>(), w);
    RSCHOL_LAUNCH_CHECK();
  }
  if (!std::is_same<T, double>::value) {
    convert_kernel<T, double><<<(n + 255) / 256, 256, 0, st>>>(w, w64, n);
    RSCHOL_LAUNCH_CHECK();
  }
}

template class SolveEngine<double>;
template class SolveEngine<float>;

}  // namespace rschol
