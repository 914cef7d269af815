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

// f := L^{-1} f with the inverted 64 x 64 diagonal blocks of L (block b:
// h_b x h_b row-major at D + 4096 b; only the last block can be smaller).
// f (n) and t (64) in shared memory.  A warp per row: loads coalesced along
// the row of L or D.
template <class T>
__device__ void trsv_dinv(const T* __restrict__ L, int ld, int n, const T* __restrict__ D, T* f, T* t) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int i0 = 0; i0 < n; i0 += 64) {
    const int h = min(64, n - i0);
    for (int i = warp; i < h; i += nwarp) {
      const T* row = L + (size_t)(i0 + i) * ld;
      T s = T(0);
      for (int j = lane; j < i0; j += 32) s += row[j] * f[j];
      s = warp_sum(s);
      if (lane == 0) t[i] = f[i0 + i] - s;
    }
    __syncthreads();
    const T* Db = D + (size_t)i0 * 64;
    for (int i = warp; i < h; i += nwarp) {
      const T* row = Db + (size_t)i * h;
      T s = T(0);
      for (int j = lane; j <= i; j += 32) s += row[j] * t[j];
      s = warp_sum(s);
      if (lane == 0) f[i0 + i] = s;
    }
    __syncthreads();
  }
}

// f := L^{-T} f with the same inverted diagonal blocks.  red: 4 x 64 shared.
template <class T>
__device__ void trsv_dinv_t(const T* __restrict__ L, int ld, int n, const T* __restrict__ D, T* f, T* t,
                            T (*red)[64]) {
  const int c = threadIdx.x & 63, grp = threadIdx.x >> 6, ngrp = blockDim.x >> 6;
  if (n <= 0) return;
  for (int i0 = ((n - 1) / 64) * 64; i0 >= 0; i0 -= 64) {
    const int h = min(64, n - i0);
    T s = T(0);
    if (c < h)
      for (int i = i0 + h + grp; i < n; i += ngrp) s += L[(size_t)i * ld + i0 + c] * f[i];
    red[grp][c] = s;
    __syncthreads();
    if (threadIdx.x < h) {
      T u = T(0);
      for (int g = 0; g < ngrp; ++g) u += red[g][threadIdx.x];
      t[threadIdx.x] = f[i0 + threadIdx.x] - u;
    }
    __syncthreads();
    if (threadIdx.x < h) {
      const T* Db = D + (size_t)i0 * 64;
      T x = T(0);
      for (int i = threadIdx.x; i < h; ++i) x += Db[(size_t)i * h + threadIdx.x] * t[i];
      f[i0 + threadIdx.x] = x;
    }
    __syncthreads();
  }
}

// Interior supernodes: one thread block per (supernode, 128-row chunk of its
// off-diagonal rows).  Every chunk block assembles and solves the supernode's
// own n columns (n is small); chunk 0 stores y.
constexpr int ICH = 128;

template <class T>
__global__ void __launch_bounds__(256) interior_forward_chunks(const SNode<T>* __restrict__ nodes,
                                                               const RowBlock* __restrict__ work,
                                                               const int* __restrict__ rel,
                                                               const int* __restrict__ child,
                                                               const T* __restrict__ w, T* __restrict__ yout,
                                                               T* __restrict__ wu) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* f = reinterpret_cast<T*>(smraw);
  __shared__ T tb[64];
  const RowBlock wk = work[blockIdx.x];
  const SNode<T>& nd = nodes[wk.node];
  const int n = nd.n, a0 = wk.b * ICH, a1 = min(nd.m, a0 + ICH);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* wud = wu + nd.wuOff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) f[i] = w[nd.c0 + i];
  for (int a = a0 + threadIdx.x; a < a1; a += blockDim.x) wud[a] = T(0);
  __syncthreads();
  // children's update vectors, in child order
  for (int c = nd.childBegin; c < nd.childEnd; ++c) {
    const SNode<T>& cn = nodes[child[c]];
    const T* wuc = wu + cn.wuOff;
    const int* rl = rel + cn.relOff;
    for (int a = threadIdx.x; a < cn.m; a += blockDim.x) {
      const int t = rl[a];
      if (t < n) f[t] += wuc[a];
      else if (t - n >= a0 && t - n < a1) wud[t - n] += wuc[a];
    }
    __syncthreads();
  }
  trsv_dinv<T>(nd.L, nd.ld, n, nd.Dinv, f, tb);
  // y goes to a separate vector: the other chunk blocks still read w
  if (wk.b == 0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) yout[nd.c0 + i] = f[i];
  // wud[a] -= L21[a] . y: a warp per 4 rows (loads coalesced along the rows)
  for (int a = a0 + warp * 4; a < a1; a += 32) {
    T s[4] = {T(0), T(0), T(0), T(0)};
    const T* row = nd.L + (size_t)(n + a) * nd.ld;
    for (int j = lane; j < n; j += 32) {
      const T fj = f[j];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (a + q < a1) s[q] += row[(size_t)q * nd.ld + j] * fj;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const T v = warp_sum(s[q]);
      if (lane == 0 && a + q < a1) wud[a + q] -= v;
    }
  }
}

// Backward: each chunk block forms its part of L21^T x_R; the last chunk
// block of the supernode to finish sums the parts in fixed order and solves
// with L11^T.
template <class T>
__global__ void __launch_bounds__(256) interior_backward_chunks(const SNode<T>* __restrict__ nodes,
                                                                const RowBlock* __restrict__ work,
                                                                const int* __restrict__ rows,
                                                                int* __restrict__ sync, T* __restrict__ ipart,
                                                                const T* __restrict__ yin, T* __restrict__ w) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ T tb[64];
  __shared__ T red[8][256];
  __shared__ int sLast;
  const RowBlock wk = work[blockIdx.x];
  const SNode<T>& nd = nodes[wk.node];
  const int n = nd.n, a0 = wk.b * ICH, a1 = min(nd.m, a0 + ICH);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* f = reinterpret_cast<T*>(smraw);   // n values
  T* xr = f + ((n + 1) & ~1);           // ICH values
  const int nch = (nd.m + ICH - 1) / ICH;
  if (nch > 0) {
    const int* rw = rows + nd.rowsOff;
    for (int a = a0 + threadIdx.x; a < a1; a += blockDim.x) xr[a - a0] = w[rw[a]];
    __syncthreads();
    // part[j] = sum_{a in chunk} L21[a][j] x_a: warp w takes rows w, w+8, ...
    // (lanes along the row), then the 8 warp partials are summed in order
    const T* L21 = nd.L + (size_t)(n + a0) * nd.ld;
    for (int jt = 0; jt < n; jt += 256) {
      T acc[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[q] = T(0);
      for (int a = warp; a < a1 - a0; a += 8) {
        const T x = xr[a];
        const T* row = L21 + (size_t)a * nd.ld + jt;
#pragma unroll
        for (int q = 0; q < 8; ++q)
          if (jt + lane + 32 * q < n) acc[q] += row[lane + 32 * q] * x;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) red[warp][lane + 32 * q] = acc[q];
      __syncthreads();
      const int j = jt + threadIdx.x;
      if (threadIdx.x < 256 && j < n) {
        T s = T(0);
#pragma unroll
        for (int q = 0; q < 8; ++q) s += red[q][threadIdx.x];
        ipart[nd.zpOff + (size_t)wk.b * n + j] = s;
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      __threadfence();
      sLast = (atomicAdd(sync + nd.syncOff, 1) == nch - 1);
      __threadfence();
    }
    __syncthreads();
    if (!sLast) return;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T t = T(0);
    for (int c = 0; c < nch; ++c) t += __ldcg(ipart + nd.zpOff + (size_t)c * n + i);
    f[i] = yin[nd.c0 + i] - t;
  }
  __syncthreads();
  trsv_dinv_t<T>(nd.L, nd.ld, n, nd.Dinv, f, tb, reinterpret_cast<T(*)[64]>(&red[0][0]));
  for (int i = threadIdx.x; i < n; i += blockDim.x) w[nd.c0 + i] = f[i];
  if (threadIdx.x == 0 && nch > 0) sync[nd.syncOff] = 0;
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
    if (flag) st_release(flag, 1);   // release: the block's stores, ordered by the barrier, become visible first
    __threadfence();
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

// t[rr][0..1] = P[row][2l], P[row][2l+1] of a 64-column tile (rows
// 8w+rr < h, zero elsewhere).
template <class T>
__device__ __forceinline__ void load_tile(const T* __restrict__ P, int ld, int h, T (&t)[8][2]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int rr = 0; rr < 8; ++rr) {
    const int i = warp * 8 + rr;
    if (i < h) {
      const T* p = P + (size_t)i * ld + 2 * lane;
      t[rr][0] = p[0];
      t[rr][1] = p[1];
    } else {
      t[rr][0] = T(0);
      t[rr][1] = T(0);
    }
  }
}

// Forward row block: f_b = w_b + contributions - sum_{k<b} L[b,k] y_k,
// y_b = Dinv_b f_b, partial z_b = U_b^T y_b.
template <class T>
__global__ void __launch_bounds__(256) compressed_forward_blocks(const SNode<T>* __restrict__ nodes,
                                                                 const RowBlock* __restrict__ tickets,
                                                                 const long long* __restrict__ cstart,
                                                                 const T* const* __restrict__ ent,
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
  // 1. right-hand side rows with their contribution lists (warp per row,
  // lanes over the row's contributions)
  const long long* cs = cstart + nd.cOff;
  for (int rr = 0; rr < 8; ++rr) {
    const int i = warp * 8 + rr;
    T acc = T(0);
    if (i < h)
      for (long long e = cs[i0 + i] + lane; e < cs[i0 + i + 1]; e += 32) acc += *ent[e];
    acc = warp_sum(acc);
    if (lane == 0) fb[i] = (i < h) ? wn[i0 + i] + acc : T(0);
  }
  // 2. earlier row blocks, as they become ready; the L tile of the next
  // block is loaded before waiting on the current one
  T acc[8], cur[8][2], dv[8][2];
#pragma unroll
  for (int rr = 0; rr < 8; ++rr) acc[rr] = T(0);
  load_tile<T>(nd.Dinv + (size_t)tk.b * SOLVE_RB * SOLVE_RB, SOLVE_RB, h, dv);
  const T* Lrow = nd.L + (size_t)i0 * nd.ld;
  if (tk.b > 0) load_tile<T>(Lrow, nd.ld, h, cur);
  bool ok = true;
  for (int kb = 0; kb < tk.b && ok; ++kb) {
    T nxt[8][2] = {};
    if (kb + 1 < tk.b) load_tile<T>(Lrow + (kb + 1) * SOLVE_RB, nd.ld, h, nxt);
    ok = wait_ready(flags + kb, err);
    const T y0 = __ldcg(wn + kb * SOLVE_RB + 2 * lane), y1 = __ldcg(wn + kb * SOLVE_RB + 2 * lane + 1);
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      acc[rr] += cur[rr][0] * y0 + cur[rr][1] * y1;
      cur[rr][0] = nxt[rr][0];
      cur[rr][1] = nxt[rr][1];
    }
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
    const T f0 = fb[2 * lane], f1 = fb[2 * lane + 1];
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) d[rr] = dv[rr][0] * f0 + dv[rr][1] * f1;
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
  // y_b is final: publish it before the (off the critical path) z partial
  if (threadIdx.x == 0) st_release(flags + tk.b, 1);
  // 4. partial z_b = U_b^T y_b
  const int r = nd.r;
  for (int k = threadIdx.x; k < r; k += blockDim.x) {
    T s = T(0);
    for (int i = 0; i < h; ++i) s += nd.U[(size_t)(i0 + i) * r + k] * yb[i];
    zpart[nd.zpOff + (size_t)tk.b * r + k] = s;
  }
  const int nb = nd.nb;
  if (finish_row_block(nullptr, flags + nb, nb, &sync[levelSync], &sync[levelSync + 1], &sLast)) {
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

// u = -V z of every compressed supernode of a level (its contribution to the
// right-hand sides of its ancestors), a warp per row.
template <class T>
__global__ void __launch_bounds__(256) compressed_vz_kernel(const SNode<T>* __restrict__ nodes,
                                                            const int* __restrict__ lvl, T* __restrict__ wu) {
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int r = nd.r;
  const T* z = wu + nd.wuOff;
  T* u = wu + nd.wuOff + 2 * r;
  for (int a = blockIdx.x * 8 + warp; a < nd.m; a += gridDim.x * 8) {
    const T* v = nd.V + (size_t)a * r;
    T s = T(0);
    for (int k = lane; k < r; k += 32) s += v[k] * z[k];
    s = warp_sum(s);
    if (lane == 0) u[a] = -s;
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
  // 2. later row blocks: column block b of L below the diagonal, transposed;
  // the tile of the next block is loaded before waiting on the current one
  T p0 = T(0), p1 = T(0), cur[8][2], dv[8][2];
  load_tile<T>(nd.Dinv + (size_t)tk.b * SOLVE_RB * SOLVE_RB, SOLVE_RB, SOLVE_RB, dv);
  const T* Lcol = nd.L + i0;
  if (nb - 1 > tk.b) {
    const int k0 = (nb - 1) * SOLVE_RB;
    load_tile<T>(Lcol + (size_t)k0 * nd.ld, nd.ld, min(SOLVE_RB, n - k0), cur);
  }
  bool ok = true;
  for (int kb = nb - 1; kb > tk.b && ok; --kb) {
    T nxt[8][2] = {};
    if (kb - 1 > tk.b) load_tile<T>(Lcol + (size_t)(kb - 1) * SOLVE_RB * nd.ld, nd.ld, SOLVE_RB, nxt);
    ok = wait_ready(flags + kb, err);
    const int k0 = kb * SOLVE_RB, kh = min(SOLVE_RB, n - k0);
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      const int i = warp * 8 + rr;
      const T xi = (i < kh) ? __ldcg(wn + k0 + i) : T(0);
      p0 += cur[rr][0] * xi;
      p1 += cur[rr][1] * xi;
      cur[rr][0] = nxt[rr][0];
      cur[rr][1] = nxt[rr][1];
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
    T q0 = T(0), q1 = T(0);
#pragma unroll
    for (int rr = 0; rr < 8; ++rr) {
      const T vi = vb[warp * 8 + rr];
      q0 += dv[rr][0] * vi;
      q1 += dv[rr][1] * vi;
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
// forward substitution), written as pad x pad (row-major, ld pad) with zeros
// outside the h x h lower triangle.
template <class T>
__global__ void __launch_bounds__(64) invert_diag_blocks(const DinvTask<T>* __restrict__ tasks) {
  __shared__ T Ls[SOLVE_RB][SOLVE_RB + 1];
  const DinvTask<T> t = tasks[blockIdx.x];
  const int h = t.h, pad = t.pad, c = threadIdx.x;
  for (int idx = threadIdx.x; idx < h * h; idx += blockDim.x) {
    const int i = idx / h, j = idx - i * h;
    Ls[i][j] = (j <= i) ? t.L[(size_t)i * t.ld + j] : T(0);
  }
  T* D = t.D;
  if (c < pad)
    for (int i = 0; i < pad; ++i) D[i * pad + c] = T(0);
  __syncthreads();
  if (c < h) {
    for (int i = c; i < h; ++i) {
      T s = (i == c) ? T(1) : T(0);
      for (int k = c; k < i; ++k) s -= Ls[i][k] * D[k * pad + c];
      D[i * pad + c] = s / Ls[i][i];
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
  long long wuCur = 0, dinvCur = 0, zpCur = 0, spCur = 0, ipCur = 0;
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
      sn.nch = (nd.m() + ICH - 1) / ICH;
      sn.syncOff = syncCur;
      syncCur += 1;
      sn.zpOff = ipCur;
      ipCur += (long long)sn.nch * nd.n;
      // inverted 64 x 64 diagonal blocks, the last one stored h x h
      const int nbI = (nd.n + SOLVE_RB - 1) / SOLVE_RB;
      for (int b = 0; b < nbI; ++b) {
        DinvTask<T> t{};
        t.L = sn.L + (size_t)b * SOLVE_RB * sn.ld + (size_t)b * SOLVE_RB;
        t.ld = sn.ld;
        t.h = std::min(SOLVE_RB, nd.n - b * SOLVE_RB);
        t.pad = t.h;
        dinvTasks.push_back(t);
        dinvTaskOff.push_back(dinvCur + (long long)b * SOLVE_RB * SOLVE_RB);
      }
      dinvNodeOff[s] = dinvCur;
      {
        const int hl = nd.n - (nbI - 1) * SOLVE_RB;
        dinvCur += (long long)(nbI - 1) * SOLVE_RB * SOLVE_RB + (long long)hl * hl;
      }
      bytesPerApply_ += 2.0 * sizeof(T) * (double)(nd.n * (nd.n + 1) / 2 + (double)nd.m() * nd.n);
    } else {
      sn.L = F_.compressed() + F_.frontOff[s];
      sn.r = F_.rank[s];
      sn.V = sn.r ? F_.vu() + F_.vOff[s] : nullptr;
      sn.U = sn.r ? F_.vu() + F_.uOff[s] : nullptr;
      sn.wuOff = wuCur;
      wuCur += 2LL * sn.r + sn.m;   // z | s | u = -V z
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
        t.pad = SOLVE_RB;
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
  std::vector<RowBlock> iwork;
  for (auto& lv : F_.interiorLevels) {
    iLevels_.push_back({(long long)iwork.size(), 0});
    size_t f = 8, b = 8;
    for (int d : lv) {
      for (int c = 0; c < std::max(1, nodes_[d].nch); ++c) iwork.push_back(RowBlock{d, c});
      f = std::max(f, sizeof(T) * S.nodes[d].n);
      b = std::max(b, sizeof(T) * (((S.nodes[d].n + 1) & ~1) + ICH));
    }
    iLevels_.back().second = (int)(iwork.size() - iLevels_.back().first);
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
  cVzGrid_.clear();
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
    int maxM = 1;
    for (int j : lv) maxM = std::max(maxM, nodes_[j].m);
    cVzGrid_.push_back(std::min(64, (maxM + 7) / 8));
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
  dIp_.alloc(sizeof(T) * std::max(1LL, ipCur));
  dYi_.alloc(sizeof(T) * std::max(1, S.n));
  for (size_t q = 0; q < dinvTasks.size(); ++q) dinvTasks[q].D = dDinv_.as<T>() + dinvTaskOff[q];
  for (int s = 0; s < nn; ++s) nodes_[s].Dinv = dDinv_.as<T>() + dinvNodeOff[s];
  nDinv_ = (int)dinvTasks.size();
  // per-row contribution lists of the compressed supernodes (in source order)
  {
    std::vector<long long> cstart;
    std::vector<const T*> ents;
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
          // interior root: its update vector; compressed: u = -V z
          const T* e = (P.kind == 0) ? wuBase + src.wuOff + a : wuBase + src.wuOff + 2 * src.r + a;
          ents[base + fill[S.nodes[P.src].rows[a] - nd.c0]++] = e;
        }
      }
    }
    up(dCStart_, cstart.data(), cstart.size() * sizeof(long long));
    up(dCEnt_, ents.data(), ents.size() * sizeof(const T*));
  }
  up(dNodes_, nodes_.data(), nodes_.size() * sizeof(SNode<T>));
  up(dRows_, rowsAll.data(), rowsAll.size() * sizeof(int));
  up(dRel_, rel.data(), rel.size() * sizeof(int));
  up(dChild_, child.data(), child.size() * sizeof(int));
  up(dLevelNodes_, lvlNodes.data(), lvlNodes.size() * sizeof(int));
  up(dIWork_, iwork.data(), iwork.size() * sizeof(RowBlock));
  up(dTickF_, tickF.data(), tickF.size() * sizeof(RowBlock));
  up(dTickB_, tickB.data(), tickB.size() * sizeof(RowBlock));
  up(dDinvTasks_, dinvTasks.data(), dinvTasks.size() * sizeof(DinvTask<T>));
  syncInts_ = syncCur;
  dSync_.alloc(sizeof(int) * syncCur);
  RSCHOL_CUDA(cudaMemsetAsync(dSync_.p, 0, sizeof(int) * syncCur, st));
  if (!std::is_same<T, double>::value) dW_.alloc(sizeof(T) * std::max(1, S.n));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  const int maxSmem = 200 * 1024;
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_forward_chunks<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_backward_chunks<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  launchesPerApply_ = 2 * (long long)iLevels_.size() + 4 * (long long)cLevels_.size() - (cLevels_.empty() ? 0 : 1) +
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
  const RowBlock* iwork = dIWork_.as<RowBlock>();
  for (size_t l = 0; l < iLevels_.size(); ++l) {
    interior_forward_chunks<T><<<iLevels_[l].second, 256, smemIF_[l], st>>>(
        dNodes_.as<SNode<T>>(), iwork + iLevels_[l].first, dRel_.as<int>(), dChild_.as<int>(), w, dYi_.as<T>(),
        dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  for (size_t l = 0; l < cLevels_.size(); ++l) {
    compressed_forward_blocks<T><<<cBlocks_[l], 256, 0, st>>>(
        dNodes_.as<SNode<T>>(), dTickF_.as<RowBlock>() + tickOff_[l], dCStart_.as<long long>(),
        dCEnt_.as<const T*>(), sync, 1 + 4 * (int)l, dZp_.as<T>(), w, dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    if (l + 1 < cLevels_.size()) {   // the top level's u feeds no one
      compressed_vz_kernel<T><<<dim3(cVzGrid_[l], cLevels_[l].second), 256, 0, st>>>(
          dNodes_.as<SNode<T>>(), lvl + cLevels_[l].first, dWu_.as<T>());
      RSCHOL_LAUNCH_CHECK();
    }
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
    interior_backward_chunks<T><<<iLevels_[l].second, 256, smemIB_[l], st>>>(
        dNodes_.as<SNode<T>>(), iwork + iLevels_[l].first, dRows_.as<int>(), sync, dIp_.as<T>(), dYi_.as<T>(), w);
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
