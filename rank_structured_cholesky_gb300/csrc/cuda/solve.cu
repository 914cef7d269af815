#include <algorithm>
#include <mutex>
#include <cstdlib>
#include <type_traits>

#include "solve.cuh"
#include "solve_dev.cuh"

namespace rschol {

namespace {

using namespace solvedev;

// out[k] = sum_{i < rows} M[i][k] v[i] (v == nullptr: v[i] = 1, and M was
// written by other blocks of this launch, so its loads bypass L1) for k < r,
// M row-major with leading dimension ld.  Eight warps split the rows, lanes
// run along k (coalesced), and the eight warp partials are added in a fixed
// order.  blockDim.x == 256; red: 8 x 256 shared; every thread must call it.
template <class T>
__device__ void rows_t_gemv(const T* __restrict__ M, int ld, int rows, int r, const T* v, T* out, T (*red)[256]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k0 = 0; k0 < r; k0 += 256) {
    T acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = T(0);
    for (int i = warp; i < rows; i += 8) {
      const T vi = v ? v[i] : T(1);
      const T* row = M + (size_t)i * ld + k0;
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (k0 + lane + 32 * c < r) acc[c] += (v ? row[lane + 32 * c] : __ldcg(row + lane + 32 * c)) * vi;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) red[warp][lane + 32 * c] = acc[c];
    __syncthreads();
    if (k0 + (int)threadIdx.x < r) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < 8; ++q) s += red[q][threadIdx.x];
      out[k0 + threadIdx.x] = s;
    }
    __syncthreads();
  }
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

// Small interior supernodes (n <= IW_N, m <= ICH: one chunk) take a warp
// each, eight to a block, so the thousands of bottom-level supernodes do not
// each pay a block's scheduling, ticket and barrier latencies.  (Widening
// this to n <= 64, m <= 320 -- a warp per supernode of the next two levels --
// measured slower on c2: 1.15 vs 0.92 ms per apply; to m <= 192, the same.)  The steps and
// the waits are those of a chunk block below; the per-warp shared buffers
// hold f (IW_N) and the update vector (ICH).
constexpr int IW_N = 32;

template <class T>
__device__ void interior_forward_warp(const SNode<T>* __restrict__ nodes, int s, const int* __restrict__ rel,
                                      const int* __restrict__ child, int* sync, int epoch, const T* w, T* yout, T* wu,
                                      T* f, T* u) {
  const int lane = threadIdx.x & 31;
  int* err = sync;
  const SNode<T>& nd = nodes[s];
  const int n = nd.n, m = nd.m;
  for (int c = nd.childBegin; c < nd.childEnd; ++c) {   // every child has stored its update vector
    const SNode<T>& cn = nodes[child[c]];
    if (!wait_geq(sync + cn.syncOff + 1, epoch * max(1, cn.nch), err)) break;
  }
  if (lane < n) f[lane] = w[nd.c0 + lane];
  for (int a = lane; a < m; a += 32) u[a] = T(0);
  __syncwarp();
  for (int c = nd.childBegin; c < nd.childEnd; ++c) {   // children's update vectors, in child order
    const SNode<T>& cn = nodes[child[c]];
    const T* wuc = wu + cn.wuOff;
    const int* rl = rel + cn.relOff;
    for (int a = lane; a < cn.m; a += 32) {
      const int t = rl[a];
      const T v = __ldcg(wuc + a);
      if (t < n) f[t] += v;
      else u[t - n] += v;
    }
    __syncwarp();
  }
  // y = L11^{-1} f through the inverted diagonal block (n x n, row-major)
  T y = T(0);
  if (lane < n)
    for (int j = 0; j <= lane; ++j) y += nd.Dinv[lane * n + j] * f[j];
  __syncwarp();
  if (lane < n) {
    f[lane] = y;
    yout[nd.c0 + lane] = y;
  }
  __syncwarp();
  T* wud = wu + nd.wuOff;
  for (int a = lane; a < m; a += 32) {   // u_a -= L21[a] . y
    const T* row = nd.L + (size_t)(n + a) * nd.ld;
    T acc = T(0);
    for (int j = 0; j < n; ++j) acc += row[j] * f[j];
    wud[a] = u[a] - acc;
  }
  __syncwarp();
  if (lane == 0) {
    __threadfence();
    atomicAdd(sync + nd.syncOff + 1, 1);
  }
}

template <class T>
__device__ void interior_backward_warp(const SNode<T>* __restrict__ nodes, int s, const int* __restrict__ rows,
                                       int* sync, int epoch, const T* yin, T* w, T* f, T* xr) {
  const int lane = threadIdx.x & 31;
  int* err = sync;
  const SNode<T>& nd = nodes[s];
  const int n = nd.n, m = nd.m;
  if (nd.parentI >= 0) wait_geq(sync + nodes[nd.parentI].syncOff + 2, epoch, err);   // ancestors solved
  const int* rw = rows + nd.rowsOff;
  for (int a = lane; a < m; a += 32) xr[a] = __ldcg(w + rw[a]);
  __syncwarp();
  T t = T(0);   // f_j = y_j - (L21^T x_R)_j, lanes over the columns
  if (lane < n) {
    for (int a = 0; a < m; ++a) t += nd.L[(size_t)(n + a) * nd.ld + lane] * xr[a];
    f[lane] = yin[nd.c0 + lane] - t;
  }
  __syncwarp();
  T x = T(0);   // x = L11^{-T} f: x_i = sum_{k >= i} D_ki f_k
  if (lane < n) {
    for (int k = lane; k < n; ++k) x += nd.Dinv[k * n + lane] * f[k];
    w[nd.c0 + lane] = x;
  }
  __syncwarp();
  if (lane == 0) {
    __threadfence();
    st_release(sync + nd.syncOff + 2, epoch);   // x of this supernode is final
  }
}

// Interior supernodes: all levels in one launch per direction.  A block takes
// the next (supernode, 128-row chunk of its off-diagonal rows) from a ticket
// counter, in level order, so it only waits on blocks that started before it:
// forward, on the chunk blocks of the supernode's children (per-supernode
// completion counters that grow by one per chunk); backward, on the solve of
// its interior parent (a flag set to 1).  The apply's last kernel clears the
// counters (clear_piece), so every apply starts from zeros with no host
// state and the same launches replay unchanged inside a CUDA graph.  Every
// chunk block assembles and solves the supernode's own n columns (n is
// small); chunk 0 stores y.

template <class T>
__global__ void __launch_bounds__(256) interior_forward_chunks(const SNode<T>* __restrict__ nodes,
                                                               const RowBlock* __restrict__ work,
                                                               const int* __restrict__ rel,
                                                               const int* __restrict__ child,
                                                               int* __restrict__ sync, int epoch,
                                                               const T* __restrict__ w, T* __restrict__ yout,
                                                               T* __restrict__ wu, const int* __restrict__ small) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smraw[];
  T* f = reinterpret_cast<T*>(smraw);
  __shared__ T tb[64];
  __shared__ int sTicket;
  int* err = sync;
  if (threadIdx.x == 0) sTicket = atomicAdd(&sync[SYNC_TICK_F], 1);
  __syncthreads();
  if (sTicket >= (int)gridDim.x) {   // counters not reset: report, touch nothing
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const RowBlock wk = work[sTicket];
  if (wk.node < 0) {   // a group of small supernodes (node = -1 - group, b = count), a warp each
    const int warp = threadIdx.x >> 5;
    if (warp < wk.b)
      interior_forward_warp<T>(nodes, small[8 * (-1 - wk.node) + warp], rel, child, sync, epoch, w, yout, wu,
                               f + warp * (IW_N + ICH), f + warp * (IW_N + ICH) + IW_N);
    launch_done(&sync[SYNC_TICK_F], &sync[SYNC_DONE_F]);
    return;
  }
  const SNode<T>& nd = nodes[wk.node];
  const int n = nd.n, a0 = wk.b * ICH, a1 = min(nd.m, a0 + ICH);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* wud = wu + nd.wuOff;
  if (warp == 0)   // every chunk block of every child has stored its update rows
    for (int c = nd.childBegin; c < nd.childEnd; ++c) {
      const SNode<T>& cn = nodes[child[c]];
      if (!wait_geq(sync + cn.syncOff + 1, epoch * max(1, cn.nch), err)) break;
    }
  __syncthreads();
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
      if (t < n) f[t] += __ldcg(wuc + a);
      else if (t - n >= a0 && t - n < a1) wud[t - n] += __ldcg(wuc + a);
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
  __syncthreads();
  if (threadIdx.x == 0) {   // this chunk's rows of the update vector are final
    __threadfence();
    atomicAdd(sync + nd.syncOff + 1, 1);
  }
  launch_done(&sync[SYNC_TICK_F], &sync[SYNC_DONE_F]);
}

// Backward: each chunk block forms its part of L21^T x_R; the last chunk
// block of the supernode to finish sums the parts in fixed order and solves
// with L11^T.
template <class T>
__global__ void __launch_bounds__(256) interior_backward_chunks(const SNode<T>* __restrict__ nodes,
                                                                const RowBlock* __restrict__ work,
                                                                const int* __restrict__ rows,
                                                                int* __restrict__ sync, int epoch,
                                                                T* __restrict__ ipart, const T* __restrict__ yin,
                                                                T* __restrict__ w, const int* __restrict__ small) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ T tb[64];
  __shared__ T red[8][256];
  __shared__ int sLast, sTicket;
  int* err = sync;
  if (threadIdx.x == 0) sTicket = atomicAdd(&sync[SYNC_TICK_B], 1);
  __syncthreads();
  if (sTicket >= (int)gridDim.x) {   // counters not reset: report, touch nothing
    if (threadIdx.x == 0) atomicExch(err, 2);
    return;
  }
  const RowBlock wk = work[sTicket];
  if (wk.node < 0) {   // a group of small supernodes, a warp each
    const int warp = threadIdx.x >> 5;
    T* fw = reinterpret_cast<T*>(smraw) + warp * (IW_N + ICH);
    if (warp < wk.b)
      interior_backward_warp<T>(nodes, small[8 * (-1 - wk.node) + warp], rows, sync, epoch, yin, w, fw, fw + IW_N);
    launch_done(&sync[SYNC_TICK_B], &sync[SYNC_DONE_B]);
    return;
  }
  const SNode<T>& nd = nodes[wk.node];
  if (nd.parentI >= 0 && (threadIdx.x >> 5) == 0)   // the parent (and so every ancestor) is solved
    wait_geq(sync + nodes[nd.parentI].syncOff + 2, epoch, err);
  __syncthreads();
  const int n = nd.n, a0 = wk.b * ICH, a1 = min(nd.m, a0 + ICH);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T* f = reinterpret_cast<T*>(smraw);   // n values
  T* xr = f + ((n + 1) & ~1);           // ICH values
  const int nch = (nd.m + ICH - 1) / ICH;
  if (nch > 0) {
    const int* rw = rows + nd.rowsOff;
    for (int a = a0 + threadIdx.x; a < a1; a += blockDim.x) xr[a - a0] = __ldcg(w + rw[a]);
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
    if (!sLast) {
      launch_done(&sync[SYNC_TICK_B], &sync[SYNC_DONE_B]);
      return;
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    T t = T(0);
    for (int c = 0; c < nch; ++c) t += __ldcg(ipart + nd.zpOff + (size_t)c * n + i);
    f[i] = yin[nd.c0 + i] - t;
  }
  __syncthreads();
  trsv_dinv_t<T>(nd.L, nd.ld, n, nd.Dinv, f, tb, reinterpret_cast<T(*)[64]>(&red[0][0]));
  for (int i = threadIdx.x; i < n; i += blockDim.x) w[nd.c0 + i] = f[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    if (nch > 0) sync[nd.syncOff] = 0;
    st_release(sync + nd.syncOff + 2, epoch);   // x of this supernode is final
  }
  launch_done(&sync[SYNC_TICK_B], &sync[SYNC_DONE_B]);
}

// ---------------------------------------------------------------------------
// Compressed supernodes.  X = L11^{-1} is formed once per factorisation, so
// the triangular solves are GEMVs: every 64-row (or 64-column) block of a
// supernode is an independent thread block.

// The pieces of a compressed level, as device functions of one thread block
// (a warp per row where rows are independent).  Data another block wrote is
// read through L2 (ld.global.cg).

// w[c0 + i] += the fixed-order contribution list of row i (one warp).
template <class T>
__device__ void cgather_row(const SNode<T>& nd, int i, const long long* __restrict__ cstart,
                            const long long* __restrict__ ent, const T* wu, T* w) {
  const int lane = threadIdx.x & 31;
  const long long* cs = cstart + nd.cOff;
  T acc = T(0);
  for (long long e = cs[i] + lane; e < cs[i + 1]; e += 32) acc += __ldcg(wu + ent[e]);
  acc = warp_sum(acc);
  if (lane == 0) w[nd.c0 + i] = __ldcg(w + nd.c0 + i) + acc;
}

// Partial products of y = X f and x = X^T g over 64 x 256 tiles of X (tiles
// entirely above the diagonal are not listed): a level's tiles are spread
// over all SMs, each thread keeping 64 independent loads in flight.
//   P[i][jb] = sum_{j in column block jb} X[i][j] f_j    (forward)
//   Q[j][ib] = sum_{i in row block ib} X[i][j] g_i       (backward)
template <class T>
__device__ void cytile(const SNode<T>& nd, const XTile& tl, const T* w, T* part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n = nd.n;
  const int i0 = tl.ib * SOLVE_RB + warp * 8, j0 = tl.jb * XT_COLS;
  T fj[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int j = j0 + lane + 32 * c;
    fj[c] = (j < n) ? __ldcg(w + nd.c0 + j) : T(0);
  }
  T acc[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    acc[q] = T(0);
    const int i = i0 + q;
    if (i < n) {
      const T* xr = nd.X + (size_t)i * n;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int j = j0 + lane + 32 * c;
        if (j < n) acc[q] += xr[j] * fj[c];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const T v = warp_sum(acc[q]);
    if (lane == 0 && i0 + q < n) part[nd.zpOff2 + (size_t)(i0 + q) * nd.ncb + tl.jb] = v;
  }
}

// gs: SOLVE_RB shared.
template <class T>
__device__ void cxtile(const SNode<T>& nd, const XTile& tl, const T* gv, T* part, T* gs) {
  const int n = nd.n, i0 = tl.ib * SOLVE_RB, h = min(SOLVE_RB, n - i0);
  if (threadIdx.x < SOLVE_RB) gs[threadIdx.x] = (threadIdx.x < h) ? __ldcg(gv + nd.c0 + i0 + threadIdx.x) : T(0);
  __syncthreads();
  const int j = tl.jb * XT_COLS + threadIdx.x;
  if (j < n) {
    T s = T(0);
#pragma unroll 16
    for (int i = 0; i < h; ++i) s += nd.X[(size_t)(i0 + i) * n + j] * gs[i];
    part[nd.zpOff2 + (size_t)j * nd.nb + tl.ib] = s;
  }
  __syncthreads();
}

// y_i = sum of its tile partials (fixed order) for one 64-row block, then the
// block's part of z = U^T y; the last block of the supernode to finish sums
// the parts in fixed order.  yb: SOLVE_RB shared, red: 8 x 256 shared.
template <class T>
__device__ void cy_block(const SNode<T>& nd, int b, int* sync, T* zpart, const T* ypart, T* yv, T* wu, T* yb,
                         T (*red)[256], int* sLast) {
  const int n = nd.n, i0 = b * SOLVE_RB, h = min(SOLVE_RB, n - i0);
  if (threadIdx.x < SOLVE_RB) {
    const int i = threadIdx.x;
    T s = T(0);
    if (i < h) {
      const int jbEnd = min(nd.ncb - 1, (i0 + SOLVE_RB - 1) / XT_COLS);
      const T* p = ypart + nd.zpOff2 + (size_t)(i0 + i) * nd.ncb;
      for (int jb = 0; jb <= jbEnd; ++jb) s += __ldcg(p + jb);
      yv[nd.c0 + i0 + i] = s;
    }
    yb[i] = s;
  }
  __syncthreads();
  const int r = nd.r;
  rows_t_gemv<T>(nd.U + (size_t)i0 * r, r, h, r, yb, zpart + nd.zpOff + (size_t)b * r, red);
  int* done = sync + nd.syncOff;
  if (threadIdx.x == 0) {
    __threadfence();
    *sLast = (atomicAdd(done, 1) == nd.nb - 1);
    __threadfence();
  }
  __syncthreads();
  if (!*sLast) return;
  rows_t_gemv<T>(zpart + nd.zpOff, r, nd.nb, r, nullptr, wu + nd.wuOff, red);
  if (threadIdx.x == 0) *done = 0;
  __syncthreads();
}

// x_j = sum of its tile partials over the row blocks ib >= 4 jb (fixed order).
template <class T>
__device__ void cx_reduce_col(const SNode<T>& nd, int j, const T* xpart, T* w) {
  const T* p = xpart + nd.zpOff2 + (size_t)j * nd.nb;
  T s = T(0);
  for (int ib = (j / XT_COLS) * (XT_COLS / SOLVE_RB); ib < nd.nb; ++ib) s += __ldcg(p + ib);
  w[nd.c0 + j] = s;
}

// u_a = -(V z)_a, the supernode's contribution to its ancestors' right-hand
// sides (one warp).
template <class T>
__device__ void cvz_row(const SNode<T>& nd, int a, T* wu) {
  const int lane = threadIdx.x & 31, r = nd.r;
  const T* z = wu + nd.wuOff;
  const T* v = nd.V + (size_t)a * r;
  T s = T(0);
  for (int k = lane; k < r; k += 32) s += v[k] * __ldcg(z + k);
  s = warp_sum(s);
  if (lane == 0) wu[nd.wuOff + 2 * r + a] = -s;
}

// s = V^T x_R for one 128-row chunk; the last chunk to finish sums the chunk
// partials in fixed order.  xs: 128 shared, red: 8 x 256 shared.
template <class T>
__device__ void cvtx_chunk(const SNode<T>& nd, int ch, const int* __restrict__ rows, int* sync, T* spart,
                           const T* w, T* sv, T* xs, T (*red)[256], int* sLast) {
  const int r = nd.r, a0 = ch * 128, ah = min(128, nd.m - a0);
  const int* rw = rows + nd.rowsOff + a0;
  for (int a = threadIdx.x; a < ah; a += blockDim.x) xs[a] = __ldcg(w + rw[a]);
  __syncthreads();
  rows_t_gemv<T>(nd.V + (size_t)a0 * r, r, ah, r, xs, spart + nd.spOff + (size_t)ch * r, red);
  int* done = sync + nd.syncOff + 1;
  if (threadIdx.x == 0) {
    __threadfence();
    *sLast = (atomicAdd(done, 1) == nd.nch - 1);
    __threadfence();
  }
  __syncthreads();
  if (!*sLast) return;
  rows_t_gemv<T>(spart + nd.spOff, r, nd.nch, r, nullptr, sv + nd.wuOff + r, red);
  if (threadIdx.x == 0) *done = 0;
  __syncthreads();
}

// g_i = y_i - (U s)_i in place (one warp).
template <class T>
__device__ void cg_row(const SNode<T>& nd, int i, const T* sv, T* yv) {
  const int lane = threadIdx.x & 31, r = nd.r;
  const T* s = sv + nd.wuOff + r;
  const T* u = nd.U + (size_t)i * r;
  T acc = T(0);
  for (int k = lane; k < r; k += 32) acc += u[k] * __ldcg(s + k);
  acc = warp_sum(acc);
  if (lane == 0) yv[nd.c0 + i] = __ldcg(yv + nd.c0 + i) - acc;
}

// One launch per piece and level, chained by programmatic dependent launch.
// (All levels of a direction as one ticketed launch, with each phase waiting
// on the previous one through counters, measured slower on c2: 1.19 vs 1.07
// ms per apply -- the dependent launches already start without gaps; running
// the y and x reductions at the tail of the tile launches, by the last tile
// of each block, measured the same: 0.936 vs 0.919 ms.)
template <class T>
__global__ void __launch_bounds__(256) compressed_gather_rows(const SNode<T>* __restrict__ nodes,
                                                              const int* __restrict__ lvl,
                                                              const long long* __restrict__ cstart,
                                                              const long long* __restrict__ ent,
                                                              const T* __restrict__ wu, T* __restrict__ w) {
  pdl_enter();
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i < nd.n) cgather_row<T>(nd, i, cstart, ent, wu, w);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_ytile_kernel(const SNode<T>* __restrict__ nodes,
                                                               const XTile* __restrict__ tiles,
                                                               const T* __restrict__ w, T* __restrict__ part) {
  pdl_enter();
  const XTile tl = tiles[blockIdx.x];
  cytile<T>(nodes[tl.node], tl, w, part);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_xtile_kernel(const SNode<T>* __restrict__ nodes,
                                                               const XTile* __restrict__ tiles,
                                                               const T* __restrict__ gv, T* __restrict__ part) {
  pdl_enter();
  __shared__ T gs[SOLVE_RB];
  const XTile tl = tiles[blockIdx.x];
  cxtile<T>(nodes[tl.node], tl, gv, part, gs);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_y_kernel(const SNode<T>* __restrict__ nodes,
                                                           const RowBlock* __restrict__ work, int* __restrict__ sync,
                                                           T* __restrict__ zpart, const T* __restrict__ ypart,
                                                           T* __restrict__ yv, T* __restrict__ wu) {
  pdl_enter();
  __shared__ T yb[SOLVE_RB];
  __shared__ T red[8][256];
  __shared__ int sLast;
  const RowBlock wk = work[blockIdx.x];
  cy_block<T>(nodes[wk.node], wk.b, sync, zpart, ypart, yv, wu, yb, red, &sLast);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_x_reduce(const SNode<T>* __restrict__ nodes,
                                                           const int* __restrict__ lvl, const T* __restrict__ xpart,
                                                           T* __restrict__ w) {
  pdl_enter();
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nd.n) cx_reduce_col<T>(nd, j, xpart, w);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_vz_kernel(const SNode<T>* __restrict__ nodes,
                                                            const int* __restrict__ lvl, T* __restrict__ wu) {
  pdl_enter();
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  for (int a = blockIdx.x * 8 + (threadIdx.x >> 5); a < nd.m; a += gridDim.x * 8) cvz_row<T>(nd, a, wu);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_vtx_kernel(const SNode<T>* __restrict__ nodes,
                                                             const int* __restrict__ lvl,
                                                             const int* __restrict__ rows,
                                                             int* __restrict__ sync, T* __restrict__ spart,
                                                             const T* __restrict__ w, T* __restrict__ sv) {
  pdl_enter();
  __shared__ T xs[128];
  __shared__ T red[8][256];
  __shared__ int sLast;
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  if (blockIdx.x < nd.nch) cvtx_chunk<T>(nd, blockIdx.x, rows, sync, spart, w, sv, xs, red, &sLast);
}

template <class T>
__global__ void __launch_bounds__(256) compressed_g_kernel(const SNode<T>* __restrict__ nodes,
                                                           const int* __restrict__ lvl, const T* __restrict__ sv,
                                                           T* __restrict__ yv) {
  pdl_enter();
  const SNode<T>& nd = nodes[lvl[blockIdx.y]];
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i < nd.n && nd.r > 0 && nd.m > 0) cg_row<T>(nd, i, sv, yv);
}

// Inverse of each lower-triangular diagonal block (column c by thread c,
// forward substitution), written as pad x pad (row-major, row stride ldD)
// with zeros outside the h x h lower triangle.  The columns are formed in
// shared memory (Xs[i][c], conflict-free across threads) and stored once, in
// rows: the substitution's reads of earlier entries never go to global memory
// (writing and re-reading D instead: c2 factorisation 21.64 vs 21.52 ms).
// Dynamic shared memory: two SOLVE_RB x (SOLVE_RB + 1) tiles of T.
template <class T>
__global__ void __launch_bounds__(64) invert_diag_blocks(const DinvTask<T>* __restrict__ tasks) {
  extern __shared__ __align__(16) unsigned char idb_smem[];
  T (*Ls)[SOLVE_RB + 1] = reinterpret_cast<T (*)[SOLVE_RB + 1]>(idb_smem);
  T (*Xs)[SOLVE_RB + 1] = reinterpret_cast<T (*)[SOLVE_RB + 1]>(idb_smem + sizeof(T) * SOLVE_RB * (SOLVE_RB + 1));
  const DinvTask<T> t = tasks[blockIdx.x];
  const int h = t.h, pad = t.pad, ldD = t.ldD, c = threadIdx.x;
  for (int idx = threadIdx.x; idx < h * h; idx += blockDim.x) {
    const int i = idx / h, j = idx - i * h;
    Ls[i][j] = (j <= i) ? t.L[(size_t)i * t.ld + j] : T(0);
  }
  for (int i = 0; i < SOLVE_RB; ++i) Xs[i][c] = T(0);
  __syncthreads();
  if (c < h) {
    for (int i = c; i < h; ++i) {
      T s = (i == c) ? T(1) : T(0);
      for (int k = c; k < i; ++k) s -= Ls[i][k] * Xs[k][c];
      Xs[i][c] = s / Ls[i][i];
    }
  }
  __syncthreads();
  T* D = t.D;
  if (c < pad)
    for (int i = 0; i < pad; ++i) D[(size_t)i * ldD + c] = (i < h && c < h) ? Xs[i][c] : T(0);
}

template <class A, class B>
__global__ void convert_kernel(const A* __restrict__ src, B* __restrict__ dst, int n) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (B)src[i];
}

// Zero the interior completion counters and solved flags after their last
// reader (the backward launch), grid-stride.
__device__ __forceinline__ void clear_piece(int* c, int count) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) c[i] = 0;
}

__global__ void clear_counters(int* __restrict__ c, int count) {
  pdl_enter();
  clear_piece(c, count);
}

// last kernel of a mixed-precision apply: w64 = (double) w and the counters cleared
template <class T>
__global__ void convert_out_kernel(const T* __restrict__ src, double* __restrict__ dst, int n, int* __restrict__ c,
                                   int count) {
  pdl_enter();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
  if (c) clear_piece(c, count);
}

}  // namespace

template <class T>
SolveEngine<T>::SolveEngine(FactorEngine<T>& F) : F_(F) {
  const char* e = std::getenv("RSCHOL_AUTOTUNE");
  autotune_ = e && e[0] == '1';
}

template <class T>
void SolveEngine<T>::plan() {
  PlanClock clk("solve plan");
  const Symbolic& S = F_.S;
  const int nn = (int)S.nodes.size();
  nodes_.assign(nn, SNode<T>{});
  std::vector<int> rowsAll, rel, child, lvlNodes;
  long long wuCur = 0, dinvCur = 0, zpCur = 0, spCur = 0, ipCur = 0, xCur = 0, xpCur = 0;
  int syncCur = SYNC_GLOBAL;   // error word, ticket and completion counters of the interior launches
  std::vector<long long> xOff(nn, -1);
  std::vector<long long> xTaskOff;   // per compressed diagonal-block task: offset in the X arena
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
      syncCur += 3;   // backward chunk counter, forward completion count, backward solved flag
      sn.parentI = (nd.parent >= 0 && !S.nodes[nd.parent].compressed) ? nd.parent : -1;
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
        t.ldD = t.h;
        dinvTasks.push_back(t);
        dinvTaskOff.push_back(dinvCur + (long long)b * SOLVE_RB * SOLVE_RB);
        xTaskOff.push_back(-1);
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
      syncCur += 2;   // row blocks of y done, V chunks of s done
      sn.ncb = (nd.n + XT_COLS - 1) / XT_COLS;
      sn.zpOff2 = xpCur;
      xpCur += (long long)nd.n * sn.nb;
      sn.zpOff = zpCur;
      zpCur += (long long)sn.nb * sn.r;
      sn.spOff = spCur;
      spCur += (long long)sn.nch * sn.r;
      // X = L11^{-1}: the inverted 64 x 64 diagonal blocks go in place
      xOff[s] = xCur;
      for (int b = 0; b < sn.nb; ++b) {
        DinvTask<T> t{};
        t.L = sn.L + (size_t)b * SOLVE_RB * sn.ld + (size_t)b * SOLVE_RB;
        t.ld = sn.ld;
        t.h = std::min(SOLVE_RB, nd.n - b * SOLVE_RB);
        t.pad = t.h;
        t.ldD = nd.n;
        dinvTasks.push_back(t);
        dinvTaskOff.push_back(-1);
        xTaskOff.push_back(xCur + (long long)b * SOLVE_RB * nd.n + (long long)b * SOLVE_RB);
      }
      xCur += (long long)nd.n * nd.n;
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
  // backward order: the levels top-down
  std::vector<RowBlock> iworkB;
  for (int l = (int)iLevels_.size() - 1; l >= 0; --l)
    iworkB.insert(iworkB.end(), iwork.begin() + iLevels_[l].first,
                  iwork.begin() + iLevels_[l].first + iLevels_[l].second);
  // the single-vector apply: per level, the small supernodes in groups of
  // eight (a warp each), then the chunk blocks of the others
  std::vector<RowBlock> iworkS, iworkSB;
  std::vector<int> small;
  {
    std::vector<std::pair<size_t, size_t>> lvRange;   // per level: [begin, end) in iworkS
    bool anySmall = false;
    for (auto& lv : F_.interiorLevels) {
      const size_t b0 = iworkS.size();
      std::vector<int> sm;
      for (int d : lv)
        if (S.nodes[d].n <= IW_N && S.nodes[d].m() <= ICH) sm.push_back(d);
      for (size_t g = 0; g < sm.size(); g += 8) {
        const int cnt = (int)std::min<size_t>(8, sm.size() - g);
        iworkS.push_back(RowBlock{-1 - (int)(small.size() / 8), cnt});
        for (int q = 0; q < 8; ++q) small.push_back(q < cnt ? sm[g + q] : -1);
        anySmall = true;
      }
      for (int d : lv)
        if (!(S.nodes[d].n <= IW_N && S.nodes[d].m() <= ICH))
          for (int c = 0; c < std::max(1, nodes_[d].nch); ++c) iworkS.push_back(RowBlock{d, c});
      lvRange.push_back({b0, iworkS.size()});
    }
    for (int l = (int)lvRange.size() - 1; l >= 0; --l)
      iworkSB.insert(iworkSB.end(), iworkS.begin() + lvRange[l].first, iworkS.begin() + lvRange[l].second);
    smemWarps_ = anySmall ? sizeof(T) * 8 * (IW_N + ICH) : 0;
  }
  for (size_t v : smemIB_)
    if (v > 200 * 1024) throw std::runtime_error("interior front too large for the shared-memory solve");
  // compressed levels: (supernode, 64-row block) work lists
  std::vector<RowBlock> tickF;
  tickOff_.clear();
  cBlocks_.clear();
  cMaxCh_.clear();
  cVzGrid_.clear();
  cRowGrid_.clear();
  cColGrid_.clear();
  cMRowGrid_.clear();
  std::vector<XTile> xtiles;
  cTiles_.clear();
  for (auto& lv : F_.compressedLevels) {
    cLevels_.push_back({(long long)lvlNodes.size(), (int)lv.size()});
    lvlNodes.insert(lvlNodes.end(), lv.begin(), lv.end());
    tickOff_.push_back((long long)tickF.size());
    const long long t0 = (long long)xtiles.size();
    for (int j : lv)   // tiles with a part on or below the diagonal
      for (int ib = 0; ib < nodes_[j].nb; ++ib)
        for (int jb = 0; jb < nodes_[j].ncb && jb * XT_COLS <= ib * SOLVE_RB + SOLVE_RB - 1; ++jb)
          xtiles.push_back(XTile{j, ib, jb});
    cTiles_.push_back({t0, (int)((long long)xtiles.size() - t0)});
    int maxCh = 1, blocks = 0, maxN = 1, maxM = 1;
    for (int j : lv) {
      maxCh = std::max(maxCh, nodes_[j].nch);
      blocks += nodes_[j].nb;
      maxN = std::max(maxN, nodes_[j].n);
      maxM = std::max(maxM, nodes_[j].m);
      for (int b = 0; b < nodes_[j].nb; ++b) tickF.push_back(RowBlock{j, b});
    }
    cBlocks_.push_back(blocks);
    cMaxCh_.push_back(maxCh);
    cVzGrid_.push_back(std::min(64, (maxM + 7) / 8));
    cRowGrid_.push_back((maxN + 7) / 8);
    cMRowGrid_.push_back((maxM + 7) / 8);
    cColGrid_.push_back((maxN + 255) / 256);
  }
  clk.mark("layout");
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
  dXp_.alloc(sizeof(T) * std::max(1LL, xpCur));
  dX_.alloc(sizeof(T) * std::max(1LL, xCur));
  RSCHOL_CUDA(cudaMemsetAsync(dX_.p, 0, sizeof(T) * std::max(1LL, xCur), st));   // upper triangles stay zero
  for (size_t q = 0; q < dinvTasks.size(); ++q)
    dinvTasks[q].D = xTaskOff[q] >= 0 ? dX_.as<T>() + xTaskOff[q] : dDinv_.as<T>() + dinvTaskOff[q];
  for (int s = 0; s < nn; ++s) {
    if (S.nodes[s].compressed) nodes_[s].X = dX_.as<T>() + xOff[s];
    else nodes_[s].Dinv = dDinv_.as<T>() + dinvNodeOff[s];
  }
  nDinv_ = (int)dinvTasks.size();
  clk.mark("arenas");
  plan_inverse(xOff);
  clk.mark("inverse");
  // per-row contribution lists of the compressed supernodes (in source order)
  {
    std::vector<long long> cstart;
    std::vector<long long> ents;   // offsets into the update-vector arena
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
          const long long e = (P.kind == 0) ? src.wuOff + a : src.wuOff + 2 * src.r + a;
          ents[base + fill[S.nodes[P.src].rows[a] - nd.c0]++] = e;
        }
      }
    }
    up(dCStart_, cstart.data(), cstart.size() * sizeof(long long));
    up(dCEnt_, ents.data(), ents.size() * sizeof(long long));
  }
  up(dNodes_, nodes_.data(), nodes_.size() * sizeof(SNode<T>));
  up(dRows_, rowsAll.data(), rowsAll.size() * sizeof(int));
  up(dRel_, rel.data(), rel.size() * sizeof(int));
  up(dChild_, child.data(), child.size() * sizeof(int));
  up(dLevelNodes_, lvlNodes.data(), lvlNodes.size() * sizeof(int));
  up(dIWork_, iwork.data(), iwork.size() * sizeof(RowBlock));
  up(dIWorkB_, iworkB.data(), iworkB.size() * sizeof(RowBlock));
  nIWork_ = (int)iwork.size();
  up(dIWorkS_, iworkS.data(), iworkS.size() * sizeof(RowBlock));
  up(dIWorkSB_, iworkSB.data(), iworkSB.size() * sizeof(RowBlock));
  up(dSmall_, small.data(), small.size() * sizeof(int));
  nIWorkS_ = (int)iworkS.size();
  wuTotal_ = wuCur;
  ipTotal_ = ipCur;
  maxNI_ = 0;
  for (int s = 0; s < nn; ++s)
    if (!S.nodes[s].compressed) maxNI_ = std::max(maxNI_, S.nodes[s].n);
  kB_ = 0;   // the batched apply re-plans on its next use
  smemIFmax_ = 8;
  smemIBmax_ = 8;
  for (size_t v : smemIF_) smemIFmax_ = std::max(smemIFmax_, v);
  for (size_t v : smemIB_) smemIBmax_ = std::max(smemIBmax_, v);
  up(dTickF_, tickF.data(), tickF.size() * sizeof(RowBlock));
  up(dTiles_, xtiles.data(), xtiles.size() * sizeof(XTile));
  up(dDinvTasks_, dinvTasks.data(), dinvTasks.size() * sizeof(DinvTask<T>));
  syncInts_ = syncCur;
  dSync_.alloc(sizeof(int) * syncCur);
  RSCHOL_CUDA(cudaMemsetAsync(dSync_.p, 0, sizeof(int) * syncCur, st));
  if (!std::is_same<T, double>::value) dW_.alloc(sizeof(T) * std::max(1, S.n));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  clk.mark("upload");
  const int maxSmem = 200 * 1024;
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_forward_chunks<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_backward_chunks<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  launchesPerApply_ = (iLevels_.empty() ? 0 : 2) + 8 * (long long)cLevels_.size() - (cLevels_.empty() ? 0 : 1) +
                      (std::is_same<T, double>::value ? (nIWorkS_ > 0 ? 1 : 0) : 2);
  bytesPerApply_ += 8.0 * 4 * S.n;
}

template <class T>
void SolveEngine<T>::plan_inverse(const std::vector<long long>& xOff) {
  // X = L11^{-1} of every compressed supernode by recursive doubling: with
  // the diagonal 64 x 64 inverses in place, for block sizes sz = 64, 128, ...
  // every pair (A, B) of consecutive sz-blocks gets X_BA = -X_BB (L_BA X_AA).
  // Both products run by 64-column (64-row) blocks whose K stops at the
  // triangle, so the work is n^3 / 3 per supernode.
  const Symbolic& S = F_.S;
  const bool tc = std::is_same<T, float>::value && F_.tensor_cores();
  const int rpt = tc ? 128 : 64;
  const int nn = (int)S.nodes.size();
  int maxN = 0;
  for (int s = 0; s < nn; ++s)
    if (S.nodes[s].compressed) maxN = std::max(maxN, S.nodes[s].n);
  long long t1Max = 1;
  for (int sz = SOLVE_RB; sz < maxN; sz *= 2) {
    long long t1 = 0;
    for (int s = 0; s < nn; ++s) {
      const int n = S.nodes[s].n;
      if (!S.nodes[s].compressed) continue;
      for (int A0 = 0; A0 + sz < n; A0 += 2 * sz) t1 += (long long)std::min(sz, n - A0 - sz) * sz;
    }
    t1Max = std::max(t1Max, t1);
  }
  dT1_.alloc(sizeof(T) * t1Max);
  std::vector<GemmTask<T>> tasks;
  xSteps_.clear();
  auto mk = [&](const T* A, int lda, const T* B, int ldb, T* C, int ldc, int M, int N, int K, T alpha) {
    GemmTask<T> t{};
    t.A = A;
    t.B = B;
    t.C = C;
    t.M = M;
    t.N = N;
    t.K = K;
    t.lda = lda;
    t.ldb = ldb;
    t.ldc = ldc;
    t.alpha = alpha;
    t.beta = T(0);
    t.tilesN = (N + 63) / 64;
    t.split = 1;
    t.kSplit = 1;
    t.kLen = K;
    return t;
  };
  auto flush = [&](std::vector<GemmTask<T>>& batch) {
    if (batch.empty()) return;
    int maxN = 0;
    for (auto& t : batch) maxN = std::max(maxN, t.N);
    const int bn = tc ? tc_tile_n(maxN) : 64;
    int tiles = 0;
    for (auto& t : batch) {
      t.tilesN = (t.N + bn - 1) / bn;
      t.bn = bn;
      t.tileBase = tiles;
      tiles += ((t.M + rpt - 1) / rpt) * t.tilesN;
    }
    XStep xs{(long long)tasks.size(), (int)batch.size(), tiles, tc ? 1 : 0};
    xs.bn = bn;
    xSteps_.push_back(xs);
    tasks.insert(tasks.end(), batch.begin(), batch.end());
    batch.clear();
  };
  for (int sz = SOLVE_RB; sz < maxN; sz *= 2) {
    std::vector<GemmTask<T>> b1, b2;
    long long t1cur = 0;
    for (int s = 0; s < nn; ++s) {
      if (!S.nodes[s].compressed) continue;
      const int n = S.nodes[s].n, ld = nodes_[s].ld;
      const T* L = nodes_[s].L;
      T* X = dX_.as<T>() + xOff[s];
      for (int A0 = 0; A0 + sz < n; A0 += 2 * sz) {
        const int B0 = A0 + sz, bsz = std::min(sz, n - B0);
        T* T1 = dT1_.as<T>() + t1cur;
        t1cur += (long long)bsz * sz;
        for (int a = 0; a * SOLVE_RB < sz; ++a)   // T1[:, a] = L_BA[:, a:] X_AA[a:, a]
          b1.push_back(mk(L + (size_t)B0 * ld + A0 + a * SOLVE_RB, ld,
                          X + (size_t)(A0 + a * SOLVE_RB) * n + A0 + a * SOLVE_RB, n, T1 + a * SOLVE_RB, sz, bsz,
                          SOLVE_RB, sz - a * SOLVE_RB, T(1)));
        for (int b = 0; b * SOLVE_RB < bsz; ++b) {   // X_BA[b, :] = -X_BB[b, :b] T1[:b, :]
          const int hb = std::min(SOLVE_RB, bsz - b * SOLVE_RB), K = std::min(bsz, (b + 1) * SOLVE_RB);
          b2.push_back(mk(X + (size_t)(B0 + b * SOLVE_RB) * n + B0, n, T1, sz,
                          X + (size_t)(B0 + b * SOLVE_RB) * n + A0, n, hb, sz, K, T(-1)));
        }
      }
    }
    flush(b1);
    flush(b2);
  }
  dXGemm_.alloc(std::max<size_t>(16, tasks.size() * sizeof(GemmTask<T>)));
  if (!tasks.empty())
    RSCHOL_CUDA(cudaMemcpyAsync(dXGemm_.p, tasks.data(), tasks.size() * sizeof(GemmTask<T>), cudaMemcpyHostToDevice,
                                F_.stream));
}

template <class T>
int SolveEngine<T>::prepare(cudaStream_t st) {
  int launches = 0;
  if (nDinv_ > 0) {
    constexpr int smem = 2 * (int)sizeof(T) * SOLVE_RB * (SOLVE_RB + 1);
    static std::once_flag once;
    std::call_once(once, [] {
      RSCHOL_CUDA(cudaFuncSetAttribute(invert_diag_blocks<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    });
    invert_diag_blocks<T><<<nDinv_, SOLVE_RB, smem, st>>>(dDinvTasks_.as<DinvTask<T>>());
    RSCHOL_LAUNCH_CHECK();
    ++launches;
  }
  for (const XStep& x : xSteps_) {
    const GemmTask<T>* d = dXGemm_.as<GemmTask<T>>() + x.off;
    if constexpr (std::is_same<T, float>::value) {
      if (F_.tensor_cores()) launch_gemm_tc(d, x.count, x.tiles, F_.dFlag.template as<int>() + 1, st, x.bn);
      else launch_gemm<T>(d, x.count, x.tiles, st);
    } else {
      launch_gemm<T>(d, x.count, x.tiles, st);
    }
    ++launches;
  }
  return launches;
}

template <class T>
int SolveEngine<T>::take_error(cudaStream_t st) {
  int e = 0;
  if (!dSync_.p) return 0;
  RSCHOL_CUDA(cudaMemcpyAsync(&e, dSync_.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  if (e) {
    // a wait gave up: counters and flags are in an unknown state; start over
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
    launch_k(convert_kernel<double, T>, dim3((n + 255) / 256), dim3(256), 0, st, w64, w, n);
    RSCHOL_LAUNCH_CHECK();
  }
  const int* lvl = dLevelNodes_.as<int>();
  int* sync = dSync_.as<int>();
  const int epoch = 1;   // completion targets: every apply starts its counters at zero
  if (nIWorkS_ > 0) {
    launch_k(interior_forward_chunks<T>, dim3(nIWorkS_), dim3(256), std::max(smemIFmax_, smemWarps_), st, dNodes_.as<SNode<T>>(), dIWorkS_.as<RowBlock>(), dRel_.as<int>(), dChild_.as<int>(), sync, epoch, w, dYi_.as<T>(), dWu_.as<T>(), dSmall_.as<int>());
    RSCHOL_LAUNCH_CHECK();
  }
  T* yv = dYi_.as<T>();
  for (size_t l = 0; l < cLevels_.size(); ++l) {
    const int* lv = lvl + cLevels_[l].first;
    launch_k(compressed_gather_rows<T>, dim3(cRowGrid_[l], cLevels_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), lv, dCStart_.as<long long>(), dCEnt_.as<long long>(), dWu_.as<T>(), w);
    RSCHOL_LAUNCH_CHECK();
    launch_k(compressed_ytile_kernel<T>, dim3(cTiles_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), dTiles_.as<XTile>() + cTiles_[l].first, w, dXp_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    launch_k(compressed_y_kernel<T>, dim3(cBlocks_[l]), dim3(256), 0, st, dNodes_.as<SNode<T>>(), dTickF_.as<RowBlock>() + tickOff_[l], sync, dZp_.as<T>(), dXp_.as<T>(), yv, dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    if (l + 1 < cLevels_.size()) {   // the top level's u feeds no one
      launch_k(compressed_vz_kernel<T>, dim3(cVzGrid_[l], cLevels_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), lv, dWu_.as<T>());
      RSCHOL_LAUNCH_CHECK();
    }
  }
  for (int l = (int)cLevels_.size() - 1; l >= 0; --l) {
    const int* lv = lvl + cLevels_[l].first;
    launch_k(compressed_vtx_kernel<T>, dim3(cMaxCh_[l], cLevels_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), lv, dRows_.as<int>(), sync, dSp_.as<T>(), w, dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    launch_k(compressed_g_kernel<T>, dim3(cRowGrid_[l], cLevels_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), lv, dWu_.as<T>(), yv);
    RSCHOL_LAUNCH_CHECK();
    launch_k(compressed_xtile_kernel<T>, dim3(cTiles_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), dTiles_.as<XTile>() + cTiles_[l].first, yv, dXp_.as<T>());
    RSCHOL_LAUNCH_CHECK();
    launch_k(compressed_x_reduce<T>, dim3(cColGrid_[l], cLevels_[l].second), dim3(256), 0, st, dNodes_.as<SNode<T>>(), lv, dXp_.as<T>(), w);
    RSCHOL_LAUNCH_CHECK();
  }
  if (nIWorkS_ > 0) {
    launch_k(interior_backward_chunks<T>, dim3(nIWorkS_), dim3(256), std::max(smemIBmax_, smemWarps_), st, dNodes_.as<SNode<T>>(), dIWorkSB_.as<RowBlock>(), dRows_.as<int>(), sync, epoch, dIp_.as<T>(), dYi_.as<T>(), w, dSmall_.as<int>());
    RSCHOL_LAUNCH_CHECK();
  }
  // the interior counters are cleared by the apply's last kernel
  int* clr = nIWorkS_ > 0 ? sync + SYNC_GLOBAL : nullptr;
  const int nClr = nIWorkS_ > 0 ? syncInts_ - SYNC_GLOBAL : 0;
  if (!std::is_same<T, double>::value) {
    launch_k(convert_out_kernel<T>, dim3((n + 255) / 256), dim3(256), 0, st, (const T*)w, w64, n, clr, nClr);
    RSCHOL_LAUNCH_CHECK();
  } else if (nClr > 0) {
    launch_k(clear_counters, dim3((nClr + 1023) / 1024), dim3(256), 0, st, clr, nClr);
    RSCHOL_LAUNCH_CHECK();
  }
}

template class SolveEngine<double>;
template class SolveEngine<float>;

}  // namespace rschol
