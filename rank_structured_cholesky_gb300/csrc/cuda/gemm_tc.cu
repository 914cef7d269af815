// Batched FP32 GEMM on the 5th-generation tensor cores (tcgen05, kind::tf32).
//
// Same task semantics as the SIMT gemm_kernel (C = alpha op(A) op(B) +
// beta C, row-major, per-task shapes; lower tasks skip tiles above the
// diagonal), one 128 x BN output tile (BN = 64 or 128 per launch, the task's
// bn; and K slice) per CTA.  Operands are staged into shared memory in the
// K-major 128-byte swizzled layout (a row of 32 TF32 per 128 bytes, 16-byte
// chunks XORed with the row index) by producer warps, a multi-stage mbarrier
// pipeline feeds a single MMA-issuing thread (tcgen05.mma into a TMEM
// accumulator), and the epilogue reads TMEM with tcgen05.ld and writes C
// through shared memory in coalesced rows (gemm_tc_kernel below).  Tasks with
// a large K and few tiles are split along K (kSplit slices write FP32
// partials to a workspace; gemm_splitk_reduce sums them in slice order).
//
// Split precision (task.split != 0): a = a_hi + a_lo with a_hi = tf32(a),
// a_lo = tf32(a - a_hi), and A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi (three
// MMAs per K step, FP32 accuracy up to the dropped A_lo B_lo term), for the
// Schur-complement updates whose errors the factor cannot absorb.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "dense.cuh"
#include "tc_dev.cuh"

namespace rschol {

namespace {

constexpr int TC_BM = 128, TC_BN = 64, TC_BK = 32;   // TC_BN: the tile width of tasks that state none
using namespace tcdev;


// ---------------------------------------------------------------------------
// The kernel.  One 128 x BN output tile (and K slice) per CTA of 640 threads,
// warp-specialised:
//   warps 0-15 producers, in one of two ways per task:
//              TMA (the task carries tensor maps: K-major, 16-byte-aligned
//              operands of a TF32 launch): warp 0 issues each K tile's two
//              boxes (raw FP32, already in the swizzled layout) as soon as the
//              stage is free; warps 1-15 round the landed tile to TF32 in
//              place, write the split remainders, and arrive on "full";
//              registers (the rest): each K tile of 32 goes global ->
//              registers (16-byte vector loads along the operand's contiguous
//              dimension) -> TF32 (or BF16) hi and lo, transposed when the
//              operand's contiguous dimension is M or N -> one of NS stages in
//              the K-major 128-byte-swizzled layout; then one arrival per
//              thread on the stage's "full" barrier;
//   warp 16    lane 0 issues the stage's tcgen05.mma (M 128, N BN, K 8; three
//              per K step for split products) into the TMEM accumulator as soon
//              as the stage is full, and commits to the stage's "empty"
//              barrier, which frees it for the producers;
//   warps 16-19 epilogue: after the final commit, TMEM -> registers
//              (tcgen05.ld, 32 lanes each) -> shared rows -> C (or the
//              K-slice partials) in coalesced rows, by all threads.
// NS stages keep NS K tiles in flight, so loads, conversion and MMAs of
// different stages overlap.  The producers' global-load latency bounds a
// stage: the c2 factor took 25.49 ms with four producer warps, 24.39 with
// eight, 24.27 with sixteen.  (Measured
// against it on the c2 factor's GEMM steps: both operands' loads issued
// before either is stored, with L2 prefetches of the tiles ahead, 4.33 vs
// 4.15 ms; asynchronous 16-byte copies into three raw stages converted into
// two MMA stages, 5.15 ms.)  Every wait is bounded; a wait that gives up sets
// *err, stops the loops, waits (bounded) for the CTA's issued MMAs and frees
// the TMEM before returning.
// ---------------------------------------------------------------------------
constexpr int WS_PW = 16;                         // producer warps
constexpr int WS_PT = 32 * WS_PW;                 // producer threads
constexpr int WS_THREADS = WS_PT + 128;           // + the MMA / epilogue warpgroup

// One ROWS x 32 K tile of an operand into the stage's swizzled K-major
// buffers (hi at dst, lo at dst + loOff when split).  Element (r, k) of the
// tile is src[(row0 + r) * ld + k0 + k] (kContig) or src[(k0 + k) * ld + row0
// + r]; rows >= nRows and k >= kEnd read as zero.  vec: the 16-byte loads
// along the contiguous dimension are aligned (checked per task).  BF: the
// tile is stored as BF16 (hi = bf16(a), lo = bf16(a - hi)) at element
// positions kPos .. kPos + 31 of the 64-element (128-byte) rows; otherwise as
// TF32 filling the 32-element rows.
template <int ROWS, bool BF>
__device__ __forceinline__ void ws_load_tile(const float* __restrict__ src, int ld, bool kContig, bool vec, int row0,
                                             int nRows, int k0, int kEnd, uint32_t dst, uint32_t loOff, bool split,
                                             int tid, int kPos = 0) {
  constexpr int PER = ROWS * 32 / 4 / WS_PT;   // float4 groups per producer thread
  float4 v[PER];
  if (kContig) {
    // group g: row g >> 3, k 4 (g & 7) .. +3
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int g = tid + WS_PT * q, r = g >> 3, kk = (g & 7) * 4;
      const int gr = row0 + r, gk = k0 + kk;
      const float* p = src + (size_t)gr * ld + gk;
      if (gr < nRows && vec && gk + 3 < kEnd) {
        v[q] = __ldg(reinterpret_cast<const float4*>(p));
      } else {
        v[q].x = (gr < nRows && gk < kEnd) ? __ldg(p) : 0.f;
        v[q].y = (gr < nRows && gk + 1 < kEnd) ? __ldg(p + 1) : 0.f;
        v[q].z = (gr < nRows && gk + 2 < kEnd) ? __ldg(p + 2) : 0.f;
        v[q].w = (gr < nRows && gk + 3 < kEnd) ? __ldg(p + 3) : 0.f;
      }
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int g = tid + WS_PT * q, r = g >> 3, kk = (g & 7) * 4;
      if constexpr (BF) {
        const uint32_t off = tc_off16(r, kPos + kk);
        float l[4];
        const uint32_t h01 = split_bf16x2(v[q].x, v[q].y, l[0], l[1]), h23 = split_bf16x2(v[q].z, v[q].w, l[2], l[3]);
        st_shared_v2(dst + off, h01, h23);
        if (split) st_shared_v2(dst + loOff + off, pack_bf16x2(l[0], l[1]), pack_bf16x2(l[2], l[3]));
      } else {
        const uint32_t off = tc_off(r, kk);
        const uint32_t h0 = to_tf32(v[q].x), h1 = to_tf32(v[q].y), h2 = to_tf32(v[q].z), h3 = to_tf32(v[q].w);
        st_shared_v4(dst + off, h0, h1, h2, h3);
        if (split)
          st_shared_v4(dst + loOff + off, to_tf32(v[q].x - __uint_as_float(h0)),
                       to_tf32(v[q].y - __uint_as_float(h1)), to_tf32(v[q].z - __uint_as_float(h2)),
                       to_tf32(v[q].w - __uint_as_float(h3)));
      }
    }
  } else {
    // group g: k g / (ROWS / 4), rows 4 (g mod ROWS / 4) .. +3
    constexpr int GR = ROWS / 4;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int g = tid + WS_PT * q, kk = g / GR, r = (g % GR) * 4;
      const int gr = row0 + r, gk = k0 + kk;
      const float* p = src + (size_t)gk * ld + gr;
      if (gk < kEnd && vec && gr + 3 < nRows) {
        v[q] = __ldg(reinterpret_cast<const float4*>(p));
      } else {
        v[q].x = (gk < kEnd && gr < nRows) ? __ldg(p) : 0.f;
        v[q].y = (gk < kEnd && gr + 1 < nRows) ? __ldg(p + 1) : 0.f;
        v[q].z = (gk < kEnd && gr + 2 < nRows) ? __ldg(p + 2) : 0.f;
        v[q].w = (gk < kEnd && gr + 3 < nRows) ? __ldg(p + 3) : 0.f;
      }
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
      const int g = tid + WS_PT * q, kk = g / GR, r = (g % GR) * 4;
      const float e[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if constexpr (BF) {
          const uint32_t off = tc_off16(r + u, kPos + kk);
          const __nv_bfloat16 h = __float2bfloat16_rn(e[u]);
          st_shared_b16(dst + off, __bfloat16_as_ushort(h));
          if (split)
            st_shared_b16(dst + loOff + off, __bfloat16_as_ushort(__float2bfloat16_rn(e[u] - __bfloat162float(h))));
        } else {
          const uint32_t off = tc_off(r + u, kk), h = to_tf32(e[u]);
          st_shared_b32(dst + off, h);
          if (split) st_shared_b32(dst + loOff + off, to_tf32(e[u] - __uint_as_float(h)));
        }
      }
    }
  }
}

// A stage buffer of raw FP32 (bytes at base) rounded to TF32 in place; split:
// the remainders tf32(a - hi) to the lo buffer that follows it.  The layout is
// elementwise, so the swizzle needs no decoding.  Thread ctid of nThreads.
__device__ __forceinline__ void tf32_in_place(uint32_t base, int bytes, bool split, int ctid, int nThreads) {
  for (int off = ctid * 16; off < bytes; off += nThreads * 16) {
    const float4 v = ld_shared_v4(base + off);
    const uint32_t h0 = to_tf32(v.x), h1 = to_tf32(v.y), h2 = to_tf32(v.z), h3 = to_tf32(v.w);
    st_shared_v4(base + off, h0, h1, h2, h3);
    if (split)
      st_shared_v4(base + bytes + off, to_tf32(v.x - __uint_as_float(h0)), to_tf32(v.y - __uint_as_float(h1)),
                   to_tf32(v.z - __uint_as_float(h2)), to_tf32(v.w - __uint_as_float(h3)));
  }
}

template <int BN, int NS, bool BF>
__global__ void __launch_bounds__(WS_THREADS, 1) gemm_tc_kernel(const GemmTask<float>* __restrict__ tasks,
                                                                  int nTasks, int* __restrict__ err) {
  // a stage holds 128-byte rows: 32 K as TF32, or 64 K as BF16
  constexpr int SK = BF ? 2 * TC_BK : TC_BK;
  constexpr int A_BYTES = TC_BM * 128, B_BYTES = BN * 128;
  constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;   // hi and lo of both operands
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t fullB[NS], emptyB[NS], tmaB[NS], doneB;
  __shared__ uint32_t tmemBase;
  __shared__ volatile int sAbort;
  int lo = 0, hi = nTasks - 1;
  const int bid = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tasks[mid].tileBase <= bid) lo = mid;
    else hi = mid - 1;
  }
  const GemmTask<float> t = tasks[lo];
  const int tilesPer = ((t.M + TC_BM - 1) / TC_BM) * t.tilesN;
  const int local = bid - t.tileBase;
  const int slice = local / tilesPer, tl = local - slice * tilesPer;
  const int ti = tl / t.tilesN, tj = tl - ti * t.tilesN;
  const int row0 = ti * TC_BM, col0 = tj * BN;
  if (t.lower && row0 + TC_BM - 1 < col0) return;   // uniform over the block, before any allocation
  const int kl = t.kLen > 0 ? t.kLen : t.K;
  const int kBeg = slice * kl, kEnd = min(t.K, kBeg + kl);
  const int nk = kEnd > kBeg ? (kEnd - kBeg + SK - 1) / SK : 0;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool split = t.split != 0;
  const uint32_t sraw = (uint32_t)__cvta_generic_to_shared(tc_smem);
  const uint32_t sbase = (sraw + 1023u) & ~1023u;
  const uint32_t full0 = (uint32_t)__cvta_generic_to_shared(&fullB[0]);
  const uint32_t empty0 = (uint32_t)__cvta_generic_to_shared(&emptyB[0]);
  const uint32_t done = (uint32_t)__cvta_generic_to_shared(&doneB);
  const uint32_t tma0 = (uint32_t)__cvta_generic_to_shared(&tmaB[0]);

  if (warp == WS_PW) {
    tmem_alloc((uint32_t)__cvta_generic_to_shared(&tmemBase), BN);
  }
  bool viaTma = false;
  if constexpr (!BF) viaTma = t.tmA != nullptr && t.tmB != nullptr;
  if (tid == 0) {
    for (int st = 0; st < NS; ++st) {
      mbar_init(full0 + 8u * st, viaTma ? WS_PT - 32 : WS_PT);   // TMA staging: warp 0 issues, the rest convert
      mbar_init(empty0 + 8u * st, 1);
      mbar_init(tma0 + 8u * st, 1);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sAbort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;

  if (warp == 0 && viaTma) {
    // ---- TMA staging, issuer: lane 0 refills each stage as soon as the MMAs
    // have released it (up to NS stages ahead of the conversion); the boxes
    // are raw FP32 in the swizzled layout, zeros beyond the operands' extents
    if (lane == 0) {
      const uint64_t mA = reinterpret_cast<uint64_t>(t.tmA), mB = reinterpret_cast<uint64_t>(t.tmB);
      tmap_acquire(mA);
      tmap_acquire(mB);
      for (int kt = 0; kt < nk; ++kt) {
        const int st = kt % NS, use = kt / NS;
        if (use > 0 && !mbar_wait(empty0 + 8u * st, (uint32_t)((use - 1) & 1))) {
          atomicExch(err, 1);
          sAbort = 1;
        }
        if (sAbort) break;
        const uint32_t a = sbase + (uint32_t)(st * STAGE), b = a + 2 * A_BYTES;
        const int k0 = kBeg + kt * TC_BK;   // slices start on a K tile: a box never crosses into the next slice
        mbar_arrive_expect_tx(tma0 + 8u * st, (uint32_t)(A_BYTES + B_BYTES));
        tma_load_2d(a, mA, k0, row0, tma0 + 8u * st);
        tma_load_2d(b, mB, k0, col0, tma0 + 8u * st);
      }
    }
    __syncwarp();
  } else if (warp < WS_PW && viaTma) {
    // ---- TMA staging, converters (warps 1..): round each landed stage to
    // TF32 in place and, for split products, write the remainders to its lo
    // buffers; then one arrival per thread on the stage's "full" barrier
    const int ctid = tid - 32, nct = WS_PT - 32;
    for (int kt = 0; kt < nk; ++kt) {
      const int st = kt % NS, use = kt / NS;
      if (!mbar_wait(tma0 + 8u * st, (uint32_t)(use & 1))) {
        atomicExch(err, 1);
        sAbort = 1;
      }
      if (sAbort) break;
      const uint32_t a = sbase + (uint32_t)(st * STAGE), b = a + 2 * A_BYTES;
      tf32_in_place(a, A_BYTES, split, ctid, nct);
      tf32_in_place(b, B_BYTES, split, ctid, nct);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(full0 + 8u * st);
    }
  } else if (warp < WS_PW) {
    // ---- producers, register staging
    // 16-byte loads need the operand and its leading dimension aligned
    const bool aK = !t.tA, bK = t.tB != 0;   // K contiguous in memory
    const bool aVec = ((reinterpret_cast<uintptr_t>(t.A) & 15u) == 0) && (t.lda & 3) == 0;
    const bool bVec = ((reinterpret_cast<uintptr_t>(t.B) & 15u) == 0) && (t.ldb & 3) == 0;
    for (int kt = 0; kt < nk; ++kt) {
      const int st = kt % NS, use = kt / NS;
      if (use > 0 && !mbar_wait(empty0 + 8u * st, (uint32_t)((use - 1) & 1))) {
        atomicExch(err, 1);
        sAbort = 1;
      }
      if (sAbort) break;
      const uint32_t a = sbase + (uint32_t)(st * STAGE), b = a + 2 * A_BYTES;
      const int k0 = kBeg + kt * SK;
#pragma unroll
      for (int h = 0; h < SK / TC_BK; ++h) {
        ws_load_tile<TC_BM, BF>(t.A, t.lda, aK, aVec, row0, t.M, k0 + TC_BK * h, kEnd, a, A_BYTES, split, tid,
                                TC_BK * h);
        ws_load_tile<BN, BF>(t.B, t.ldb, bK, bVec, col0, t.N, k0 + TC_BK * h, kEnd, b, B_BYTES, split, tid,
                             TC_BK * h);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(full0 + 8u * st);
    }
  } else if (warp == WS_PW) {
    // ---- MMA issue (one thread); the whole warp then joins the epilogue
    if (lane == 0) {
      int issued = 0;
      for (int kt = 0; kt < nk; ++kt) {
        const int st = kt % NS, use = kt / NS;
        if (!mbar_wait(full0 + 8u * st, (uint32_t)(use & 1))) {
          atomicExch(err, 1);
          sAbort = 1;
        }
        if (sAbort) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t a = sbase + (uint32_t)(st * STAGE), b = a + 2 * A_BYTES;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          const uint32_t step = (uint32_t)kk * 32u;   // 8 TF32 or 16 BF16 = 32 bytes along the swizzled row
          const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
          ws_mma<BN, BF>(tmem, tc_smem_desc(a + step), tc_smem_desc(b + step), acc);
          if (split) {
            ws_mma<BN, BF>(tmem, tc_smem_desc(a + step), tc_smem_desc(b + B_BYTES + step), 1u);
            ws_mma<BN, BF>(tmem, tc_smem_desc(a + A_BYTES + step), tc_smem_desc(b + step), 1u);
          }
        }
        tc_commit(empty0 + 8u * st);
        issued = kt + 1;
      }
      if (issued > 0) tc_commit(done);   // completes once every MMA issued above has
      else mbar_arrive(done);
    }
    __syncwarp();
  }
  // C of this tile into registers while the MMAs finish (all warps; rows warp + NW r, columns lane + 32 c):
  // the write-out then needs no dependent global load per row
  constexpr int NW = WS_THREADS / 32, RPW = (TC_BM + NW - 1) / NW, CPL = BN / 32;
  float cpre[RPW][CPL];
  const bool prefetchC = t.kSplit <= 1 && t.beta != 0.f;
  if (prefetchC) {
#pragma unroll
    for (int q = 0; q < RPW; ++q) {
      const int i = warp + NW * q, gm = row0 + i;
#pragma unroll
      for (int c = 0; c < CPL; ++c) {
        const int gn = col0 + lane + 32 * c;
        cpre[q][c] = (i < TC_BM && gm < t.M && gn < t.N) ? __ldg(t.C + (size_t)gm * t.ldc + gn) : 0.f;
      }
    }
  }
  // ---- epilogue: the last four warps take the accumulator rows 32 (warp - WS_PW) + lane (their TMEM lane
  // quarters: warp % 4 == warp - WS_PW)
  float* buf = reinterpret_cast<float*>(tc_smem + (sbase - sraw));   // 128 x (BN + 1), stages are free now
  bool ok = true;
  if (warp >= WS_PW) {
    ok = mbar_wait(done, 0u);
    if (!ok) {
      atomicExch(err, 1);
      sAbort = 1;
    }
  }
  __syncthreads();   // producers done too: the stage buffers may be reused
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const bool abort = sAbort != 0;
  if (!abort && warp >= WS_PW) {
    const int row = 32 * (warp - WS_PW) + lane;
    const uint32_t taddr = tmem + ((uint32_t)(32 * (warp - WS_PW)) << 16);
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 32) {
      uint32_t r[32];
      if (nk > 0) {
        tmem_ld32(taddr + (uint32_t)c0, r);
      } else {
#pragma unroll
        for (int c = 0; c < 32; ++c) r[c] = 0u;
      }
      float* rowp = buf + row * (BN + 1) + c0;
#pragma unroll
      for (int c = 0; c < 32; ++c) rowp[c] = __uint_as_float(r[c]);
    }
  }
  __syncthreads();
  if (!abort) {
    // coalesced write-out: a warp per row, lanes over columns
    if (t.kSplit > 1) {
      float* part = t.ws + ((size_t)slice * tilesPer + tl) * (TC_BM * BN);
      for (int i = warp; i < TC_BM; i += WS_THREADS / 32)
        for (int c = lane; c < BN; c += 32) part[i * BN + c] = buf[i * (BN + 1) + c];
    } else {
#pragma unroll
      for (int q = 0; q < RPW; ++q) {
        const int i = warp + NW * q, gm = row0 + i;
        if (i >= TC_BM || gm >= t.M) continue;
        float* crow = t.C + (size_t)gm * t.ldc;
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
          const int cc = lane + 32 * c, gn = col0 + cc;
          if (gn < t.N) {
            float v = t.alpha * buf[i * (BN + 1) + cc];
            if (prefetchC) v = fmaf(t.beta, cpre[q][c], v);
            crow[gn] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == WS_PW)
    tmem_dealloc(tmem, BN);
}

// C = alpha * (sum of the K-slice partials, in slice order) + beta * C for
// the split tasks of a launch; one thread per element of C.
__global__ void gemm_splitk_reduce(const GemmTask<float>* __restrict__ tasks, const int* __restrict__ ids, int nIds,
                                   const long long* __restrict__ elemBase) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= elemBase[nIds]) return;
  int lo = 0, hi = nIds - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (elemBase[mid] <= e) lo = mid;
    else hi = mid - 1;
  }
  const GemmTask<float> t = tasks[ids[lo]];
  const long long le = e - elemBase[lo];
  const int i = (int)(le / t.N), j = (int)(le - (long long)i * t.N);
  const int bn = t.bn > 0 ? t.bn : TC_BN;
  const int tilesPer = ((t.M + TC_BM - 1) / TC_BM) * t.tilesN;
  const int tl = (i / TC_BM) * t.tilesN + j / bn;
  const int off = (i % TC_BM) * bn + (j % bn);
  float s = 0.f;
  for (int sl = 0; sl < t.kSplit; ++sl) s += t.ws[((size_t)sl * tilesPer + tl) * (TC_BM * bn) + off];
  float* c = t.C + (size_t)i * t.ldc + j;
  float v = t.alpha * s;
  if (t.beta != 0.f) v = fmaf(t.beta, *c, v);
  *c = v;
}

}  // namespace

template <int BN, int NS, bool BF>
void launch_ws(const GemmTask<float>* d, int nTasks, int tiles, int* dErr, cudaStream_t s) {
  constexpr int smem = NS * (2 * TC_BM * 128 + 2 * BN * 128) + 1024;
  static_assert(smem <= 227 * 1024, "stages exceed shared memory");
  static std::once_flag once;
  std::call_once(once, [] {
    RSCHOL_CUDA(cudaFuncSetAttribute(gemm_tc_kernel<BN, NS, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  });
  gemm_tc_kernel<BN, NS, BF><<<tiles, WS_THREADS, smem, s>>>(d, nTasks, dErr);
  RSCHOL_LAUNCH_CHECK();
}

void launch_gemm_tc(const GemmTask<float>* d, int nTasks, int tiles, int* dErr, cudaStream_t s, int bn, int bf16) {
  if (nTasks <= 0 || tiles <= 0) return;
  if (bf16) {
    if (bn > 64) launch_ws<128, 3, true>(d, nTasks, tiles, dErr, s);
    else launch_ws<64, 4, true>(d, nTasks, tiles, dErr, s);
  } else {
    if (bn > 64) launch_ws<128, 3, false>(d, nTasks, tiles, dErr, s);
    else launch_ws<64, 4, false>(d, nTasks, tiles, dErr, s);
  }
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    const char* e = std::getenv("RSCHOL_TMA");
    if (e && e[0] == '0') return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  }();
  return fn;
}

// The map of a K-major operand: `rows` rows of K floats, row stride ld
// floats; boxes of 32 K x boxRows rows in the 128-byte swizzle (the layout the
// MMA's shared-memory descriptors read); zeros beyond K and rows.
bool encode_operand(PFN_cuTensorMapEncodeTiled_v12000 enc, TensorMapBytes& out, const float* base, int rows, int K,
                    int ld, int boxRows) {
  static_assert(sizeof(TensorMapBytes) == sizeof(CUtensorMap), "tensor map size");
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * sizeof(float)};
  const cuuint32_t box[2] = {32u, (cuuint32_t)boxRows};
  const cuuint32_t estr[2] = {1u, 1u};
  CUtensorMap m;
  const CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  std::memcpy(out.b, &m, sizeof(m));
  return true;
}

}  // namespace

int encode_gemm_tmaps(GemmTask<float>* tasks, int count, int bn, std::vector<TensorMapBytes>& maps) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return 0;
  int got = 0;
  for (int q = 0; q < count; ++q) {
    GemmTask<float>& t = tasks[q];
    t.tmA = t.tmB = nullptr;
    const bool aligned = ((reinterpret_cast<uintptr_t>(t.A) | reinterpret_cast<uintptr_t>(t.B)) & 15u) == 0 &&
                         (t.lda & 3) == 0 && (t.ldb & 3) == 0;
    if (t.tA || !t.tB || !aligned || t.M <= 0 || t.N <= 0 || t.K <= 0) continue;
    TensorMapBytes a, b;
    if (!encode_operand(enc, a, t.A, t.M, t.K, t.lda, TC_BM) || !encode_operand(enc, b, t.B, t.N, t.K, t.ldb, bn))
      continue;
    maps.push_back(a);
    t.tmA = reinterpret_cast<const void*>((uintptr_t)maps.size());
    maps.push_back(b);
    t.tmB = reinterpret_cast<const void*>((uintptr_t)maps.size());
    ++got;
  }
  return got;
}

void launch_gemm_splitk_reduce(const GemmTask<float>* d, const int* ids, int nIds, const long long* elemBase,
                               long long elems, cudaStream_t s) {
  if (nIds <= 0 || elems <= 0) return;
  gemm_splitk_reduce<<<(unsigned)((elems + 255) / 256), 256, 0, s>>>(d, ids, nIds, elemBase);
  RSCHOL_LAUNCH_CHECK();
}

}  // namespace rschol
