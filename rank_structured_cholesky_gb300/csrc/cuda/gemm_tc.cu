// Batched FP32 GEMM on the 5th-generation tensor cores (tcgen05, kind::tf32).
//
// Same task semantics as the SIMT gemm_kernel (C = alpha op(A) op(B) +
// beta C, row-major, per-task shapes; lower tasks skip tiles above the
// diagonal), one 128 x 64 output tile (and K slice) per CTA.  Operands are
// staged by the CTA's threads into shared memory in the K-major 128-byte
// swizzled layout (a row of 32 TF32 per 128 bytes, 16-byte chunks XORed with
// the row index: coalesced global loads and conflict-free stores), rounded to
// TF32; one thread issues tcgen05.mma (M = 128, N = 64, K = 8) into a TMEM
// accumulator and commits to an mbarrier per stage (two stages: loads of
// stage k+1 overlap the MMAs of stage k); the epilogue reads TMEM with
// tcgen05.ld and writes C through shared memory in coalesced rows.  Tasks
// with a large K and few tiles are split along K (kSplit slices write FP32
// partials to a workspace; gemm_splitk_reduce sums them in slice order).
//
// Split precision (task.split != 0): a = a_hi + a_lo with a_hi = tf32(a),
// a_lo = tf32(a - a_hi), and A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi (three
// MMAs per K step, FP32 accuracy up to the dropped A_lo B_lo term), for the
// Schur-complement updates whose errors the factor cannot absorb.
#include <cstdint>
#include <mutex>

#include "common.cuh"
#include "dense.cuh"

namespace rschol {

namespace {

constexpr int TC_BM = 128, TC_BN = 64, TC_BK = 32, TC_THREADS = 128, TC_STAGES = 2;
constexpr int TC_A_BYTES = TC_BM * TC_BK * 4;            // 16 KB per A tile (hi or lo)
constexpr int TC_B_BYTES = TC_BN * TC_BK * 4;            // 8 KB per B tile
constexpr int TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024;   // + alignment of the stage base
constexpr int TC_TMEM_COLS = 64;
constexpr int TC_SPIN_LIMIT = 1 << 22;

// Byte offset of element (r, k) of a K-major operand tile in the 128-byte
// swizzled layout: row r occupies 128 bytes (32 TF32) of an 8-row, 1024-byte
// atom; its 16-byte chunk c is stored at chunk c ^ (r & 7).
__device__ __forceinline__ uint32_t tc_off(int r, int k) {
  return (uint32_t)(((r >> 3) << 10) + ((r & 7) << 7) + ((((k >> 2) ^ (r & 7)) & 7) << 4) + ((k & 3) << 2));
}

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);            // start address (advances 32 B per K = 8)
  d |= (uint64_t)1 << 16;                             // leading byte offset (unused within a 128 B row)
  d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;      // stride byte offset: next 8-row atom
  d |= (uint64_t)1 << 46;                             // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                             // 128-byte swizzle (atoms 1024-byte aligned)
  return d;
}

// Instruction descriptor: D f32, A and B tf32, both K-major, M = 128, N = 64.
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TC_BN >> 3) << 17) |
                              ((uint32_t)(TC_BM >> 4) << 24);

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// 16-byte asynchronous copy global -> shared; bytes < 16 zero-fills the rest
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(addr), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the mbarrier phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
  for (int it = 0; it < TC_SPIN_LIMIT; ++it)
    if (mbar_try_wait(addr, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__global__ void __launch_bounds__(TC_THREADS) gemm_tc_kernel(const GemmTask<float>* __restrict__ tasks, int nTasks,
                                                             int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t mbar[TC_STAGES];
  __shared__ uint32_t tmemBase;
  __shared__ int sAbort;
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
  const int row0 = ti * TC_BM, col0 = tj * TC_BN;
  if (t.lower && row0 + TC_BM - 1 < col0) return;   // uniform over the block, before any allocation
  const int kl = t.kLen > 0 ? t.kLen : t.K;
  const int kBeg = slice * kl, kEnd = min(t.K, kBeg + kl);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool split = t.split != 0;
  const uint32_t sraw = (uint32_t)__cvta_generic_to_shared(tc_smem);
  const uint32_t sbase = (sraw + 1023u) & ~1023u;
  auto aHi = [&](int st) { return sbase + (uint32_t)(st * TC_STAGE_BYTES); };
  auto aLo = [&](int st) { return aHi(st) + TC_A_BYTES; };
  auto bHi = [&](int st) { return aHi(st) + 2 * TC_A_BYTES; };
  auto bLo = [&](int st) { return bHi(st) + TC_B_BYTES; };
  const uint32_t mb0 = (uint32_t)__cvta_generic_to_shared(&mbar[0]);

  if (warp == 0) {
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tmemBase);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int st = 0; st < TC_STAGES; ++st) mbar_init(mb0 + 8u * st, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sAbort = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;

  const int nk = kEnd > kBeg ? (kEnd - kBeg + TC_BK - 1) / TC_BK : 0;
  // Operand tiles go global -> registers (all loads of a tile in flight at
  // once, issued while the previous tile's MMAs run) -> shared.
  float ra[TC_BM * TC_BK / TC_THREADS], rb[TC_BN * TC_BK / TC_THREADS];
  auto load_tiles = [&](int k0) {
#pragma unroll
    for (int q = 0; q < TC_BM * TC_BK / TC_THREADS; ++q) {
      const int idx = tid + q * TC_THREADS;
      int m, k;
      if (!t.tA) { m = idx >> 5; k = idx & 31; }
      else { m = idx & 127; k = idx >> 7; }
      const int gm = row0 + m, gk = k0 + k;
      ra[q] = (gm < t.M && gk < kEnd) ? (t.tA ? t.A[(size_t)gk * t.lda + gm] : t.A[(size_t)gm * t.lda + gk]) : 0.f;
    }
#pragma unroll
    for (int q = 0; q < TC_BN * TC_BK / TC_THREADS; ++q) {
      const int idx = tid + q * TC_THREADS;
      int n, k;
      if (!t.tB) { n = idx & 63; k = idx >> 6; }
      else { n = idx >> 5; k = idx & 31; }
      const int gn = col0 + n, gk = k0 + k;
      rb[q] = (gn < t.N && gk < kEnd) ? (t.tB ? t.B[(size_t)gn * t.ldb + gk] : t.B[(size_t)gk * t.ldb + gn]) : 0.f;
    }
  };
  auto store_tiles = [&](int st) {
    unsigned char* base = tc_smem + (sbase - sraw) + (size_t)st * TC_STAGE_BYTES;
#pragma unroll
    for (int q = 0; q < TC_BM * TC_BK / TC_THREADS; ++q) {
      const int idx = tid + q * TC_THREADS;
      int m, k;
      if (!t.tA) { m = idx >> 5; k = idx & 31; }
      else { m = idx & 127; k = idx >> 7; }
      const uint32_t off = tc_off(m, k), h = to_tf32(ra[q]);
      *reinterpret_cast<uint32_t*>(base + off) = h;
      if (split) *reinterpret_cast<uint32_t*>(base + TC_A_BYTES + off) = to_tf32(ra[q] - __uint_as_float(h));
    }
#pragma unroll
    for (int q = 0; q < TC_BN * TC_BK / TC_THREADS; ++q) {
      const int idx = tid + q * TC_THREADS;
      int n, k;
      if (!t.tB) { n = idx & 63; k = idx >> 6; }
      else { n = idx >> 5; k = idx & 31; }
      const uint32_t off = tc_off(n, k), h = to_tf32(rb[q]);
      *reinterpret_cast<uint32_t*>(base + 2 * TC_A_BYTES + off) = h;
      if (split)
        *reinterpret_cast<uint32_t*>(base + 2 * TC_A_BYTES + TC_B_BYTES + off) = to_tf32(rb[q] - __uint_as_float(h));
    }
  };
  // MMAs of one staged K tile (issued by thread 0), then a commit to the
  // stage's barrier
  auto mma_stage = [&](int st, int kt) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
    for (int kk = 0; kk < TC_BK / 8; ++kk) {
      const uint32_t step = (uint32_t)kk * 32u;   // 8 TF32 = 32 bytes along the swizzled row
      const uint32_t acc = (kt > 0 || kk > 0) ? 1u : 0u;
      tc_mma(tmem, tc_smem_desc(aHi(st) + step), tc_smem_desc(bHi(st) + step), acc);
      if (split) {
        tc_mma(tmem, tc_smem_desc(aHi(st) + step), tc_smem_desc(bLo(st) + step), 1u);
        tc_mma(tmem, tc_smem_desc(aLo(st) + step), tc_smem_desc(bHi(st) + step), 1u);
      }
    }
    tc_commit(mb0 + 8u * st);
  };
  // Async path: A row-major (K contiguous) and B stored N x K, both 16-byte
  // aligned with leading dimensions that keep every 4-float chunk aligned.
  // The tiles arrive by 16-byte cp.async straight into the swizzled layout
  // (the 128-byte swizzle permutes whole 16-byte chunks), the next tile in
  // flight while the current one is converted and multiplied; the TF32
  // rounding (and the split's low parts) is a linear pass over the stage.
  const bool fast = !t.tA && t.tB &&
                    ((reinterpret_cast<uintptr_t>(t.A) | reinterpret_cast<uintptr_t>(t.B)) & 15u) == 0 &&
                    (t.lda & 3) == 0 && (t.ldb & 3) == 0;
  auto issue_async = [&](int k0, int st) {
    const uint32_t a0 = aHi(st), b0 = bHi(st);
    for (int c = tid; c < TC_BM * (TC_BK / 4); c += TC_THREADS) {
      const int r = c >> 3, ch = c & 7;
      const int gm = row0 + r, gk = k0 + 4 * ch;
      const int valid = gm < t.M ? max(0, min(4, kEnd - gk)) : 0;
      const float* src = valid > 0 ? t.A + (size_t)gm * t.lda + gk : t.A;
      cp_async16(a0 + tc_off(r, 4 * ch), src, 4 * valid);
    }
    for (int c = tid; c < TC_BN * (TC_BK / 4); c += TC_THREADS) {
      const int r = c >> 3, ch = c & 7;
      const int gn = col0 + r, gk = k0 + 4 * ch;
      const int valid = gn < t.N ? max(0, min(4, kEnd - gk)) : 0;
      const float* src = valid > 0 ? t.B + (size_t)gn * t.ldb + gk : t.B;
      cp_async16(b0 + tc_off(r, 4 * ch), src, 4 * valid);
    }
    cp_async_commit();
  };
  auto convert_stage = [&](int st) {
    unsigned char* base = tc_smem + (sbase - sraw) + (size_t)st * TC_STAGE_BYTES;
    auto conv = [&](unsigned char* hiB, unsigned char* loB, int words) {
      for (int w = tid; w < words / 4; w += TC_THREADS) {
        float4* hp = reinterpret_cast<float4*>(hiB) + w;
        const float4 v = *hp;
        float4 h, l;
        h.x = __uint_as_float(to_tf32(v.x));
        h.y = __uint_as_float(to_tf32(v.y));
        h.z = __uint_as_float(to_tf32(v.z));
        h.w = __uint_as_float(to_tf32(v.w));
        *hp = h;
        if (split) {
          l.x = __uint_as_float(to_tf32(v.x - h.x));
          l.y = __uint_as_float(to_tf32(v.y - h.y));
          l.z = __uint_as_float(to_tf32(v.z - h.z));
          l.w = __uint_as_float(to_tf32(v.w - h.w));
          *(reinterpret_cast<float4*>(loB) + w) = l;
        }
      }
    };
    conv(base, base + TC_A_BYTES, TC_BM * TC_BK);
    conv(base + 2 * TC_A_BYTES, base + 2 * TC_A_BYTES + TC_B_BYTES, TC_BN * TC_BK);
  };
  uint32_t parity[TC_STAGES] = {0u, 0u};
  int issued = 0;   // k tiles whose MMAs were committed
  if (fast) {
    if (nk > 0) issue_async(kBeg, 0);
    for (int kt = 0; kt < nk; ++kt) {
      const int st = kt & 1;
      if (kt + 1 < nk) {
        if (kt >= 1) {   // stage st ^ 1 held tile kt - 1: its MMAs must be done before it is refilled
          if (tid == 0 && !mbar_wait(mb0 + 8u * (st ^ 1), parity[st ^ 1])) {
            atomicExch(err, 1);
            sAbort = 1;
          }
          parity[st ^ 1] ^= 1u;
        }
        __syncthreads();
        if (sAbort) break;
        issue_async(kBeg + (kt + 1) * TC_BK, st ^ 1);
        cp_async_wait<1>();   // tile kt has landed (kt + 1 may still be in flight)
      } else {
        cp_async_wait<0>();
      }
      __syncthreads();
      convert_stage(st);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) mma_stage(st, kt);
      issued = kt + 1;
    }
    cp_async_wait<0>();   // nothing of this CTA stays in flight
  }
  if (!fast) {
  if (nk > 0) load_tiles(kBeg);
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt & 1;
    if (kt >= TC_STAGES) {   // the MMAs of tile kt - 2 must be done with stage st
      if (tid == 0 && !mbar_wait(mb0 + 8u * st, parity[st])) {
        atomicExch(err, 1);
        sAbort = 1;
      }
      parity[st] ^= 1u;
    }
    __syncthreads();
    if (sAbort) break;
    store_tiles(st);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) mma_stage(st, kt);
    issued = kt + 1;
    if (kt + 1 < nk) load_tiles(kBeg + (kt + 1) * TC_BK);
  }
  }
  // The last commit completes after every earlier MMA of this thread.
  if (tid == 0 && issued > 0) {
    const int st = (issued - 1) & 1;
    if (!mbar_wait(mb0 + 8u * st, parity[st])) {
      atomicExch(err, 1);
      sAbort = 1;
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (!sAbort) {
    // TMEM -> registers (row 32 w + lane, 64 columns) -> shared [128][65]
    float* buf = reinterpret_cast<float*>(tc_smem + (sbase - sraw));
    if (issued > 0) {
      uint32_t r[64];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
          "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
          "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, "
          "%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, "
          "%48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
            "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
            "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
            "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
            "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      float* row = buf + (warp * 32 + lane) * (TC_BN + 1);
#pragma unroll
      for (int c = 0; c < 64; ++c) row[c] = __uint_as_float(r[c]);
    } else {
      float* row = buf + (warp * 32 + lane) * (TC_BN + 1);
      for (int c = 0; c < 64; ++c) row[c] = 0.f;
    }
    __syncthreads();
    // coalesced write-out: a warp per row, lanes over columns
    if (t.kSplit > 1) {
      float* part = t.ws + ((size_t)slice * tilesPer + tl) * (TC_BM * TC_BN);
      for (int i = warp; i < TC_BM; i += TC_THREADS / 32)
        for (int c = lane; c < TC_BN; c += 32) part[i * TC_BN + c] = buf[i * (TC_BN + 1) + c];
    } else {
      for (int i = warp; i < TC_BM; i += TC_THREADS / 32) {
        const int gm = row0 + i;
        if (gm >= t.M) break;
        float* crow = t.C + (size_t)gm * t.ldc;
        for (int c = lane; c < TC_BN; c += 32) {
          const int gn = col0 + c;
          if (gn < t.N) {
            float v = t.alpha * buf[i * (TC_BN + 1) + c];
            if (t.beta != 0.f) v = fmaf(t.beta, crow[gn], v);
            crow[gn] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
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
  const int tilesPer = ((t.M + TC_BM - 1) / TC_BM) * t.tilesN;
  const int tl = (i / TC_BM) * t.tilesN + j / TC_BN;
  const int off = (i % TC_BM) * TC_BN + (j % TC_BN);
  float s = 0.f;
  for (int sl = 0; sl < t.kSplit; ++sl) s += t.ws[((size_t)sl * tilesPer + tl) * (TC_BM * TC_BN) + off];
  float* c = t.C + (size_t)i * t.ldc + j;
  float v = t.alpha * s;
  if (t.beta != 0.f) v = fmaf(t.beta, *c, v);
  *c = v;
}

}  // namespace

void launch_gemm_tc(const GemmTask<float>* d, int nTasks, int tiles, int* dErr, cudaStream_t s) {
  if (nTasks <= 0 || tiles <= 0) return;
  static std::once_flag once;
  std::call_once(once, [] {
    RSCHOL_CUDA(cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
  });
  gemm_tc_kernel<<<tiles, TC_THREADS, TC_SMEM, s>>>(d, nTasks, dErr);
  RSCHOL_LAUNCH_CHECK();
}

void launch_gemm_splitk_reduce(const GemmTask<float>* d, const int* ids, int nIds, const long long* elemBase,
                               long long elems, cudaStream_t s) {
  if (nIds <= 0 || elems <= 0) return;
  gemm_splitk_reduce<<<(unsigned)((elems + 255) / 256), 256, 0, s>>>(d, ids, nIds, elemBase);
  RSCHOL_LAUNCH_CHECK();
}

}  // namespace rschol
