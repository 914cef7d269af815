// Device helpers shared by the single-vector and batched solves: warp
// reductions, bounded inter-block waits, and the ticket / completion counter
// layout of the interior launches.
#pragma once
#include <cuda_runtime.h>

namespace rschol {
namespace solvedev {

constexpr unsigned FULL = 0xffffffffu;

template <class V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

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

// Warp-uniform bounded wait for *p >= target.  Returns false when the wait
// gave up (after `limit` polls, or as soon as another block reported an
// error); the error word is then set.
__device__ __forceinline__ bool wait_geq(const int* p, int target, int* err, int limit = SPIN_LIMIT) {
  if (__all_sync(FULL, ld_acquire(p) >= target)) return true;
  for (int it = 1; it <= limit; ++it) {
    __nanosleep(64);
    if (__all_sync(FULL, ld_acquire(p) >= target)) return true;
    if ((it & 63) == 0 && __any_sync(FULL, ld_volatile(err) != 0)) return false;
  }
  if ((threadIdx.x & 31) == 0) atomicExch(err, 1);
  return false;
}

// Same, with the poll limit read from *limitP only once the first poll has
// failed (the fast path adds no dependent load to the caller's critical path).
__device__ __forceinline__ bool wait_geq_lim(const int* p, int target, int* err, const int* limitP) {
  if (__all_sync(FULL, ld_acquire(p) >= target)) return true;
  return wait_geq(p, target, err, __ldcg(limitP));
}

// Every block of a ticketed launch calls this once when it is done; the last
// one resets the ticket and completion counters for the next launch.
__device__ __forceinline__ void launch_done(int* tick, int* done) {
  __syncthreads();
  if (threadIdx.x == 0 && atomicAdd(done, 1) == (int)gridDim.x - 1) {
    atomicExch(tick, 0);
    atomicExch(done, 0);
  }
}

constexpr int ICH = 128;   // off-diagonal rows per interior chunk block
constexpr int SYNC_TICK_F = 1, SYNC_DONE_F = 2, SYNC_TICK_B = 3, SYNC_DONE_B = 4, SYNC_GLOBAL = 5;

}  // namespace solvedev
}  // namespace rschol
