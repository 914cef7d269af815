// Shared CUDA helpers for the GB300 factor / solve / PCG kernels.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>

namespace rschol {

// RSCHOL_PLAN_TRACE=1: the host seconds of each planning phase, one line on
// stderr per plan (the phases between successive mark() calls).
struct PlanClock {
  bool on = false;
  std::chrono::steady_clock::time_point t;
  std::string line;
  explicit PlanClock(const char* what) {
    const char* e = std::getenv("RSCHOL_PLAN_TRACE");
    on = e && e[0] == '1';
    if (on) {
      line = what;
      t = std::chrono::steady_clock::now();
    }
  }
  void mark(const char* phase) {
    if (!on) return;
    const auto u = std::chrono::steady_clock::now();
    line += std::string(" ") + phase + " " + std::to_string(std::chrono::duration<double>(u - t).count());
    t = u;
  }
  ~PlanClock() {
    if (on) std::fprintf(stderr, "%s\n", line.c_str());
  }
};

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

// A bounded wait inside a factorisation kernel (a fused-Cholesky tile
// counter or a tensor-core mbarrier) gave up: the kernel returned early and
// the factor is invalid, but the context stays usable.
struct FactorWaitTimeout : CudaError {
  explicit FactorWaitTimeout(const std::string& s) : CudaError(s) {}
};

#define RSCHOL_CUDA(call)                                                                          \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      throw ::rschol::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + " at " +      \
                                __FILE__ + ":" + std::to_string(__LINE__));                        \
  } while (0)

#define RSCHOL_LAUNCH_CHECK() RSCHOL_CUDA(cudaGetLastError())

// Programmatic dependent launch.  A kernel launched with launch_k may start
// while the previous kernel on the stream drains: it first lets its own
// successor launch, then waits until its predecessor has completed and its
// writes are visible (griddepcontrol), so every kernel so launched must call
// pdl_enter() before it touches memory.  (A successor grid launches only after
// every block of its predecessor has started, so waiting blocks never keep a
// predecessor's blocks off the SMs.)  Both instructions are no-ops for a
// kernel launched without the attribute.  RSCHOL_PDL=0 turns it off.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

bool pdl_enabled();

template <class... KArgs, class... Args>
void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  RSCHOL_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// Live device bytes are charged to the account current on the allocating
// thread (each factor has one, made current by its entry points) and credited
// back to the same account on release, from whichever thread releases.
extern thread_local std::atomic<long long>* g_devAccount;

struct AccountScope {
  std::atomic<long long>* prev;
  explicit AccountScope(std::atomic<long long>* a) : prev(g_devAccount) { g_devAccount = a; }
  ~AccountScope() { g_devAccount = prev; }
  AccountScope(const AccountScope&) = delete;
  AccountScope& operator=(const AccountScope&) = delete;
};

// Device allocation owned by the host object that created it.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  std::atomic<long long>* acct = nullptr;   // the account charged for these bytes
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes), acct(o.acct) {
    o.p = nullptr;
    o.bytes = 0;
    o.acct = nullptr;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      acct = o.acct;
      o.p = nullptr;
      o.bytes = 0;
      o.acct = nullptr;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t b) {
    release();
    if (b == 0) return;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      p = nullptr;
      throw CudaError(std::string("cudaMalloc(") + std::to_string(b) + "): " + cudaGetErrorString(e));
    }
    bytes = b;
    acct = g_devAccount;
    if (acct) acct->fetch_add((long long)b);
  }
  void release() {
    if (p) {
      cudaFree(p);
      if (acct) acct->fetch_sub((long long)bytes);
    }
    p = nullptr;
    bytes = 0;
    acct = nullptr;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

}  // namespace rschol
