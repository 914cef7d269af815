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

// The loops below give every (row, right-hand side) pair to one thread,
// pairs numbered row-major (p = row * k + c) across the block, and form each
// pair's dot product serially in a fixed order: every column's arithmetic is
// the same whatever k is, all threads have work even at k = 1, and for wide
// blocks consecutive threads take consecutive columns of one row.

// f := L^{-1} f for k right-hand sides (f: n x k in shared memory, row
// stride k) with the inverted 64 x 64 diagonal blocks of L; t: 64 x k
// shared.
template <class T>
__device__ void trsv_dinv_k(const T* __restrict__ L, int ld, int n, const T* __restrict__ D, T* f, T* t, int k) {
  for (int i0 = 0; i0 < n; i0 += 64) {
    const int h = min(64, n - i0);
    for (int p = threadIdx.x; p < h * k; p += blockDim.x) {
      const int i = p / k, c = p - i * k;
      const T* row = L + (size_t)(i0 + i) * ld;
      T s = f[(size_t)(i0 + i) * k + c];
      for (int j = 0; j < i0; ++j) s -= row[j] * f[(size_t)j * k + c];
      t[(size_t)i * k + c] = s;
    }
    __syncthreads();
    const T* Db = D + (size_t)i0 * 64;
    for (int p = threadIdx.x; p < h * k; p += blockDim.x) {
      const int i = p / k, c = p - i * k;
      const T* row = Db + (size_t)i * h;
      T s = T(0);
      for (int j = 0; j <= i; ++j) s += row[j] * t[(size_t)j * k + c];
      f[(size_t)(i0 + i) * k + c] = s;
    }
    __syncthreads();
  }
}

// f := L^{-T} f for k right-hand sides, same blocks.
template <class T>
__device__ void trsv_dinv_t_k(const T* __restrict__ L, int ld, int n, const T* __restrict__ D, T* f, T* t, int k) {
  if (n <= 0) return;
  for (int i0 = ((n - 1) / 64) * 64; i0 >= 0; i0 -= 64) {
    const int h = min(64, n - i0);
    for (int p = threadIdx.x; p < h * k; p += blockDim.x) {
      const int j = p / k, c = p - j * k;
      T s = f[(size_t)(i0 + j) * k + c];
      for (int i = i0 + h; i < n; ++i) s -= L[(size_t)i * ld + i0 + j] * f[(size_t)i * k + c];
      t[(size_t)j * k + c] = s;
    }
    __syncthreads();
    const T* Db = D + (size_t)i0 * 64;
    for (int p = threadIdx.x; p < h * k; p += blockDim.x) {
      const int j = p / k, c = p - j * k;
      T s = T(0);
      for (int i = j; i < h; ++i) s += Db[(size_t)i * h + j] * t[(size_t)i * k + c];
      f[(size_t)(i0 + j) * k + c] = s;
    }
    __syncthreads();
  }
}

template <class T>
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
  trsv_dinv_k<T>(nd.L, nd.ld, n, nd.Dinv, f, t, k);
  if (wk.b == 0)
    for (int idx = threadIdx.x; idx < n * k; idx += blockDim.x) yout[(size_t)nd.c0 * k + idx] = f[idx];
  // wud[a][c] -= L21[a] . y[:, c], a thread per (row, column)
  for (int p = threadIdx.x; p < (a1 - a0) * k; p += blockDim.x) {
    const int a = a0 + p / k, c = p % k;
    const T* row = nd.L + (size_t)(n + a) * nd.ld;
    T s = T(0);
    for (int j = 0; j < n; ++j) s += row[j] * f[(size_t)j * k + c];
    wud[(size_t)a * k + c] -= s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(sync + nd.syncOff + 1, 1);
  }
  launch_done(&sync[SYNC_TICK_F], &sync[SYNC_DONE_F]);
}

template <class T>
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
    // part[j][c] = sum_{a in chunk} L21[a][j] x_{rows[a]}[c], a thread per (j, column)
    const int* rw = rows + nd.rowsOff;
    const T* L21 = nd.L + (size_t)n * nd.ld;
    T* part = ipart + (nd.zpOff + (size_t)wk.b * n) * k;
    for (int p = threadIdx.x; p < n * k; p += blockDim.x) {
      const int j = p / k, c = p - j * k;
      T s = T(0);
      for (int a = a0; a < a1; ++a) s += L21[(size_t)a * nd.ld + j] * __ldcg(w + (size_t)rw[a] * k + c);
      part[(size_t)j * k + c] = s;
    }
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
  trsv_dinv_t_k<T>(nd.L, nd.ld, n, nd.Dinv, f, t, k);
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
__global__ void convert_k_kernel(const A* __restrict__ src, B* __restrict__ dst, long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (B)src[i];
}

}  // namespace

template <class T>
int SolveEngine<T>::batch_capacity() const {
  const size_t per = sizeof(T) * (size_t)(maxNI_ + 64);
  const int bySmem = (int)std::min<size_t>(64, (200 * 1024) / std::max<size_t>(per, 1));
  return std::max(1, bySmem);
}

template <class T>
void SolveEngine<T>::plan_batch(int k) {
  if (k == kB_) return;
  const Symbolic& S = F_.S;
  cudaStream_t st = F_.stream;
  if (k > kAllocB_) {
    dWuB_.alloc(sizeof(T) * std::max(1LL, wuTotal_ * k));
    dYB_.alloc(sizeof(T) * std::max<long long>(1, (long long)S.n * k));
    dIpB_.alloc(sizeof(T) * std::max(1LL, ipTotal_ * k));
    if (!dSyncB_.p) {
      dSyncB_.alloc(sizeof(int) * syncInts_);
      RSCHOL_CUDA(cudaMemsetAsync(dSyncB_.p, 0, sizeof(int) * syncInts_, st));
      epochB_ = 0;
    }
    dWB_.alloc(sizeof(T) * std::max<long long>(1, (long long)S.n * k));   // the working copy of W
    kAllocB_ = k;
    bPlans_.clear();   // the task lists point into the old buffers
  }
  auto found = bPlans_.find(k);
  if (found != bPlans_.end()) {
    bPlan_ = &found->second;
    kB_ = k;
    return;
  }
  BatchPlan& plan = bPlans_[k];
  // batched GEMMs of the compressed levels
  const bool tc = std::is_same<T, float>::value && F_.tensor_cores();
  std::vector<GemmTask<T>> tasks;
  auto& steps = plan.steps;
  steps.assign(6 * cLevels_.size(), {});
  T* wu = dWuB_.as<T>();
  T* yb = dYB_.as<T>();
  T* w = dWB_.as<T>();
  auto mk = [&](const T* A, int lda, bool tA, const T* B, int ldb, T* C, int ldc, int M, int N, int K, T alpha,
                T beta) {
    GemmTask<T> g{};
    g.A = A;
    g.B = B;
    g.C = C;
    g.M = M;
    g.N = N;
    g.K = K;
    g.lda = lda;
    g.ldb = ldb;
    g.ldc = ldc;
    g.tA = tA;
    g.tB = 0;
    g.alpha = alpha;
    g.beta = beta;
    g.tilesN = (N + 63) / 64;
    g.split = 1;
    g.kSplit = 1;
    g.kLen = K;
    return g;
  };
  // K slicing: tasks with K above kSliceMin run as slices of kSlice
  constexpr int kSlice = 512, kSliceMin = 768;
  std::vector<SliceSum<T>> sums;
  std::vector<std::pair<size_t, long long>> taskWs;   // (task, workspace offset) to patch
  std::vector<std::pair<size_t, long long>> sumWs;    // (sum, workspace offset) to patch
  long long wsTotal = 0;
  auto flush = [&](std::vector<GemmTask<T>>& batch, int slot) {
    if (batch.empty()) return;
    int maxK = 0;
    for (auto& g : batch) maxK = std::max(maxK, g.K);
    const bool useTc = tc && maxK >= 128;
    const int rpt = useTc ? 128 : 64;
    std::vector<GemmTask<T>> run;
    const long long sum0 = (long long)sums.size();
    long long maxMN = 0, wsStep = 0;
    for (const GemmTask<T>& g : batch) {
      if (g.K <= kSliceMin) {
        run.push_back(g);
        continue;
      }
      const int ns = (g.K + kSlice - 1) / kSlice;
      const long long mn = (long long)g.M * g.N;
      SliceSum<T> sm{g.C, nullptr, g.ldc, g.M, g.N, ns, g.alpha, g.beta};
      sumWs.push_back({sums.size(), wsStep});
      sums.push_back(sm);
      for (int q = 0; q < ns; ++q) {
        GemmTask<T> t = g;
        t.K = std::min(kSlice, g.K - q * kSlice);
        t.kLen = t.K;
        t.A = g.tA ? g.A + (size_t)q * kSlice * g.lda : g.A + (size_t)q * kSlice;
        t.B = g.B + (size_t)q * kSlice * g.ldb;
        t.C = nullptr;
        t.ldc = g.N;
        t.alpha = T(1);
        t.beta = T(0);
        t.lower = 0;
        taskWs.push_back({tasks.size() + run.size(), wsStep + q * mn});
        run.push_back(t);
      }
      wsStep += ns * mn;
      maxMN = std::max(maxMN, mn);
    }
    // every step's slice products start at the workspace base: steps run in stream order
    wsTotal = std::max(wsTotal, wsStep);
    int tiles = 0;
    for (auto& g : run) {
      g.tileBase = tiles;
      tiles += ((g.M + rpt - 1) / rpt) * g.tilesN;
    }
    XStep xs{(long long)tasks.size(), (int)run.size(), tiles, useTc ? 1 : 0};
    xs.redOff = sum0;
    xs.redCount = (int)(sums.size() - sum0);
    xs.redGrid = (int)std::min<long long>(64, (maxMN + 255) / 256);
    steps[slot].push_back(xs);
    tasks.insert(tasks.end(), run.begin(), run.end());
    batch.clear();
  };
  const int L = (int)cLevels_.size();
  for (int l = 0; l < L; ++l) {
    std::vector<GemmTask<T>> gy, gz, gu, gs, gg, gx;
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
  plan.tasks.alloc(std::max<size_t>(16, tasks.size() * sizeof(GemmTask<T>)));
  if (!tasks.empty())
    RSCHOL_CUDA(cudaMemcpyAsync(plan.tasks.p, tasks.data(), tasks.size() * sizeof(GemmTask<T>),
                                cudaMemcpyHostToDevice, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  bPlan_ = &plan;
  kB_ = k;
}

template <class T>
void SolveEngine<T>::apply_batch(double* W64, int k, cudaStream_t st) {
  if (k <= 0) return;
  if (k > batch_capacity()) throw std::runtime_error("apply_batch: more right-hand sides than one pass handles");
  plan_batch(k);
  const int n = F_.S.n;
  const long long nk = (long long)n * k;
  T* w = dWB_.as<T>();
  convert_k_kernel<double, T><<<(unsigned)std::min<long long>((nk + 255) / 256, 4096), 256, 0, st>>>(W64, w, nk);
  RSCHOL_LAUNCH_CHECK();
  if (++epochB_ >= (1 << 24)) {
    RSCHOL_CUDA(cudaMemsetAsync(dSyncB_.p, 0, sizeof(int) * syncInts_, st));
    epochB_ = 1;
  }
  int* sync = dSyncB_.as<int>();
  const size_t smem = sizeof(T) * (size_t)(maxNI_ + 64) * k;
  static std::once_flag once;
  std::call_once(once, [] {
    RSCHOL_CUDA(cudaFuncSetAttribute(interior_forward_k<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    RSCHOL_CUDA(cudaFuncSetAttribute(interior_backward_k<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  });
  if (nIWork_ > 0) {
    interior_forward_k<T><<<nIWork_, 256, smem, st>>>(dNodes_.as<SNode<T>>(), dIWork_.as<RowBlock>(), dRel_.as<int>(),
                                                       dChild_.as<int>(), sync, epochB_, k, w, dYB_.as<T>(),
                                                       dWuB_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  const int* lvl = dLevelNodes_.as<int>();
  const GemmTask<T>* bg = bPlan_->tasks.template as<GemmTask<T>>();
  auto gemm = [&](int slot) {
    for (const XStep& x : bPlan_->steps[slot]) {
      if constexpr (std::is_same<T, float>::value) {
        if (x.tc) launch_gemm_tc(bg + x.off, x.count, x.tiles, F_.dFlag.template as<int>() + 1, st);
        else launch_gemm<T>(bg + x.off, x.count, x.tiles, st);
      } else {
        launch_gemm<T>(bg + x.off, x.count, x.tiles, st);
      }
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
    interior_backward_k<T><<<nIWork_, 256, smem, st>>>(dNodes_.as<SNode<T>>(), dIWorkB_.as<RowBlock>(),
                                                        dRows_.as<int>(), sync, epochB_, k, dIpB_.as<T>(),
                                                        dYB_.as<T>(), w);
    RSCHOL_LAUNCH_CHECK();
  }
  convert_k_kernel<T, double><<<(unsigned)std::min<long long>((nk + 255) / 256, 4096), 256, 0, st>>>(w, W64, nk);
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
    epochB_ = 0;
  }
  return e;
}

template int SolveEngine<double>::batch_capacity() const;
template int SolveEngine<float>::batch_capacity() const;
template void SolveEngine<double>::plan_batch(int);
template void SolveEngine<float>::plan_batch(int);
template void SolveEngine<double>::apply_batch(double*, int, cudaStream_t);
template void SolveEngine<float>::apply_batch(double*, int, cudaStream_t);
template int SolveEngine<double>::take_error_batch(cudaStream_t);
template int SolveEngine<float>::take_error_batch(cudaStream_t);

}  // namespace rschol
