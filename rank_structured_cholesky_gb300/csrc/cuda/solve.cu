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

template <class T>
__global__ void __launch_bounds__(1024) compressed_forward_kernel(const SNode<T>* __restrict__ nodes,
                                                                  const int* __restrict__ lvl,
                                                                  const int* __restrict__ rows,
                                                                  const SPull* __restrict__ pulls,
                                                                  T* __restrict__ w, T* __restrict__ wu) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* f = reinterpret_cast<T*>(smraw);
  __shared__ T tile[32][33];
  __shared__ T scratch[1024];
  const SNode<T> nd = nodes[lvl[blockIdx.x]];
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) f[i] = w[nd.c0 + i];
  __syncthreads();
  for (int p = nd.childBegin; p < nd.childEnd; ++p) {
    const SPull P = pulls[p];
    const SNode<T> src = nodes[P.src];
    const int* srows = rows + src.rowsOff;
    if (P.kind == 0) {
      const T* wus = wu + src.wuOff;
      for (int a = P.a0 + threadIdx.x; a < P.a1; a += blockDim.x) f[srows[a] - nd.c0] += wus[a];
    } else {
      const T* z = wu + src.wuOff;
      for (int a = P.a0 + threadIdx.x; a < P.a1; a += blockDim.x) {
        const T* v = src.V + (size_t)a * src.r;
        T s = T(0);
        for (int k = 0; k < src.r; ++k) s += v[k] * z[k];
        f[srows[a] - nd.c0] -= s;
      }
    }
    __syncthreads();
  }
  trsv_lower<T>(nd.L, nd.ld, nd.n, f, tile);
  if (nd.r > 0) gemv_t_split<T>(nd.U, nd.r, nd.n, nd.r, [&](int i) { return f[i]; }, wu + nd.wuOff, scratch);
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) w[nd.c0 + i] = f[i];
}

template <class T>
__global__ void __launch_bounds__(1024) compressed_backward_kernel(const SNode<T>* __restrict__ nodes,
                                                                   const int* __restrict__ lvl,
                                                                   const int* __restrict__ rows,
                                                                   T* __restrict__ w) {
  extern __shared__ __align__(16) unsigned char smraw[];
  T* sm = reinterpret_cast<T*>(smraw);
  __shared__ T tile[32][33];
  __shared__ T scratch[1024];
  const SNode<T> nd = nodes[lvl[blockIdx.x]];
  T* f = sm;
  T* s = sm + nd.n;
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) f[i] = w[nd.c0 + i];
  __syncthreads();
  if (nd.r > 0 && nd.m > 0) {
    const int* rw = rows + nd.rowsOff;
    gemv_t_split<T>(nd.V, nd.r, nd.m, nd.r, [&](int a) { return w[rw[a]]; }, s, scratch);
    for (int i = threadIdx.x; i < nd.n; i += blockDim.x) {
      const T* u = nd.U + (size_t)i * nd.r;
      T acc = T(0);
      for (int k = 0; k < nd.r; ++k) acc += u[k] * s[k];
      f[i] -= acc;
    }
  }
  __syncthreads();
  trsv_lower_t<T>(nd.L, nd.ld, nd.n, f, tile);
  for (int i = threadIdx.x; i < nd.n; i += blockDim.x) w[nd.c0 + i] = f[i];
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
  std::vector<SPull> pulls;
  long long wuCur = 0;
  bytesPerApply_ = 0;
  std::vector<int> pos(S.n, -1);
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
      wuCur += sn.r;
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
  // compressed pulls: interior roots' update vectors, then compressed V z
  std::vector<std::vector<SPull>> pl(nn);
  for (int c = 0; c < nn; ++c) {
    const Node& cn = S.nodes[c];
    bool isRoot = !cn.compressed && (cn.parent < 0 || S.nodes[cn.parent].compressed);
    if (!cn.compressed && !isRoot) continue;
    for (size_t q = 0; q < cn.interNode.size(); ++q)
      pl[cn.interNode[q]].push_back(SPull{c, cn.interStart[q], cn.interStart[q + 1], cn.compressed ? 1 : 0});
  }
  for (int s = 0; s < nn; ++s) {
    if (!S.nodes[s].compressed) continue;
    std::stable_sort(pl[s].begin(), pl[s].end(), [](const SPull& a, const SPull& b) { return a.kind < b.kind; });
    nodes_[s].childBegin = (int)pulls.size();
    pulls.insert(pulls.end(), pl[s].begin(), pl[s].end());
    nodes_[s].childEnd = (int)pulls.size();
  }
  iLevels_.clear();
  cLevels_.clear();
  maxCompN_ = 0;
  smemIF_.clear();
  smemIB_.clear();
  smemCF_.clear();
  smemCB_.clear();
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
  for (auto& lv : F_.compressedLevels) {
    cLevels_.push_back({(long long)lvlNodes.size(), (int)lv.size()});
    lvlNodes.insert(lvlNodes.end(), lv.begin(), lv.end());
    size_t f = 8, b = 8;
    for (int j : lv) {
      maxCompN_ = std::max(maxCompN_, S.nodes[j].n + nodes_[j].r);
      f = std::max(f, sizeof(T) * S.nodes[j].n);
      b = std::max(b, sizeof(T) * (S.nodes[j].n + nodes_[j].r));
    }
    smemCF_.push_back(f);
    smemCB_.push_back(b);
  }
  for (size_t v : smemIB_)
    if (v > 200 * 1024) throw std::runtime_error("interior front too large for the shared-memory solve");
  for (size_t v : smemCB_)
    if (v > 200 * 1024) throw std::runtime_error("compressed supernode too large for the shared-memory solve");
  cudaStream_t st = F_.stream;
  auto up = [&](DevBuf& b, const void* src, size_t bytes) {
    b.alloc(std::max<size_t>(bytes, 16));
    if (bytes) RSCHOL_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, st));
  };
  up(dNodes_, nodes_.data(), nodes_.size() * sizeof(SNode<T>));
  up(dRows_, rowsAll.data(), rowsAll.size() * sizeof(int));
  up(dRel_, rel.data(), rel.size() * sizeof(int));
  up(dChild_, child.data(), child.size() * sizeof(int));
  up(dPull_, pulls.data(), pulls.size() * sizeof(SPull));
  up(dLevelNodes_, lvlNodes.data(), lvlNodes.size() * sizeof(int));
  dWu_.alloc(sizeof(T) * std::max(1LL, wuCur));
  if (!std::is_same<T, double>::value) dW_.alloc(sizeof(T) * std::max(1, S.n));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  const int maxSmem = 200 * 1024;
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  RSCHOL_CUDA(cudaFuncSetAttribute(interior_backward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  RSCHOL_CUDA(cudaFuncSetAttribute(compressed_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  RSCHOL_CUDA(cudaFuncSetAttribute(compressed_backward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, maxSmem));
  launchesPerApply_ = 2 * ((long long)iLevels_.size() + (long long)cLevels_.size());
  bytesPerApply_ += 8.0 * 4 * S.n;
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
  for (size_t l = 0; l < iLevels_.size(); ++l) {
    interior_forward_kernel<T><<<iLevels_[l].second, 256, smemIF_[l], st>>>(
        dNodes_.as<SNode<T>>(), lvl + iLevels_[l].first, dRows_.as<int>(), dRel_.as<int>(), dChild_.as<int>(), w,
        dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  for (size_t l = 0; l < cLevels_.size(); ++l) {
    compressed_forward_kernel<T><<<cLevels_[l].second, 1024, smemCF_[l], st>>>(
        dNodes_.as<SNode<T>>(), lvl + cLevels_[l].first, dRows_.as<int>(), dPull_.as<SPull>(), w, dWu_.as<T>());
    RSCHOL_LAUNCH_CHECK();
  }
  for (int l = (int)cLevels_.size() - 1; l >= 0; --l) {
    compressed_backward_kernel<T><<<cLevels_[l].second, 1024, smemCB_[l], st>>>(
        dNodes_.as<SNode<T>>(), lvl + cLevels_[l].first, dRows_.as<int>(), w);
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
