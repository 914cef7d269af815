#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "pcg.cuh"

namespace rschol {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int VEC_THREADS = 256;
constexpr int VEC_BLOCKS = 152 * 8;   // fixed grid: 8 CTAs per SM on 152 SMs

enum { S_DELTA = 0, S_ALPHA, S_BETA, S_RREL, S_BNORM, S_DQ, S_DELTA_NEW, S_BREAK, S_ITERS, S_TRUE, S_COUNT };
enum { F_ALPHA = 0, F_RNORM, F_BETA, F_DELTA0, F_BNORM, F_TRUE };

__device__ __forceinline__ double block_sum(double v) {
  __shared__ double ws[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) ws[warp] = v;
  __syncthreads();
  double t = 0;
  if (warp == 0) {
    t = (lane < (int)(blockDim.x >> 5)) ? ws[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(FULL, t, o);
  }
  return t;   // valid in thread 0
}

template <int TPR>
__global__ void spmv_kernel(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                            const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y,
                            double* __restrict__ part, int withDot) {
  pdl_enter();
  const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int row = (int)(g / TPR), lane = (int)(g % TPR);
  double s = 0.0;
  if (row < n)
    for (int p = rp[row] + lane; p < rp[row + 1]; p += TPR) s += v[p] * x[ci[p]];
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o, TPR);
  double dq = 0.0;
  if (lane == 0 && row < n) {
    y[row] = s;
    dq = x[row] * s;
  }
  if (withDot) {
    double t = block_sum(dq);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}

__global__ void dot_kernel(const double* __restrict__ a, const double* __restrict__ b, int n,
                           double* __restrict__ part) {
  pdl_enter();
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += a[i] * b[i];
  double t = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void finish_kernel(const double* __restrict__ part, int count, double* __restrict__ sc, int mode) {
  pdl_enter();
  double s = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) s += part[i];
  double t = block_sum(s);
  if (threadIdx.x != 0) return;
  switch (mode) {
    case F_ALPHA: {
      sc[S_DQ] = t;
      if (fabs(t) > 0.0) sc[S_ALPHA] = sc[S_DELTA] / t;
      else { sc[S_ALPHA] = 0.0; sc[S_BREAK] = 1.0; }
      break;
    }
    case F_RNORM: sc[S_RREL] = sqrt(t) / sc[S_BNORM]; break;
    case F_BETA: {
      sc[S_DELTA_NEW] = t;
      sc[S_BETA] = t / sc[S_DELTA];
      sc[S_DELTA] = t;
      break;
    }
    case F_DELTA0: sc[S_DELTA] = t; break;
    case F_BNORM: sc[S_BNORM] = sqrt(t); break;
    case F_TRUE: sc[S_TRUE] = sqrt(t) / sc[S_BNORM]; break;
  }
}

// x += alpha d, r -= alpha q, and rcopy = r (the preconditioner's input)
__global__ void update_xr_kernel(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ d,
                                 const double* __restrict__ q, const double* __restrict__ sc, int n,
                                 double* __restrict__ part, double* __restrict__ rcopy) {
  pdl_enter();
  const double a = sc[S_ALPHA];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += a * d[i];
    const double ri = r[i] - a * q[i];
    r[i] = ri;
    rcopy[i] = ri;
    s += ri * ri;
  }
  double t = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void update_d_kernel(double* __restrict__ d, const double* __restrict__ s,
                                const double* __restrict__ sc, int n) {
  pdl_enter();
  const double b = sc[S_BETA];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = s[i] + b * d[i];
}

__global__ void residual_kernel(const double* __restrict__ b, const double* __restrict__ q, int n,
                                double* __restrict__ part) {
  pdl_enter();
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double e = b[i] - q[i];
    s += e * e;
  }
  double t = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// Control of the captured solve's WHILE node: the first iteration runs when
// maxit > 0 (the reference's loop starts with maxR = 2 eps > eps); after each
// iteration another follows while ||r|| / ||b|| > eps and iterations < maxit
// (a NaN residual stops it, as the host loop does).  ctl = {eps, maxit}.
__global__ void pcg_start_kernel(const double* __restrict__ ctl, cudaGraphConditionalHandle h) {
  pdl_enter();
  cudaGraphSetConditional(h, ctl[1] > 0.5 ? 1u : 0u);
}

__global__ void pcg_control_kernel(double* __restrict__ sc, const double* __restrict__ ctl,
                                   cudaGraphConditionalHandle h) {
  pdl_enter();
  const double it = sc[S_ITERS] + 1.0;
  sc[S_ITERS] = it;
  const double r = sc[S_RREL];
  cudaGraphSetConditional(h, (it < ctl[1] && r > ctl[0]) ? 1u : 0u);
}

__global__ void gather_kernel(const double* __restrict__ src, const int* __restrict__ perm, double* __restrict__ dst,
                              int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[perm[i]];
}

__global__ void scatter_perm_kernel(const double* __restrict__ src, const int* __restrict__ perm,
                                    double* __restrict__ dst, int n) {
  pdl_enter();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[perm[i]] = src[i];
}

__global__ void index_gather_kernel(const double* __restrict__ src, const int* __restrict__ idx,
                                    double* __restrict__ dst, long long count) {
  pdl_enter();
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < count;
       k += (long long)gridDim.x * blockDim.x)
    dst[k] = src[idx[k]];
}

}  // namespace

void launch_index_gather(const double* src, const int* idx, double* dst, long long count, cudaStream_t s) {
  if (count <= 0) return;
  launch_k(index_gather_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, s, src, idx, dst, count);
  RSCHOL_LAUNCH_CHECK();
}

void launch_gather(const double* src, const int* perm, double* dst, int n, cudaStream_t s) {
  launch_k(gather_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, s, src, perm, dst, n);
  RSCHOL_LAUNCH_CHECK();
}
void launch_scatter_perm(const double* src, const int* perm, double* dst, int n, cudaStream_t s) {
  launch_k(scatter_perm_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, s, src, perm, dst, n);
  RSCHOL_LAUNCH_CHECK();
}

PcgEngine::PcgEngine(int n_, const std::vector<int>& rowptr, const std::vector<int>& colind,
                     const std::vector<double>& vals, cudaStream_t s)
    : n(n_), stream_(s) {
  rowptr_.alloc(sizeof(int) * rowptr.size());
  colind_.alloc(sizeof(int) * std::max<size_t>(1, colind.size()));
  vals_.alloc(sizeof(double) * std::max<size_t>(1, vals.size()));
  RSCHOL_CUDA(cudaMemcpyAsync(rowptr_.p, rowptr.data(), sizeof(int) * rowptr.size(), cudaMemcpyHostToDevice, s));
  RSCHOL_CUDA(cudaMemcpyAsync(colind_.p, colind.data(), sizeof(int) * colind.size(), cudaMemcpyHostToDevice, s));
  RSCHOL_CUDA(cudaMemcpyAsync(vals_.p, vals.data(), sizeof(double) * vals.size(), cudaMemcpyHostToDevice, s));
  const double avg = n > 0 ? (double)colind.size() / n : 1.0;
  // threads per row: one (each thread's loads all in flight at once) up to 12
  // entries per row -- the c2 PCG took 20.84 ms at one, 20.99 at two, 21.14
  // at four, 21.64 at eight -- then more for longer rows
  tpr_ = avg <= 12 ? 1 : avg <= 40 ? 16 : 32;
  if (const char* e = std::getenv("RSCHOL_SPMV_TPR")) {   // threads per row of the SpMV (1 ... 32)
    const int t = std::atoi(e);
    if (t == 1 || t == 2 || t == 4 || t == 8 || t == 16 || t == 32) tpr_ = t;
  }
  nblk_ = (int)(((long long)n * tpr_ + VEC_THREADS - 1) / VEC_THREADS);
  for (auto* b : {&r_, &d_, &q_, &s_}) b->alloc(sizeof(double) * std::max(1, n));
  part_.alloc(sizeof(double) * std::max(nblk_, VEC_BLOCKS));
  scal_.alloc(sizeof(double) * S_COUNT);
  RSCHOL_CUDA(cudaMallocHost((void**)&hScal_, sizeof(double) * S_COUNT));
  ctl_.alloc(sizeof(double) * 2);
  RSCHOL_CUDA(cudaMallocHost((void**)&hCtl_, sizeof(double) * 2));
  const char* g = std::getenv("RSCHOL_PCG_GRAPH");
  useGraph_ = !(g && g[0] == '0');
  spmvBytes = 12.0 * colind.size() + 4.0 * (n + 1) + 16.0 * n;
  RSCHOL_CUDA(cudaStreamSynchronize(s));
}

PcgEngine::~PcgEngine() {
  drop_graph();
  if (hScal_) cudaFreeHost(hScal_);
  if (hScalB_) cudaFreeHost(hScalB_);
  if (hCtl_) cudaFreeHost(hCtl_);
}

void PcgEngine::drop_graph() {
  if (gExec_) cudaGraphExecDestroy(gExec_);
  gExec_ = nullptr;
  gB_ = nullptr;
  gX_ = nullptr;
}

void PcgEngine::set_values(const std::vector<double>& vals) {
  RSCHOL_CUDA(cudaMemcpyAsync(vals_.p, vals.data(), sizeof(double) * vals.size(), cudaMemcpyHostToDevice, stream_));
}

void PcgEngine::spmv(const double* x, double* y) {
  switch (tpr_) {
    case 1: launch_k(spmv_kernel<1>, dim3(nblk_), dim3(VEC_THREADS), 0, stream_, n, rowptr_.as<int>(), colind_.as<int>(), vals_.as<double>(), x, y, part_.as<double>(), 1); break;
    case 2: launch_k(spmv_kernel<2>, dim3(nblk_), dim3(VEC_THREADS), 0, stream_, n, rowptr_.as<int>(), colind_.as<int>(), vals_.as<double>(), x, y, part_.as<double>(), 1); break;
    case 4: launch_k(spmv_kernel<4>, dim3(nblk_), dim3(VEC_THREADS), 0, stream_, n, rowptr_.as<int>(), colind_.as<int>(), vals_.as<double>(), x, y, part_.as<double>(), 1); break;
    case 8: launch_k(spmv_kernel<8>, dim3(nblk_), dim3(VEC_THREADS), 0, stream_, n, rowptr_.as<int>(), colind_.as<int>(), vals_.as<double>(), x, y, part_.as<double>(), 1); break;
    case 16: launch_k(spmv_kernel<16>, dim3(nblk_), dim3(VEC_THREADS), 0, stream_, n, rowptr_.as<int>(), colind_.as<int>(), vals_.as<double>(), x, y, part_.as<double>(), 1); break;
    default: launch_k(spmv_kernel<32>, dim3(nblk_), dim3(VEC_THREADS), 0, stream_, n, rowptr_.as<int>(), colind_.as<int>(), vals_.as<double>(), x, y, part_.as<double>(), 1); break;
  }
  RSCHOL_LAUNCH_CHECK();
  ++launches;
}

// x0 = 0, r = b, ||b||, s = M^{-1} r, delta = r.s, d = s
void PcgEngine::prologue(const double* b, double* x, const std::function<void(double*)>& apply) {
  double* r = r_.as<double>();
  double* d = d_.as<double>();
  double* s = s_.as<double>();
  double* part = part_.as<double>();
  double* sc = scal_.as<double>();
  cudaStream_t st = stream_;
  RSCHOL_CUDA(cudaMemsetAsync(sc, 0, sizeof(double) * S_COUNT, st));
  RSCHOL_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  RSCHOL_CUDA(cudaMemcpyAsync(r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  launch_k(dot_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, st, b, b, n, part);
  launch_k(finish_kernel, dim3(1), dim3(1024), 0, st, part, VEC_BLOCKS, sc, F_BNORM);
  RSCHOL_CUDA(cudaMemcpyAsync(s, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  apply(s);
  launch_k(dot_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, st, r, s, n, part);
  launch_k(finish_kernel, dim3(1), dim3(1024), 0, st, part, VEC_BLOCKS, sc, F_DELTA0);
  RSCHOL_CUDA(cudaMemcpyAsync(d, s, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  launches += 4;
  RSCHOL_LAUNCH_CHECK();
}

// q = A d, alpha, x += alpha d, r -= alpha q (s = r), ||r||, s = M^{-1} r,
// beta, d = s + beta d
void PcgEngine::iteration(double* x, const std::function<void(double*)>& apply) {
  double* r = r_.as<double>();
  double* d = d_.as<double>();
  double* q = q_.as<double>();
  double* s = s_.as<double>();
  double* part = part_.as<double>();
  double* sc = scal_.as<double>();
  cudaStream_t st = stream_;
  spmv(d, q);
  launch_k(finish_kernel, dim3(1), dim3(1024), 0, st, part, nblk_, sc, F_ALPHA);
  launch_k(update_xr_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, st, x, r, d, q, sc, n, part, s);
  launch_k(finish_kernel, dim3(1), dim3(1024), 0, st, part, VEC_BLOCKS, sc, F_RNORM);
  apply(s);
  launch_k(dot_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, st, r, s, n, part);
  launch_k(finish_kernel, dim3(1), dim3(1024), 0, st, part, VEC_BLOCKS, sc, F_BETA);
  launch_k(update_d_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, st, d, s, sc, n);
  RSCHOL_LAUNCH_CHECK();
  launches += 6;
}

// true residual ||b - A x|| / ||b||
void PcgEngine::epilogue(const double* b, const double* x) {
  double* q = q_.as<double>();
  double* part = part_.as<double>();
  double* sc = scal_.as<double>();
  spmv(x, q);
  launch_k(residual_kernel, dim3(VEC_BLOCKS), dim3(VEC_THREADS), 0, stream_, b, q, n, part);
  launch_k(finish_kernel, dim3(1), dim3(1024), 0, stream_, part, VEC_BLOCKS, sc, F_TRUE);
  RSCHOL_LAUNCH_CHECK();
  launches += 2;
}

PcgResult PcgEngine::solve(const double* b, double* x, double eps, int maxit,
                           const std::function<void(double*)>& apply) {
  PcgResult res;
  cudaStream_t st = stream_;
  launches = 0;
  prologue(b, x, apply);
  double maxR = 2.0 * eps;
  int i = 0;
  while (i < maxit && maxR > eps) {
    iteration(x, apply);
    RSCHOL_CUDA(cudaMemcpyAsync(hScal_, scal_.p, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
    RSCHOL_CUDA(cudaStreamSynchronize(st));
    maxR = hScal_[S_RREL];
    if (hScal_[S_BREAK] != 0.0) res.breakdown = true;
    ++i;
    if (!(maxR == maxR)) break;   // NaN: stop
  }
  res.iterations = i;
  res.residual = maxR;
  epilogue(b, x);
  RSCHOL_CUDA(cudaMemcpyAsync(hScal_, scal_.p, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  res.trueResidual = hScal_[S_TRUE];
  return res;
}

PcgResult PcgEngine::solve_graph(const double* b, double* x, double eps, int maxit,
                                 const std::function<void(double*)>& apply, unsigned long long key) {
  if (!useGraph_) return solve(b, x, eps, maxit, apply);
  cudaStream_t st = stream_;
  if (!gExec_ || gB_ != b || gX_ != x || gKey_ != key) {
    drop_graph();
    // three captures into one graph: the prologue, the WHILE node's body,
    // the epilogue after the WHILE node
    const cudaStreamCaptureMode mode = cudaStreamCaptureModeThreadLocal;
    cudaGraph_t g = nullptr;
    RSCHOL_CUDA(cudaGraphCreate(&g, 0));
    struct GraphGuard {
      cudaGraph_t g;
      ~GraphGuard() { if (g) cudaGraphDestroy(g); }
    } guard{g};
    cudaGraphConditionalHandle h;
    RSCHOL_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
    auto capture = [&](cudaGraph_t into, const cudaGraphNode_t* deps, size_t nDeps,
                       const std::function<void()>& body) -> std::vector<cudaGraphNode_t> {
      RSCHOL_CUDA(cudaStreamBeginCaptureToGraph(st, into, deps, nullptr, nDeps, mode));
      std::vector<cudaGraphNode_t> leaves;
      try {
        body();
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* d = nullptr;
        const cudaGraphEdgeData* ed = nullptr;   // queried so that programmatic edges are not a lossy query
        size_t nd = 0;
        RSCHOL_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &d, &ed, &nd));
        leaves.assign(d, d + nd);
      } catch (...) {
        cudaGraph_t dummy;
        cudaStreamEndCapture(st, &dummy);
        throw;
      }
      cudaGraph_t out = nullptr;
      RSCHOL_CUDA(cudaStreamEndCapture(st, &out));
      return leaves;
    };
    const double* ctl = ctl_.as<double>();
    launches = 0;
    std::vector<cudaGraphNode_t> pro = capture(g, nullptr, 0, [&] {
      prologue(b, x, apply);
      launch_k(pcg_start_kernel, dim3(1), dim3(32), 0, st, ctl, h);
      ++launches;
    });
    gPro_ = launches;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cond;
    RSCHOL_CUDA(cudaGraphAddNode(&cond, g, pro.data(), nullptr, pro.size(), &cp));
    cudaGraph_t bodyGraph = cp.conditional.phGraph_out[0];
    launches = 0;
    capture(bodyGraph, nullptr, 0, [&] {
      iteration(x, apply);
      launch_k(pcg_control_kernel, dim3(1), dim3(32), 0, st, scal_.as<double>(), ctl, h);
      ++launches;
    });
    gBody_ = launches;
    launches = 0;
    capture(g, &cond, 1, [&] { epilogue(b, x); });
    gEpi_ = launches;
    RSCHOL_CUDA(cudaGraphInstantiate(&gExec_, g, 0));
    gB_ = b;
    gX_ = x;
    gKey_ = key;
  }
  hCtl_[0] = eps;
  hCtl_[1] = (double)maxit;
  RSCHOL_CUDA(cudaMemcpyAsync(ctl_.p, hCtl_, sizeof(double) * 2, cudaMemcpyHostToDevice, st));
  RSCHOL_CUDA(cudaGraphLaunch(gExec_, st));
  RSCHOL_CUDA(cudaMemcpyAsync(hScal_, scal_.p, sizeof(double) * S_COUNT, cudaMemcpyDeviceToHost, st));
  RSCHOL_CUDA(cudaStreamSynchronize(st));
  PcgResult res;
  res.iterations = (int)hScal_[S_ITERS];
  res.residual = res.iterations > 0 ? hScal_[S_RREL] : 2.0 * eps;
  res.trueResidual = hScal_[S_TRUE];
  res.breakdown = hScal_[S_BREAK] != 0.0;
  launches = gPro_ + (long long)res.iterations * gBody_ + gEpi_;
  return res;
}

}  // namespace rschol
