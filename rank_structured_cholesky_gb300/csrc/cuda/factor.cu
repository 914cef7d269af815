#include <algorithm>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <type_traits>

#include "../host/rng.h"
#include "solve_dev.cuh"
#include "factor.cuh"

namespace rschol {

namespace {
constexpr int NB = 64;           // tile width of the blocked factorisations
int tiles_of(int M, int N, int rowsPerTile) { return ((M + rowsPerTile - 1) / rowsPerTile) * ((N + 63) / 64); }

// FP32 factors run their GEMMs on the tensor cores unless
// RSCHOL_TENSOR_CORES=0 (the SIMT kernel then serves both precisions).
bool tensor_cores_enabled() {
  const char* e = std::getenv("RSCHOL_TENSOR_CORES");
  return !(e && e[0] == '0');
}
}  // namespace

template <class T>
FactorEngine<T>::FactorEngine(const Symbolic& S_, const CSC& A_, const Params& p, cudaStream_t s)
    : S(S_), A(A_), prm(p), stream(s) {
  dAvals.alloc(sizeof(double) * std::max<size_t>(1, A.x.size()));
  RSCHOL_CUDA(cudaMemcpyAsync(dAvals.p, A.x.data(), sizeof(double) * A.x.size(), cudaMemcpyHostToDevice, stream));
  dFlag.alloc(3 * sizeof(int));
  waitLimit_ = solvedev::SPIN_LIMIT;
  if (const char* wl = std::getenv("RSCHOL_WAIT_LIMIT")) {
    const long v = std::strtol(wl, nullptr, 10);
    if (v >= 16 && v <= (1L << 26)) waitLimit_ = (int)v;
  }
  const char* drop = std::getenv("RSCHOL_TEST_DROP_CHOL_ITEM");
  dropItemTest_ = drop && drop[0] == '1';
  useTc_ = std::is_same<T, float>::value && tensor_cores_enabled();
  const char* fc = std::getenv("RSCHOL_FUSED_CHOL");
  fusedChol_ = !(fc && fc[0] == '0');
  const char* g = std::getenv("RSCHOL_GRAPHS");
  useGraphs_ = !(g && g[0] == '0');
  RSCHOL_CUDA(cudaStreamSynchronize(stream));
}

template <class T>
void FactorEngine<T>::set_values(const double* lowerVals) {
  RSCHOL_CUDA(cudaMemcpyAsync(dAvals.p, lowerVals, sizeof(double) * A.x.size(), cudaMemcpyHostToDevice, stream));
}

template <>
void FactorEngine<float>::gemm_launch(const Step& st) {
  if (st.kind == ST_GEMM_REDUCE)
    launch_gemm_splitk_reduce(dGemm_.as<GemmTask<float>>(), dSplitIds_.as<int>() + st.off, st.count,
                              dSplitBase_.as<long long>() + st.aux, st.elems, stream);
  else if (st.aux)
    launch_gemm_tc(dGemm_.as<GemmTask<float>>() + st.off, st.count, st.grid, dFlag.as<int>() + 1, stream,
                   st.aux & 0xffff, st.aux >> 16);
  else
    launch_gemm<float>(dGemm_.as<GemmTask<float>>() + st.off, st.count, st.grid, stream);
}

template <>
void FactorEngine<double>::gemm_launch(const Step& st) {
  launch_gemm<double>(dGemm_.as<GemmTask<double>>() + st.off, st.count, st.grid, stream);
}

template <class T>
void FactorEngine<T>::flush_gemm(std::vector<GemmTask<T>>& batch, int) {
  if (batch.empty()) return;
  // Path: the tensor cores for FP32 steps with a real K (rank-64 updates are
  // bound by C traffic, which the SIMT kernel already streams); large-K tasks
  // of steps with few tiles are split along K (slices of at least 128) to
  // fill the SMs.
  // (rank-64 updates on the tensor cores measured slower than the SIMT kernel
  // even with both operands on the asynchronous-copy path: 24.8 vs 17.0 ms of
  // GEMM time in the c2 factor; so did a 128 x 128 SIMT tile with 8 x 8
  // outputs per thread, 15.9 vs 12.1 ms: only the K >= 69 contribution
  // updates gained, the K = 64 steps turned latency-bound in the epilogue)
  int maxK = 0, maxN = 0;
  for (auto& t : batch) {
    maxK = std::max(maxK, t.K);
    maxN = std::max(maxN, t.N);
  }
  const bool tc = useTc_ && maxK >= tcMinK_;
  // BF16 hi/lo splits for the launch when asked for and it holds split tasks
  bool bf = false;
  if (tc && prm.schur_bf16)
    for (auto& t : batch) bf = bf || t.split != 0;
  const int kAlign = bf ? 64 : 32;   // K per pipeline stage: split-K slices start on one
  const int rowsPerTile = tc ? 128 : 64;
  const int bn = tc ? tc_tile_n(maxN) : 64;   // tile width: 128 x bn on the tensor cores
  long long baseTiles = 0;
  for (auto& t : batch) baseTiles += (long long)((t.M + rowsPerTile - 1) / rowsPerTile) * ((t.N + bn - 1) / bn);
  const long long want = 2LL * 152;   // two blocks per SM
  int tiles = 0;
  std::vector<int> ids;
  std::vector<long long> base{0};
  const long long first = (long long)gemm_.size();
  for (size_t q = 0; q < batch.size(); ++q) {
    GemmTask<T>& t = batch[q];
    t.tilesN = (t.N + bn - 1) / bn;
    t.bn = bn;
    const int tilesPer = ((t.M + rowsPerTile - 1) / rowsPerTile) * t.tilesN;
    t.kSplit = 1;
    t.kLen = t.K;
    long long wsOff = -1;
    if (tc && !t.lower && t.K >= 256 && baseTiles < want) {
      int ks = (int)std::min<long long>(16, std::min<long long>(t.K / 128, (want + baseTiles - 1) / baseTiles));
      if (ks > 1) {
        const int kl = ((t.K + ks - 1) / ks + kAlign - 1) / kAlign * kAlign;
        t.kSplit = (t.K + kl - 1) / kl;
        t.kLen = kl;
        wsOff = wsCur_;
        wsCur_ += (long long)t.kSplit * tilesPer * 128 * bn;
        ids.push_back((int)(first + q));
        base.push_back(base.back() + (long long)t.M * t.N);
      }
    }
    t.tileBase = tiles;
    tiles += tilesPer * t.kSplit;
    gemmWsOff_.push_back(wsOff);
  }
  Step st{ST_GEMM, first, (int)batch.size(), tiles};
  st.aux = tc ? bn | (bf ? 1 << 16 : 0) : 0;   // the tile width, and BF16 splits in bit 16
  gemm_.insert(gemm_.end(), batch.begin(), batch.end());
  steps_.push_back(st);
  if (!ids.empty()) {
    Step r{ST_GEMM_REDUCE, (long long)splitIds_.size(), (int)ids.size(), 0};
    r.aux = (int)splitBase_.size();
    r.elems = base.back();
    splitIds_.insert(splitIds_.end(), ids.begin(), ids.end());
    splitBase_.insert(splitBase_.end(), base.begin(), base.end());
    steps_.push_back(r);
  }
  batch.clear();
}

template <class T>
void FactorEngine<T>::push_gemm(const GemmTask<T>& t0, int& tiles, std::vector<GemmTask<T>>& batch) {
  if (t0.M <= 0 || t0.N <= 0) return;
  GemmTask<T> t = t0;
  tiles += tiles_of(t.M, t.N, 64);   // tiles and bases are fixed when the batch is flushed
  batch.push_back(t);
  double f = 2.0 * t.M * t.N * std::max(t.K, 0);
  if (t.lower && t.M == t.N) f *= 0.5;
  flops += f;
}

template <class T>
void FactorEngine<T>::gemm1(const GemmTask<T>& t) {
  std::vector<GemmTask<T>> b;
  int tiles = 0;
  push_gemm(t, tiles, b);
  flush_gemm(b, tiles);
}

template <class T>
static GemmTask<T> mk_gemm(const T* A, int lda, bool tA, const T* B, int ldb, bool tB, T* C, int ldc, int M, int N,
                           int K, T alpha, T beta, bool lower = false) {
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
  t.tA = tA;
  t.tB = tB;
  t.lower = lower;
  t.alpha = alpha;
  t.beta = beta;
  t.split = 1;   // tensor-core path: FP32-accurate products unless a caller opts out
  return t;
}

// The blocked partial Cholesky of every job as one ticketed launch (step kind
// `kind`, jobs and items appended to cjobs / items): shared by the factor's
// own precision and the FP64 root separator of a mixed factor.
template <class T>
template <class U>
void FactorEngine<T>::emit_fused(const std::vector<CholJob<U>>& jobs, int kind, std::vector<CholFusedJob<U>>& cjobs,
                                 std::vector<CholItem>& items, long long& syncMax, long long& wsMax) {
  Step st{kind, (long long)items.size(), 0, 0};
  const double flops0 = flops;
  const int j0 = (int)cjobs.size();
  long long sync = 1, ws = 0;   // sync[0]: the ticket
  int maxP = 0;
  for (const auto& jb : jobs) {
    if (jb.nDiag <= 0) continue;
    CholFusedJob<U> c{};
    c.F = jb.F;
    c.ld = jb.ld;
    c.nDiag = jb.nDiag;
    c.nRows = jb.nRows;
    c.nUpd = jb.nUpd;
    c.code = jb.code;
    c.P = (jb.nDiag + NB - 1) / NB;
    c.w0 = jb.nDiag - NB * (c.P - 1);
    auto tiles = [&](int n) { return n <= c.w0 ? 1 : 1 + (n - c.w0 + NB - 1) / NB; };
    c.TR = tiles(jb.nRows);
    c.TU = tiles(jb.nUpd);
    c.r1 = c.w0;
    c.cnt = (int)(sync - 1);
    sync += (long long)c.TR * c.TU + c.TR + c.P;
    c.inv = ws;
    ws += (long long)c.P * NB * NB;
    maxP = std::max(maxP, c.P);
    cjobs.push_back(c);
    // the lower part of rows x first nUpd columns of the front: read and written once
    {
      const long long k = std::min(jb.nUpd, jb.nRows);   // sum of nRows - col over col < k
      st.bytes += 2.0 * sizeof(U) * (double)(k * jb.nRows - k * (k - 1) / 2);
    }
    for (int p = 0; p < c.P; ++p) {   // algorithmic flops, counted as the per-panel steps count them
      const int c0 = p == 0 ? 0 : c.w0 + NB * (p - 1), w = p == 0 ? c.w0 : NB;
      const int rows = jb.nRows - c0 - w, upd = jb.nUpd - c0 - w;
      flops += (double)w * w * w / 3.0 + (double)std::max(rows, 0) * w * w;
      if (rows > 0 && upd > 0) flops += 2.0 * rows * upd * w * (rows == upd ? 0.5 : 1.0);
    }
  }
  const int j1 = (int)cjobs.size();
  // Item order (a topological one, with a look-ahead of one panel): stage p
  // lists the POTRFs and TRSMs of panel p, the rest R(p - 1) of the previous
  // panel's updates (column tiles >= p + 1), then L(p), panel p's updates of
  // column tile p + 1 -- all that POTRF(p + 1) and its TRSMs wait for.  So
  // the next panel's critical pieces are taken long before the bulk of the
  // current updates is done.
  auto updates = [&](int q, int p, int bLo, int bHi) {
    const CholFusedJob<U>& c = cjobs[q];
    for (int b = std::max(bLo, p + 1); b < std::min(bHi, c.TU); ++b)
      for (int a = b; a < c.TR; ++a) items.push_back(CholItem{q, CHOL_GEMM, p, a, b});
  };
  for (int p = 0; p <= maxP; ++p) {
    for (int q = j0; q < j1; ++q)
      if (p < cjobs[q].P) items.push_back(CholItem{q, CHOL_POTRF, p, p, p});
    for (int q = j0; q < j1; ++q)
      if (p < cjobs[q].P)
        for (int a = p + 1; a < cjobs[q].TR; ++a) items.push_back(CholItem{q, CHOL_TRSM, p, a, p});
    for (int q = j0; q < j1; ++q)
      if (p >= 1 && p <= cjobs[q].P) updates(q, p - 1, p + 1, INT_MAX);   // R(p - 1)
    for (int q = j0; q < j1; ++q)
      if (p < cjobs[q].P) updates(q, p, p + 1, p + 2);                    // L(p)
  }
  if (dropItemTest_ && !droppedItem_) {   // test switch: one POTRF whose TRSMs then wait in vain
    for (size_t k = (size_t)st.off; k < items.size(); ++k)
      if (items[k].kind == CHOL_POTRF && cjobs[items[k].job].TR > items[k].p + 1) {
        items.erase(items.begin() + (long)k);
        droppedItem_ = true;
        break;
      }
  }
  st.count = st.grid = (int)(items.size() - st.off);
  st.elems = sync;
  st.flops = flops - flops0;
  if (st.count == 0) return;
  syncMax = std::max(syncMax, sync);
  wsMax = std::max(wsMax, ws);
  steps_.push_back(st);
}

template <class T>
void FactorEngine<T>::emit_chol(const std::vector<CholJob<T>>& jobs) {
  if (!rootStart_.empty()) {
    // FP64 root separator of a mixed factor: the root's blocks go through FP64
    // scratch (converted in, factored, converted back), the others as usual
    std::vector<CholJob<T>> rest;
    std::vector<CholJob<double>> root;
    std::vector<CvtTask> cv;
    int maxN = 0;
    for (const auto& jb : jobs) {
      const int node = jb.code - 1;
      auto it = rootStart_.find(node);
      if (it == rootStart_.end() || jb.nRows != jb.nDiag) {
        rest.push_back(jb);
        continue;
      }
      // the block's position in the front: its rows and columns start at d0
      T* const F0 = compressed() + frontOff[node];
      const long long e = (long long)(jb.F - F0);
      const int d0 = (int)(e / ld[node]);
      const int nn = S.nodes[node].n;
      double* D = dRoot64_.as<double>() + it->second + (long long)d0 * nn + d0;
      cv.push_back(CvtTask{reinterpret_cast<float*>(jb.F), D, jb.ld, nn, jb.nDiag});
      root.push_back(CholJob<double>{D, nn, jb.nDiag, jb.nDiag, jb.nDiag, jb.code});
      maxN = std::max(maxN, jb.nDiag);
    }
    if (!root.empty()) {
      Step in{ST_CVT, (long long)cvt_.size(), (int)cv.size(), maxN};
      in.aux = 1;
      cvt_.insert(cvt_.end(), cv.begin(), cv.end());
      steps_.push_back(in);
      emit_fused<double>(root, ST_CHOL64, cholJobs64_, cholItems64_, cholSync64_, cholWs64_);
      Step out{ST_CVT, (long long)cvt_.size(), (int)cv.size(), maxN};
      out.aux = 0;
      cvt_.insert(cvt_.end(), cv.begin(), cv.end());
      steps_.push_back(out);
    }
    if (rest.empty()) return;
    if (rest.size() != jobs.size()) {
      emit_chol_t(rest);
      return;
    }
  }
  emit_chol_t(jobs);
}

template <class T>
void FactorEngine<T>::emit_chol_t(const std::vector<CholJob<T>>& jobs) {
  if (fusedChol_) {
    emit_fused<T>(jobs, ST_CHOL, cholJobs_, cholItems_, cholSync_, cholWs_);
    return;
  }
  int maxN = 0;
  for (auto& j : jobs) maxN = std::max(maxN, j.nDiag);
  for (int kb = 0; kb < maxN; kb += NB) {
    std::vector<PotrfTask<T>> pt;
    for (auto& j : jobs) {
      if (j.nDiag <= kb) continue;
      int w = std::min(NB, j.nDiag - kb);
      pt.push_back(PotrfTask<T>{j.F + (size_t)kb * j.ld + kb, j.ld, w, j.code});
      flops += (double)w * w * w / 3.0;
    }
    if (!pt.empty()) {
      steps_.push_back(Step{ST_POTRF, (long long)potrf_.size(), (int)pt.size(), (int)pt.size()});
      potrf_.insert(potrf_.end(), pt.begin(), pt.end());
    }
    std::vector<TrsmTask<T>> tt;
    int chunks = 0;
    for (auto& j : jobs) {
      if (j.nDiag <= kb) continue;
      int w = std::min(NB, j.nDiag - kb);
      int rows = j.nRows - kb - w;
      if (rows <= 0) continue;
      TrsmTask<T> t{j.F + (size_t)kb * j.ld + kb, j.F + (size_t)(kb + w) * j.ld + kb, j.ld, j.ld, w, rows, chunks};
      chunks += (rows + trsm_rows<T>() - 1) / trsm_rows<T>();
      tt.push_back(t);
      flops += (double)rows * w * w;
    }
    if (!tt.empty()) {
      steps_.push_back(Step{ST_TRSM, (long long)trsm_.size(), (int)tt.size(), chunks});
      trsm_.insert(trsm_.end(), tt.begin(), tt.end());
    }
    std::vector<GemmTask<T>> gb;
    int tiles = 0;
    for (auto& j : jobs) {
      if (j.nDiag <= kb) continue;
      int w = std::min(NB, j.nDiag - kb);
      int M = j.nRows - kb - w, N = j.nUpd - kb - w;
      if (M <= 0 || N <= 0) continue;
      const T* P = j.F + (size_t)(kb + w) * j.ld + kb;
      push_gemm(mk_gemm<T>(P, j.ld, false, P, j.ld, true, j.F + (size_t)(kb + w) * j.ld + kb + w, j.ld, M, N, w,
                           T(-1), T(1), true),
                tiles, gb);
    }
    flush_gemm(gb, tiles);
  }
}

// Columns per block of emit_l21: the TRSM chain inside a block is 8 panels
// long, and the trailing GEMMs get K = 512 (the tensor cores' efficiency
// grows with K; the fused chain's does not).
constexpr int L21_BLOCK = 512;

template <class T>
void FactorEngine<T>::emit_l21(const std::vector<TrsmJob<T>>& jobs) {
  int maxW = 0;
  for (const auto& jb : jobs) maxW = std::max(maxW, jb.w);
  if (!useTc_ || maxW <= L21_BLOCK) {
    emit_trsm(jobs);
    return;
  }
  for (int c0 = 0; c0 < maxW; c0 += L21_BLOCK) {
    std::vector<TrsmJob<T>> tb;
    for (const auto& jb : jobs)
      if (c0 < jb.w && jb.rows > 0)
        tb.push_back(TrsmJob<T>{jb.L + (size_t)c0 * jb.ldl + c0, jb.B + c0, jb.ldl, jb.ldb, jb.rows,
                                std::min(L21_BLOCK, jb.w - c0)});
    emit_trsm(tb);
    // B[:, c1:] -= B[:, c0:c1] L[c1:, c0:c1]^T
    std::vector<GemmTask<T>> gb;
    int tiles = 0;
    const int c1 = c0 + L21_BLOCK;
    for (const auto& jb : jobs)
      if (c1 < jb.w && jb.rows > 0)
        push_gemm(mk_gemm<T>(jb.B + c0, jb.ldb, false, jb.L + (size_t)c1 * jb.ldl + c0, jb.ldl, true, jb.B + c1,
                             jb.ldb, jb.rows, jb.w - c1, L21_BLOCK, T(-1), T(1)),
                  tiles, gb);
    flush_gemm(gb, tiles);
  }
}

template <class T>
void FactorEngine<T>::emit_trsm(const std::vector<TrsmJob<T>>& jobs) {
  if (fusedChol_) {   // one ticketed launch (TRSM jobs of the fused Cholesky kernel)
    Step st{ST_CHOL, (long long)cholItems_.size(), 0, 0};
    const double flops0 = flops;
    const int j0 = (int)cholJobs_.size();
    long long sync = 1, ws = 0;
    int maxP = 0;
    for (const auto& jb : jobs) {
      if (jb.w <= 0 || jb.rows <= 0) continue;
      CholFusedJob<T> c{};
      c.F = jb.B;
      c.ld = jb.ldb;
      c.nDiag = jb.w;
      c.nRows = jb.rows;
      c.nUpd = jb.w;
      c.L = jb.L;
      c.ldl = jb.ldl;
      c.r1 = NB;
      c.P = (jb.w + NB - 1) / NB;
      c.w0 = jb.w - NB * (c.P - 1);
      c.TR = (jb.rows + NB - 1) / NB;
      c.TU = c.P;
      c.cnt = (int)(sync - 1);
      sync += (long long)c.TR * c.TU + c.TR + c.P;
      c.inv = ws;
      ws += (long long)c.P * NB * NB;
      maxP = std::max(maxP, c.P);
      cholJobs_.push_back(c);
      // B read and written once, the lower triangle of L read once
      st.bytes += sizeof(T) * (2.0 * jb.rows * jb.w + 0.5 * (double)jb.w * (jb.w + 1));
      for (int p = 0; p < c.P; ++p) {   // algorithmic flops, as the per-panel steps count them
        const int c0 = p == 0 ? 0 : c.w0 + NB * (p - 1), w = p == 0 ? c.w0 : NB;
        flops += (double)jb.rows * w * w + 2.0 * jb.rows * (double)(jb.w - c0 - w) * w;
      }
    }
    const int j1 = (int)cholJobs_.size();
    // all diagonal inverses first (no waits), then stage p: the TRSMs of panel
    // p, the rest of panel p - 1's updates, panel p's updates of column tile p + 1
    for (int q = j0; q < j1; ++q)
      for (int p = 0; p < cholJobs_[q].P; ++p) cholItems_.push_back(CholItem{q, CHOL_POTRF, p, p, p});
    auto updates = [&](int q, int p, int bLo, int bHi) {
      const CholFusedJob<T>& c = cholJobs_[q];
      for (int b = std::max(bLo, p + 1); b < std::min(bHi, c.TU); ++b)
        for (int a = 0; a < c.TR; ++a) cholItems_.push_back(CholItem{q, CHOL_GEMM, p, a, b});
    };
    for (int p = 0; p <= maxP; ++p) {
      for (int q = j0; q < j1; ++q)
        if (p < cholJobs_[q].P)
          for (int a = 0; a < cholJobs_[q].TR; ++a) cholItems_.push_back(CholItem{q, CHOL_TRSM, p, a, p});
      for (int q = j0; q < j1; ++q)
        if (p >= 1 && p <= cholJobs_[q].P) updates(q, p - 1, p + 1, INT_MAX);
      for (int q = j0; q < j1; ++q)
        if (p < cholJobs_[q].P) updates(q, p, p + 1, p + 2);
    }
    st.count = st.grid = (int)(cholItems_.size() - st.off);
    st.elems = sync;
    st.flops = flops - flops0;
    if (st.count == 0) return;
    cholSync_ = std::max(cholSync_, sync);
    cholWs_ = std::max(cholWs_, ws);
    steps_.push_back(st);
    return;
  }
  int maxW = 0;
  for (auto& j : jobs) maxW = std::max(maxW, j.rows > 0 ? j.w : 0);
  for (int kb = 0; kb < maxW; kb += NB) {
    std::vector<TrsmTask<T>> tt;
    int chunks = 0;
    for (auto& j : jobs) {
      if (j.w <= kb || j.rows <= 0) continue;
      int bw = std::min(NB, j.w - kb);
      tt.push_back(TrsmTask<T>{j.L + (size_t)kb * j.ldl + kb, j.B + kb, j.ldl, j.ldb, bw, j.rows, chunks});
      chunks += (j.rows + trsm_rows<T>() - 1) / trsm_rows<T>();
      flops += (double)j.rows * bw * bw;
    }
    if (!tt.empty()) {
      steps_.push_back(Step{ST_TRSM, (long long)trsm_.size(), (int)tt.size(), chunks});
      trsm_.insert(trsm_.end(), tt.begin(), tt.end());
    }
    std::vector<GemmTask<T>> gb;
    int tiles = 0;
    for (auto& j : jobs) {
      if (j.w <= kb || j.rows <= 0) continue;
      int bw = std::min(NB, j.w - kb);
      int N = j.w - kb - bw;
      if (N <= 0) continue;
      push_gemm(mk_gemm<T>(j.B + kb, j.ldb, false, j.L + (size_t)(kb + bw) * j.ldl + kb, j.ldl, true, j.B + kb + bw,
                           j.ldb, j.rows, N, bw, T(-1), T(1)),
                tiles, gb);
    }
    flush_gemm(gb, tiles);
  }
}

template <class T>
void FactorEngine<T>::emit_extadd(const std::vector<EaTarget>& tgs) {
  // bucket every source row by its target row (a counting sort: target rows
  // ascending, each row's segments in source order)
  const long long first = (long long)eaR_.size();
  {   // room for this level's rows and segments, growing geometrically
    size_t segs = 0, rows = 0;
    for (const EaTarget& t : tgs) {
      rows += (size_t)t.rows;
      for (const EaSrc& es : t.src) segs += (size_t)std::max(0, es.aHi - es.aLo);
    }
    if (eaSeg_.size() + segs > eaSeg_.capacity()) eaSeg_.reserve(std::max(eaSeg_.size() + segs, 2 * eaSeg_.capacity()));
    if (eaR_.size() + rows > eaR_.capacity()) eaR_.reserve(std::max(eaR_.size() + rows, 2 * eaR_.capacity()));
  }
  std::vector<int> cnt, fill;
  for (const EaTarget& t : tgs) {
    cnt.assign(t.rows + 1, 0);
    const int s0 = (int)eaS_.size();
    for (const EaSrc& es : t.src) {
      ExtAddSource<T> src = es.s;
      src.rowRel = reinterpret_cast<const int*>(es.relOff);   // rebased at upload
      eaS_.push_back(src);
      for (int a = es.aLo; a < es.aHi; ++a) cnt[ints_[es.relOff + a] + 1]++;
    }
    for (int row = 0; row < t.rows; ++row) cnt[row + 1] += cnt[row];
    const int base = (int)eaSeg_.size();
    eaSeg_.resize((size_t)base + cnt[t.rows]);
    fill.assign(cnt.begin(), cnt.end() - 1);
    int sidx = s0;
    for (const EaSrc& es : t.src) {
      for (int a = es.aLo; a < es.aHi; ++a) eaSeg_[(size_t)base + fill[ints_[es.relOff + a]]++] = ExtAddSeg{sidx, a};
      ++sidx;
    }
    for (int row = 0; row < t.rows; ++row) {
      if (cnt[row + 1] == cnt[row]) continue;
      ExtAddRow<T> R{};
      R.Frow = t.F + (size_t)row * t.ld;
      R.segBegin = base + cnt[row];
      R.segEnd = base + cnt[row + 1];
      eaR_.push_back(R);
    }
  }
  const int count = (int)((long long)eaR_.size() - first);
  if (count > 0) steps_.push_back(Step{ST_EXTADD, first, count, (count + 7) / 8});
}

template <class T>
void FactorEngine<T>::emit_rf(const std::vector<RFJob<T>>& jobs) {
  if (jobs.empty()) return;
  std::vector<GemmTask<T>> gb;
  int tiles = 0;
  // Y = F^T G and the power iteration: only the range of Y matters, so on
  // the tensor-core path these products use plain TF32
  auto sketch = [](GemmTask<T> t) {
    t.split = 0;
    return t;
  };
  for (auto& j : jobs)
    push_gemm(sketch(mk_gemm<T>(j.F, j.ld, true, j.G, j.r, false, j.Y, j.r, j.cols, j.r, j.rows, T(1), T(0))), tiles,
              gb);
  flush_gemm(gb, tiles);
  for (int it = 0; it < prm.power_iters; ++it) {
    tiles = 0;
    for (auto& j : jobs)
      push_gemm(sketch(mk_gemm<T>(j.F, j.ld, false, j.Y, j.r, false, j.X, j.r, j.rows, j.r, j.cols, T(1), T(0))),
                tiles, gb);
    flush_gemm(gb, tiles);
    tiles = 0;
    for (auto& j : jobs)
      push_gemm(sketch(mk_gemm<T>(j.F, j.ld, true, j.X, j.r, false, j.Y, j.r, j.cols, j.r, j.rows, T(1), T(0))),
                tiles, gb);
    flush_gemm(gb, tiles);
  }
  // Thin Householder QR of Y (the sketch of a fast-decaying block is
  // numerically rank deficient, so Gram-based QR variants break down), or
  // the identity basis.
  std::vector<QrTask<T>> qt;
  std::vector<IdentTask<T>> id;
  for (auto& j : jobs) {
    if (j.identity) {
      id.push_back(IdentTask<T>{j.Y, j.cols, j.r});
    } else {
      qt.push_back(QrTask<T>{j.Y, j.W, j.cols, j.r});
      flops += 4.0 * j.cols * (double)j.r * j.r;
    }
  }
  if (!id.empty()) {
    steps_.push_back(Step{ST_IDENT, (long long)ident_.size(), (int)id.size(), (int)id.size()});
    ident_.insert(ident_.end(), id.begin(), id.end());
  }
  if (!qt.empty()) {
    int maxRows = 0, maxR = 0;
    for (auto& q : qt) {
      maxRows = std::max(maxRows, q.n);
      maxR = std::max(maxR, q.r);
    }
    steps_.push_back(Step{ST_QR, (long long)qr_.size(), (int)qt.size(), maxR, maxRows});
    qr_.insert(qr_.end(), qt.begin(), qt.end());
    qrWs_ = std::max(qrWs_, householder_qr_workspace((int)qt.size(), maxRows, maxR));
  }
  // V = F U
  tiles = 0;
  for (auto& j : jobs)
    push_gemm(mk_gemm<T>(j.F, j.ld, false, j.Y, j.r, false, j.V, j.r, j.rows, j.r, j.cols, T(1), T(0)), tiles, gb);
  flush_gemm(gb, tiles);
  // Q = U^T U and / or F := V U^T
  tiles = 0;
  for (auto& j : jobs) {
    if (j.Q)
      push_gemm(mk_gemm<T>(j.Y, j.r, true, j.Y, j.r, false, j.Q, j.r, j.r, j.r, j.cols, T(1), T(0)), tiles, gb);
    if (j.expand)
      push_gemm(mk_gemm<T>(j.V, j.r, false, j.Y, j.r, true, j.F, j.ld, j.rows, j.cols, j.r, T(1), T(0)), tiles, gb);
  }
  flush_gemm(gb, tiles);
}

template <class T>
void FactorEngine<T>::plan() {
  PlanClock clk("factor plan");
  drop_graphs();   // the captured schedule points into the buffers about to be replaced
  runsSincePlan_ = 0;
  droppedItem_ = false;
  const int nn = (int)S.nodes.size();
  const int N = S.n;
  steps_.clear();
  gemm_.clear();
  potrf_.clear();
  trsm_.clear();
  eaR_.clear();
  eaSeg_.clear();
  eaS_.clear();
  gemmWsOff_.clear();
  splitIds_.clear();
  splitBase_.clear();
  wsCur_ = 0;
  qr_.clear();
  qrWs_ = 0;
  cholJobs_.clear();
  cholItems_.clear();
  cholSync_ = cholWs_ = 0;
  cvt_.clear();
  cholJobs64_.clear();
  cholItems64_.clear();
  cholSync64_ = cholWs64_ = 0;
  rootStart_.clear();
  ident_.clear();
  ints_.clear();
  flops = 0;

  // ---- levels
  std::vector<int> h(nn, 0);
  interiorLevels.clear();
  compressedLevels.clear();
  for (int s = 0; s < nn; ++s) {
    const Node& nd = S.nodes[s];
    int hh = 0;
    for (int ch : S.children[s])
      if (S.nodes[ch].compressed == nd.compressed) hh = std::max(hh, h[ch] + 1);
    h[s] = hh;
    auto& L = nd.compressed ? compressedLevels : interiorLevels;
    if ((int)L.size() <= hh) L.resize(hh + 1);
    L[hh].push_back(s);
  }

  // ---- arenas.  Leading dimensions are padded to a multiple of 4, so every
  // front row and every 64-column panel starts on a 16-byte boundary (the
  // tensor-core GEMM's asynchronous copies move 16-byte chunks).
  auto pad4 = [](int x) { return (x + 3) & ~3; };
  frontOff.assign(nn, 0);
  ld.assign(nn, 0);
  long long curI = 0, curC = 0;
  for (auto& lv : interiorLevels)
    for (int d : lv) {
      const Node& nd = S.nodes[d];
      ld[d] = pad4(nd.n + nd.m());
      frontOff[d] = curI;
      curI += (long long)ld[d] * ld[d];
    }
  for (auto& lv : compressedLevels)
    for (int j : lv) {
      const Node& nd = S.nodes[j];
      ld[j] = pad4(nd.n);
      frontOff[j] = curC;
      curC += (long long)(nd.n + nd.m()) * ld[j];
    }
  rank.assign(nn, 0);
  vOff.assign(nn, -1);
  uOff.assign(nn, -1);
  qOff.assign(nn, -1);
  std::vector<long long> xOff(nn, -1), gmOff(nn, -1);
  long long curV = 0;
  for (int j = 0; j < nn; ++j) {
    const Node& nd = S.nodes[j];
    if (!nd.compressed || nd.m() == 0) continue;
    const int r = S.offRank[j], m = nd.m(), n = nd.n;
    rank[j] = r;
    vOff[j] = curV; curV += (long long)m * r;
    uOff[j] = curV; curV += (long long)n * r;
    qOff[j] = curV; curV += (long long)r * r;
    xOff[j] = curV; curV += (long long)m * r;
    gmOff[j] = curV; curV += (long long)n * r + r;   // Householder QR scratch
  }
  // HODLR internal-node buffers, per internal node (rows x cols block, rank r):
  // V (rows*r) | Y/U (cols*r) | X (rows*r) | QR scratch (cols*r + r) |
  // coupling scratch (hmax*hmax + hmax*cols + rows*cols)
  std::vector<std::vector<long long>> hOff(nn);
  long long curH = 0;
  auto hdims = [&](const Node& nd, int q, int& rows, int& cols) {
    const HNode& x = nd.H[q];
    rows = nd.H[x.right].r1 - nd.H[x.right].r0 + 1;
    cols = nd.H[x.left].r1 - nd.H[x.left].r0 + 1;
  };
  auto hscratch = [&](int j, int q) -> long long {   // offset of the coupling scratch
    int rows, cols;
    hdims(S.nodes[j], q, rows, cols);
    const long long r = S.hRank[j][q];
    return 2 * rows * r + 2 * cols * r + r;
  };
  for (int j = 0; j < nn; ++j) {
    const Node& nd = S.nodes[j];
    hOff[j].assign(nd.H.size(), -1);
    if (!nd.compressed) continue;
    long long hmax = 0;
    for (int v : S.hRank[j]) hmax = std::max<long long>(hmax, v);
    for (size_t q = 0; q < nd.H.size(); ++q) {
      if (nd.H[q].isLeaf()) continue;
      int rows, cols;
      hdims(nd, (int)q, rows, cols);
      hOff[j][q] = curH;
      curH += hscratch(j, (int)q) + hmax * hmax + hmax * cols + (long long)rows * cols;
    }
  }
  // compressed descendants and interior roots of each compressed supernode
  struct Pair { int src, q; };
  std::vector<std::vector<Pair>> compDesc(nn), rootsOf(nn);
  for (int c = 0; c < nn; ++c) {
    const Node& cn = S.nodes[c];
    bool isRoot = !cn.compressed && (cn.parent < 0 || S.nodes[cn.parent].compressed);
    if (!cn.compressed && !isRoot) continue;
    for (size_t q = 0; q < cn.interNode.size(); ++q) {
      if (cn.compressed) compDesc[cn.interNode[q]].push_back(Pair{c, (int)q});
      else rootsOf[cn.interNode[q]].push_back(Pair{c, (int)q});
    }
  }
  std::vector<std::vector<long long>> contribOff(nn);
  long long curT = 0;
  for (int j = 0; j < nn; ++j) {
    for (const Pair& p : compDesc[j]) {
      const Node& cn = S.nodes[p.src];
      const int s0 = cn.interStart[p.q], k1 = cn.interStart[p.q + 1] - s0, r = S.offRank[p.src];
      contribOff[j].push_back(curT);
      curT += (long long)r * k1 + (long long)(cn.m() - s0) * k1;
    }
  }
  dInterior.alloc(sizeof(T) * std::max(1LL, curI));
  dCompressed.alloc(sizeof(T) * std::max(1LL, curC));
  dVU.alloc(sizeof(T) * std::max(1LL, curV));
  dHodlr.alloc(sizeof(T) * std::max(1LL, curH));
  dContrib.alloc(sizeof(T) * std::max(1LL, curT));
  dGauss.alloc(sizeof(T) * std::max(1LL, S.totalDraws));
  deviceBytes = sizeof(T) * (curI + curC + curV + curH + curT + S.totalDraws) + sizeof(double) * A.x.size();
  if (std::is_same<T, float>::value && prm.root_fp64) {
    // the root separator: compressed supernodes at the top of the tree
    long long cur = 0;
    for (int j = 0; j < nn; ++j)
      if (S.nodes[j].compressed && S.nodes[j].parent < 0) {
        rootStart_[j] = cur;
        cur += (long long)S.nodes[j].n * S.nodes[j].n;
      }
    dRoot64_.alloc(sizeof(double) * std::max(1LL, cur));
    deviceBytes += sizeof(double) * cur;
  } else {
    dRoot64_.alloc(0);
  }
  clk.mark("arenas");
  T* const I0 = interior();
  T* const C0 = compressed();
  T* const V0 = vu();
  T* const H0 = dHodlr.as<T>();
  T* const T0 = dContrib.as<T>();
  T* const G0 = dGauss.as<T>();

  // ---- Gaussian stream (reseeded generator; raw draws on the host, the
  // Box-Muller transform on the device), in chunks of 2^21 Gaussians through
  // two pinned host buffers: the host draws chunk c + 1 while chunk c is
  // copied and transformed, and no host copy of the whole raw stream (8 bytes
  // per Gaussian, 379 MB for 3D 96^3) is allocated and first-touched.  A host
  // buffer is refilled only after the event recorded behind its last copy.
  {
    const long long total = S.totalDraws;
    if (total > 0) {
      const long long chunk = std::min<long long>(total, 1LL << 21);
      struct Staging {
        cudaStream_t s = nullptr;
        uint32_t* host[2] = {nullptr, nullptr};
        cudaEvent_t copied[2] = {nullptr, nullptr};
        ~Staging() {
          if (s) cudaStreamSynchronize(s);   // nothing may still read a buffer freed here
          for (int b = 0; b < 2; ++b) {
            if (copied[b]) cudaEventDestroy(copied[b]);
            if (host[b]) cudaFreeHost(host[b]);
          }
        }
      } stg;
      stg.s = stream;
      DevBuf dRaw[2];
      for (int b = 0; b < 2; ++b) {
        RSCHOL_CUDA(cudaMallocHost(&stg.host[b], sizeof(uint32_t) * 2 * chunk));
        RSCHOL_CUDA(cudaEventCreateWithFlags(&stg.copied[b], cudaEventDisableTiming));
        dRaw[b].alloc(sizeof(uint32_t) * 2 * chunk);
      }
      MT19937 g(prm.seed);
      long long k0 = 0;
      for (int c = 0; k0 < total; ++c, k0 += chunk) {
        const int b = c & 1;
        const long long k = std::min(chunk, total - k0);
        if (c >= 2) RSCHOL_CUDA(cudaEventSynchronize(stg.copied[b]));
        g.rawDraws(2 * k, stg.host[b]);
        RSCHOL_CUDA(cudaMemcpyAsync(dRaw[b].p, stg.host[b], sizeof(uint32_t) * 2 * k, cudaMemcpyHostToDevice,
                                    stream));
        RSCHOL_CUDA(cudaEventRecord(stg.copied[b], stream));
        launch_box_muller<T>(dRaw[b].as<uint32_t>(), k, G0 + k0, stream);
      }
      RSCHOL_CUDA(cudaStreamSynchronize(stream));
    }
  }
  clk.mark("gaussians");
  auto draw_of = [&](int node, int kind, int hnode) -> const T* {
    for (const SketchDraw& d : S.draws)
      if (d.node == node && d.kind == kind && (kind == 2 || d.h == hnode)) return G0 + d.offset;
    throw std::runtime_error("missing sketch draw");
  };

  // ---- scatter maps of A's lower entries into the fronts
  std::vector<int> pos(N, -1);
  scatSrc_.clear();
  scatDst_.clear();
  std::vector<long long> csrc, cdst;
  for (int s = 0; s < nn; ++s) {
    const Node& nd = S.nodes[s];
    for (int a = 0; a < nd.m(); ++a) pos[nd.rows[a]] = a;
    for (int c = nd.c0; c <= nd.c1; ++c)
      for (int p = A.p[c]; p < A.p[c + 1]; ++p) {
        int r = A.i[p];
        long long row = (r <= nd.c1) ? (r - nd.c0) : (nd.n + pos[r]);
        long long dst = frontOff[s] + row * ld[s] + (c - nd.c0);
        if (nd.compressed) { csrc.push_back(p); cdst.push_back(dst); }
        else { scatSrc_.push_back(p); scatDst_.push_back(dst); }
      }
    for (int a = 0; a < nd.m(); ++a) pos[nd.rows[a]] = -1;
  }
  nScatI_ = (long long)scatSrc_.size();
  nScatC_ = (long long)csrc.size();
  scatSrc_.insert(scatSrc_.end(), csrc.begin(), csrc.end());
  scatDst_.insert(scatDst_.end(), cdst.begin(), cdst.end());

  clk.mark("scatter");
  // ---- interior levels: extend-add of the children's update blocks, then
  // the blocked partial Cholesky of every front (L panel + update block).
  for (auto& lv : interiorLevels) {
    std::vector<EaTarget> tgs;
    for (int p : lv) {
      const Node& pn = S.nodes[p];
      if (S.children[p].empty()) continue;
      EaTarget t;
      t.F = I0 + frontOff[p];
      t.ld = ld[p];
      t.rows = pn.n + pn.m();
      for (int a = 0; a < pn.m(); ++a) pos[pn.rows[a]] = a;
      for (int c : S.children[p]) {
        const Node& cn = S.nodes[c];
        if (cn.m() == 0) continue;
        EaSrc es{};
        es.s.D = I0 + frontOff[c] + (long long)cn.n * ld[c] + cn.n;
        es.s.ld = ld[c];
        es.s.b0 = 0;
        es.s.b1 = cn.m();
        es.s.sign = T(1);
        es.relOff = ints_.size();
        for (int a = 0; a < cn.m(); ++a) {
          int g = cn.rows[a];
          ints_.push_back(g <= pn.c1 ? g - pn.c0 : pn.n + pos[g]);
        }
        es.aLo = 0;
        es.aHi = cn.m();
        t.src.push_back(es);
      }
      for (int a = 0; a < pn.m(); ++a) pos[pn.rows[a]] = -1;
      if (!t.src.empty()) tgs.push_back(std::move(t));
    }
    emit_extadd(tgs);
    std::vector<CholJob<T>> jobs;
    for (int d : lv) {
      const Node& nd = S.nodes[d];
      const int nm = nd.n + nd.m();
      jobs.push_back(CholJob<T>{I0 + frontOff[d], ld[d], nd.n, nm, nm, d + 1});
    }
    emit_chol(jobs);
  }

  clk.mark("interior");
  // ---- compressed levels
  for (auto& lv : compressedLevels) {
    // (a) compressed-descendant contributions V_c[s0:] (Q_c V_c[s0:s1]^T)
    std::vector<GemmTask<T>> gb;
    int tiles = 0;
    for (int j : lv)
      for (size_t k = 0; k < compDesc[j].size(); ++k) {
        const Pair& p = compDesc[j][k];
        const Node& cn = S.nodes[p.src];
        const int s0 = cn.interStart[p.q], k1 = cn.interStart[p.q + 1] - s0, r = rank[p.src];
        T* W = T0 + contribOff[j][k];
        push_gemm(mk_gemm<T>(V0 + qOff[p.src], r, false, V0 + vOff[p.src] + (size_t)s0 * r, r, true, W, k1, r, k1, r,
                             T(1), T(0)),
                  tiles, gb);
      }
    flush_gemm(gb, tiles);
    tiles = 0;
    for (int j : lv)
      for (size_t k = 0; k < compDesc[j].size(); ++k) {
        const Pair& p = compDesc[j][k];
        const Node& cn = S.nodes[p.src];
        const int s0 = cn.interStart[p.q], k1 = cn.interStart[p.q + 1] - s0, r = rank[p.src];
        T* W = T0 + contribOff[j][k];
        T* Tm = W + (size_t)r * k1;
        push_gemm(mk_gemm<T>(V0 + vOff[p.src] + (size_t)s0 * r, r, false, W, k1, false, Tm, k1, cn.m() - s0, k1, r,
                             T(1), T(0)),
                  tiles, gb);
      }
    flush_gemm(gb, tiles);
    // (b) extend-add into the dense fronts [S11; S21]
    std::vector<EaTarget> tgs;
    for (int j : lv) {
      const Node& nd = S.nodes[j];
      EaTarget t;
      t.F = C0 + frontOff[j];
      t.ld = ld[j];
      t.rows = nd.n + nd.m();
      for (int a = 0; a < nd.m(); ++a) pos[nd.rows[a]] = a;
      auto rel = [&](int g) { return g <= nd.c1 ? g - nd.c0 : nd.n + pos[g]; };
      for (const Pair& p : rootsOf[j]) {
        const Node& dn = S.nodes[p.src];
        const int sq = dn.interStart[p.q], sq1 = dn.interStart[p.q + 1];
        EaSrc es{};
        es.s.D = I0 + frontOff[p.src] + (long long)dn.n * ld[p.src] + dn.n;
        es.s.ld = ld[p.src];
        es.s.b0 = sq;
        es.s.b1 = sq1;
        es.s.sign = T(1);
        es.relOff = ints_.size();
        for (int a = 0; a < dn.m(); ++a) ints_.push_back(a >= sq ? rel(dn.rows[a]) : 0);
        es.aLo = sq;
        es.aHi = dn.m();
        t.src.push_back(es);
      }
      for (size_t k = 0; k < compDesc[j].size(); ++k) {
        const Pair& p = compDesc[j][k];
        const Node& cn = S.nodes[p.src];
        const int s0 = cn.interStart[p.q], k1 = cn.interStart[p.q + 1] - s0, r = rank[p.src];
        EaSrc es{};
        es.s.D = T0 + contribOff[j][k] + (size_t)r * k1;
        es.s.ld = k1;
        es.s.b0 = 0;
        es.s.b1 = k1;
        es.s.sign = T(-1);
        es.relOff = ints_.size();
        for (int a = s0; a < cn.m(); ++a) ints_.push_back(rel(cn.rows[a]));
        es.aLo = 0;
        es.aHi = cn.m() - s0;
        t.src.push_back(es);
      }
      for (int a = 0; a < nd.m(); ++a) pos[nd.rows[a]] = -1;
      if (!t.src.empty()) tgs.push_back(std::move(t));
    }
    emit_extadd(tgs);

    // (c) diagonal factor (+ L21 for single-block diagonals)
    auto hjob = [&](int j, int q, bool identityAllowed) {
      const Node& nd = S.nodes[j];
      const HNode& x = nd.H[q];
      const HNode& lc = nd.H[x.left];
      const HNode& rc = nd.H[x.right];
      const int rows = rc.r1 - rc.r0 + 1, cols = lc.r1 - lc.r0 + 1, r = S.hRank[j][q];
      T* base = H0 + hOff[j][q];
      RFJob<T> rj{};
      rj.F = C0 + frontOff[j] + (size_t)rc.r0 * ld[j] + lc.r0;
      rj.ld = ld[j];
      rj.rows = rows;
      rj.cols = cols;
      rj.r = r;
      rj.V = base;
      rj.Y = base + (size_t)rows * r;
      rj.X = rj.Y + (size_t)cols * r;
      rj.W = rj.X + (size_t)rows * r;
      rj.Q = nullptr;
      rj.identity = identityAllowed && r >= cols;
      rj.expand = true;
      return rj;
    };
    std::vector<CholJob<T>> cj;
    std::vector<RFJob<T>> hj;
    std::vector<TrsmJob<T>> tj;
    std::vector<int> rec;
    for (int j : lv) {
      const Node& nd = S.nodes[j];
      T* F = C0 + frontOff[j];
      if (nd.H.size() == 1) {
        cj.push_back(CholJob<T>{F, ld[j], nd.n, nd.n + nd.m(), nd.n, j + 1});
      } else if (nd.blocks.size() == 1 && nd.blocks[0].expl) {
        cj.push_back(CholJob<T>{F, ld[j], nd.n, nd.n, nd.n, j + 1});
        for (size_t q = 0; q < nd.H.size(); ++q)
          if (!nd.H[q].isLeaf()) {
            RFJob<T> rj = hjob(j, (int)q, false);
            rj.G = draw_of(j, 0, (int)q);
            hj.push_back(rj);
          }
        if (nd.m() > 0) tj.push_back(TrsmJob<T>{F, F + (size_t)nd.n * ld[j], ld[j], ld[j], nd.m(), nd.n});
      } else {
        rec.push_back(j);
      }
    }
    emit_chol(cj);
    emit_rf(hj);
    emit_l21(tj);
    for (int j : rec) {   // HODLR diagonals with recursive blocks, in block-list order
      const Node& nd = S.nodes[j];
      T* F = C0 + frontOff[j];
      const int L = ld[j];
      for (const BlockEntry& be : nd.blocks) {
        const HNode& x = nd.H[be.h];
        if (be.expl) {
          const int size = x.r1 - x.r0 + 1;
          emit_chol({CholJob<T>{F + (size_t)x.r0 * L + x.r0, L, size, size, size, j + 1}});
          std::vector<RFJob<T>> sub;
          std::function<void(int)> pre = [&](int q) {
            if (nd.H[q].isLeaf()) return;
            RFJob<T> rj = hjob(j, q, false);
            rj.G = draw_of(j, 0, q);
            sub.push_back(rj);
            pre(nd.H[q].left);
            pre(nd.H[q].right);
          };
          pre(be.h);
          emit_rf(sub);
          continue;
        }
        if (!be.diag) {
          const HNode& lc = nd.H[x.left];
          const HNode& rc = nd.H[x.right];
          const int rows = rc.r1 - rc.r0 + 1, cols = lc.r1 - lc.r0 + 1;
          T* Fba = F + (size_t)rc.r0 * L + lc.r0;
          // couplings from HODLR ancestors whose right subtree holds this block
          for (int cur = be.h, anc = x.parent; anc >= 0; cur = anc, anc = nd.H[anc].parent) {
            if (nd.H[anc].right != cur) continue;
            const HNode& ax = nd.H[anc];
            const HNode& ar = nd.H[ax.right];
            const int aRows = ar.r1 - ar.r0 + 1, aCols = nd.H[ax.left].r1 - nd.H[ax.left].r0 + 1;
            const int ra = S.hRank[j][anc];
            T* abase = H0 + hOff[j][anc];
            T* aV = abase;
            T* aU = abase + (size_t)aRows * ra;
            T* scratch = H0 + hOff[j][be.h] + hscratch(j, be.h);
            T* W1 = scratch;                      // ra x ra = U^T U
            T* W2 = W1 + (size_t)ra * ra;          // ra x cols = W1 V2^T
            gemm1(mk_gemm<T>(aU, ra, true, aU, ra, false, W1, ra, ra, ra, aCols, T(1), T(0)));
            gemm1(mk_gemm<T>(W1, ra, false, aV + (size_t)(lc.r0 - ar.r0) * ra, ra, true, W2, cols, ra, cols, ra, T(1),
                             T(0)));
            gemm1(mk_gemm<T>(aV + (size_t)(rc.r0 - ar.r0) * ra, ra, false, W2, cols, false, Fba, L, rows, cols, ra,
                             T(-1), T(1)));
            (void)aRows;
          }
          emit_trsm({TrsmJob<T>{F + (size_t)lc.r0 * L + lc.r0, Fba, L, L, rows, cols}});
          RFJob<T> rj = hjob(j, be.h, true);
          rj.G = draw_of(j, 1, be.h);
          emit_rf({rj});
          continue;
        }
        // a diagonal leaf outside any explicit subtree: updateDiagonal + factor
        const int sz = x.r1 - x.r0 + 1;
        T* Lb = F + (size_t)x.r0 * L + x.r0;
        for (int cur = be.h, anc = x.parent; anc >= 0; cur = anc, anc = nd.H[anc].parent) {
          if (nd.H[anc].right != cur) continue;
          const HNode& ax = nd.H[anc];
          const HNode& ar = nd.H[ax.right];
          const int aRows = ar.r1 - ar.r0 + 1, aCols = nd.H[ax.left].r1 - nd.H[ax.left].r0 + 1;
          const int ra = S.hRank[j][anc];
          T* aV = H0 + hOff[j][anc];
          T* aU = aV + (size_t)aRows * ra;
          T* Wv = H0 + hOff[j][anc] + hscratch(j, anc);   // sz x aCols <= aRows x aCols
          gemm1(mk_gemm<T>(aV + (size_t)(x.r0 - ar.r0) * ra, ra, false, aU, ra, true, Wv, aCols, sz, aCols, ra, T(1),
                           T(0)));
          gemm1(mk_gemm<T>(Wv, aCols, false, Wv, aCols, true, Lb, L, sz, sz, aCols, T(-1), T(1), true));
        }
        emit_chol({CholJob<T>{Lb, L, sz, sz, sz, j + 1}});
      }
      if (nd.m() > 0) emit_l21({TrsmJob<T>{F, F + (size_t)nd.n * L, L, L, nd.m(), nd.n}});
    }

    // (d) off-diagonal range finder on L21 = F[n:n+m, 0:n]
    std::vector<RFJob<T>> oj;
    for (int j : lv) {
      const Node& nd = S.nodes[j];
      if (nd.m() == 0) continue;
      RFJob<T> rj{};
      rj.F = C0 + frontOff[j] + (size_t)nd.n * ld[j];
      rj.ld = ld[j];
      rj.rows = nd.m();
      rj.cols = nd.n;
      rj.r = rank[j];
      rj.G = draw_of(j, 2, -1);
      rj.Y = V0 + uOff[j];
      rj.X = V0 + xOff[j];
      rj.W = V0 + gmOff[j];
      rj.V = V0 + vOff[j];
      rj.Q = V0 + qOff[j];
      rj.identity = rank[j] >= nd.n;
      rj.expand = false;
      oj.push_back(rj);
    }
    emit_rf(oj);
  }

  clk.mark("compressed");
  // RSCHOL_PLAN_LOG=1: one line per GEMM step on stderr (tasks, tiles, flops,
  // largest M / N / K) for tuning the batched kernels
  if (const char* e = std::getenv("RSCHOL_PLAN_LOG")) {
    if (e[0] == '1') {
      for (size_t q = 0; q < steps_.size(); ++q) {
        const Step& st = steps_[q];
        if (st.kind != ST_GEMM) continue;
        double f = 0;
        int mM = 0, mN = 0, mK = 0;
        for (int k = 0; k < st.count; ++k) {
          const GemmTask<T>& g = gemm_[st.off + k];
          f += 2.0 * g.M * g.N * (double)g.K;
          mM = std::max(mM, g.M);
          mN = std::max(mN, g.N);
          mK = std::max(mK, g.K);
        }
        std::fprintf(stderr, "plan gemm step %zu tasks %d tiles %d gflop %.3f maxM %d maxN %d maxK %d tc %d\n", q,
                     st.count, st.grid, f * 1e-9, mM, mN, mK, st.aux);
      }
    }
  }

  // ---- upload the schedule
  auto up = [&](DevBuf& b, const void* src, size_t bytes) {
    b.alloc(std::max<size_t>(bytes, 16));
    if (bytes) RSCHOL_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, stream));
  };
  up(dInts_, ints_.data(), ints_.size() * sizeof(int));
  for (auto& s : eaS_) s.rowRel = dInts_.as<int>() + reinterpret_cast<size_t>(s.rowRel);
  dSplitWs_.alloc(sizeof(float) * std::max(1LL, wsCur_));
  dQrWs_.alloc(sizeof(T) * std::max(1LL, qrWs_));
  dCholSync_.alloc(sizeof(int) * std::max(1LL, cholSync_));
  dCholWs_.alloc(sizeof(T) * std::max(1LL, cholWs_));
  dCholSync64_.alloc(cholItems64_.empty() ? 0 : sizeof(int) * std::max(1LL, cholSync64_));
  dCholWs64_.alloc(cholItems64_.empty() ? 0 : sizeof(double) * std::max(1LL, cholWs64_));
  {   // diagnostics: per-item timeline of the fused steps, sized for this plan (or none)
    const char* tp = std::getenv("RSCHOL_CHOL_TRACE");
    dCholTrace_.alloc(tp && tp[0] && !cholItems_.empty() ? 4 * sizeof(unsigned long long) * cholItems_.size() : 0);
  }
  for (size_t q = 0; q < gemm_.size(); ++q)
    if (gemmWsOff_[q] >= 0) gemm_[q].ws = dSplitWs_.as<float>() + gemmWsOff_[q];
  up(dSplitIds_, splitIds_.data(), splitIds_.size() * sizeof(int));
  up(dSplitBase_, splitBase_.data(), splitBase_.size() * sizeof(long long));
  // every task pointer must now be a device address, not a plan-time offset
  auto device_ptr = [](const void* p) { return reinterpret_cast<uintptr_t>(p) >= (uintptr_t(1) << 32); };
  for (const auto& g : gemm_)
    if (!device_ptr(g.A) || !device_ptr(g.B) || !device_ptr(g.C))
      throw std::runtime_error("factor plan: a GEMM operand was not rebased to a device address");
  for (const auto& p : potrf_)
    if (!device_ptr(p.A)) throw std::runtime_error("factor plan: a POTRF task without a device address");
  for (const auto& t : trsm_)
    if (!device_ptr(t.L) || !device_ptr(t.B))
      throw std::runtime_error("factor plan: a TRSM task without a device address");
  for (const auto& c : cholJobs_)
    if (!device_ptr(c.F)) throw std::runtime_error("factor plan: a Cholesky job without a device address");
  for (const auto& c : cholJobs64_)
    if (!device_ptr(c.F)) throw std::runtime_error("factor plan: an FP64 Cholesky job without a device address");
  up(dCholJobs64_, cholJobs64_.data(), cholJobs64_.size() * sizeof(CholFusedJob<double>));
  up(dCholItems64_, cholItems64_.data(), cholItems64_.size() * sizeof(CholItem));
  up(dCvt_, cvt_.data(), cvt_.size() * sizeof(CvtTask));
  up(dCholJobs_, cholJobs_.data(), cholJobs_.size() * sizeof(CholFusedJob<T>));
  up(dCholItems_, cholItems_.data(), cholItems_.size() * sizeof(CholItem));
  if constexpr (std::is_same<T, float>::value) {   // TMA tensor maps of the TF32 tensor-core launches' operands
    std::vector<TensorMapBytes> maps;
    for (const Step& st : steps_)
      if (st.kind == ST_GEMM && st.aux && !(st.aux >> 16)) encode_gemm_tmaps(&gemm_[st.off], st.count, st.aux & 0xffff, maps);
    up(dTmaps_, maps.data(), maps.size() * sizeof(TensorMapBytes));
    for (auto& g : gemm_) {   // 1 + map index -> the map's device address
      if (g.tmA) g.tmA = dTmaps_.as<TensorMapBytes>() + ((uintptr_t)g.tmA - 1);
      if (g.tmB) g.tmB = dTmaps_.as<TensorMapBytes>() + ((uintptr_t)g.tmB - 1);
    }
  }
  up(dGemm_, gemm_.data(), gemm_.size() * sizeof(GemmTask<T>));
  up(dPotrf_, potrf_.data(), potrf_.size() * sizeof(PotrfTask<T>));
  up(dTrsm_, trsm_.data(), trsm_.size() * sizeof(TrsmTask<T>));
  up(dEaR_, eaR_.data(), eaR_.size() * sizeof(ExtAddRow<T>));
  up(dEaSeg_, eaSeg_.data(), eaSeg_.size() * sizeof(ExtAddSeg));
  up(dEaS_, eaS_.data(), eaS_.size() * sizeof(ExtAddSource<T>));
  up(dQr_, qr_.data(), qr_.size() * sizeof(QrTask<T>));
  up(dIdent_, ident_.data(), ident_.size() * sizeof(IdentTask<T>));
  up(dScatSrc_, scatSrc_.data(), scatSrc_.size() * sizeof(long long));
  up(dScatDst_, scatDst_.data(), scatDst_.size() * sizeof(long long));
  RSCHOL_CUDA(cudaStreamSynchronize(stream));
  clk.mark("upload");
  deviceBytes += ints_.size() * 4 + gemm_.size() * sizeof(GemmTask<T>) + scatSrc_.size() * 16 +
                 cholItems_.size() * sizeof(CholItem) + cholJobs_.size() * sizeof(CholFusedJob<T>) +
                 sizeof(int) * cholSync_ + sizeof(T) * cholWs_;
  planned_ = true;
}

template <class T>
void FactorEngine<T>::drop_graphs() {
  for (auto& g : graph_)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// Everything one factorisation queues on the stream, between the status
// reset and the status read.
template <class T>
void FactorEngine<T>::enqueue(bool timing, bool capturing) {
  const unsigned recFlags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  launches = 0;
  RSCHOL_CUDA(cudaMemsetAsync(dInterior.p, 0, dInterior.bytes, stream));
  RSCHOL_CUDA(cudaMemsetAsync(dCompressed.p, 0, dCompressed.bytes, stream));
  launch_init_flags(dFlag.as<int>(), waitLimit_, stream);   // POTRF code = INT_MAX, no wait error, poll limit
  launch_scatter<T>(dAvals.as<double>(), dScatSrc_.as<long long>(), dScatDst_.as<long long>(), nScatI_, interior(),
                    stream);
  launch_scatter<T>(dAvals.as<double>(), dScatSrc_.as<long long>() + nScatI_, dScatDst_.as<long long>() + nScatI_,
                    nScatC_, compressed(), stream);
  launches += 3;
  for (size_t q = 0; q < steps_.size(); ++q) {
    const Step& st = steps_[q];
    // external records inside a capture become event-record nodes, so the
    // replayed graph still times every step
    if (timing) RSCHOL_CUDA(cudaEventRecordWithFlags(stepEv_[2 * q], stream, recFlags));
    switch (st.kind) {
      case ST_GEMM:
      case ST_GEMM_REDUCE: gemm_launch(st); break;
      case ST_POTRF: launch_potrf<T>(dPotrf_.as<PotrfTask<T>>() + st.off, st.count, dFlag.as<int>(), stream); break;
      case ST_TRSM: launch_trsm<T>(dTrsm_.as<TrsmTask<T>>() + st.off, st.count, st.grid, stream); break;
      case ST_CHOL:
        launch_chol_fused<T>(dCholJobs_.as<CholFusedJob<T>>(), dCholItems_.as<CholItem>() + st.off, st.count,
                             dCholSync_.as<int>(), st.elems, dCholWs_.as<T>(), dFlag.as<int>(),
                             dCholTrace_.p ? dCholTrace_.as<unsigned long long>() + 4 * st.off : nullptr, stream);
        break;
      case ST_EXTADD:
        launch_extadd<T>(dEaR_.as<ExtAddRow<T>>() + st.off, st.count, dEaSeg_.as<ExtAddSeg>(),
                         dEaS_.as<ExtAddSource<T>>(), stream);
        break;
      case ST_QR:
        launches += launch_householder_qr<T>(dQr_.as<QrTask<T>>() + st.off, st.count, st.aux, st.grid,
                                             dQrWs_.as<T>(), stream) - 1;
        break;
      case ST_IDENT: launch_set_identity<T>(dIdent_.as<IdentTask<T>>() + st.off, st.count, stream); break;
      case ST_CVT: launch_block_convert(dCvt_.as<CvtTask>() + st.off, st.count, st.grid, st.aux, stream); break;
      case ST_CHOL64:
        launch_chol_fused<double>(dCholJobs64_.as<CholFusedJob<double>>(), dCholItems64_.as<CholItem>() + st.off,
                                  st.count, dCholSync64_.as<int>(), st.elems, dCholWs64_.as<double>(),
                                  dFlag.as<int>(), nullptr, stream);
        break;
    }
    if (timing) RSCHOL_CUDA(cudaEventRecordWithFlags(stepEv_[2 * q + 1], stream, recFlags));
    ++launches;
  }
  if (post) launches += post();
}

template <class T>
int FactorEngine<T>::run() {
  if (!planned_) plan();
  const bool timing = timeSteps && !steps_.empty();
  if (timing && stepEv_.size() < 2 * steps_.size()) {
    drop_graphs();   // the timing graph records the events it was captured with
    for (auto e : stepEv_) cudaEventDestroy(e);
    stepEv_.assign(2 * steps_.size(), nullptr);
    for (auto& e : stepEv_) RSCHOL_CUDA(cudaEventCreate(&e));
  }
  // the first run of a plan is queued directly (one-time kernel attributes
  // are set outside any capture); later runs replay a captured graph
  const int g = timing ? 1 : 0;
  if (useGraphs_ && runsSincePlan_ > 0) {
    if (!graph_[g]) {
      RSCHOL_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      cudaGraph_t graph = nullptr;
      try {
        enqueue(timing, true);
      } catch (...) {
        cudaStreamEndCapture(stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
      }
      RSCHOL_CUDA(cudaStreamEndCapture(stream, &graph));
      const cudaError_t e = cudaGraphInstantiate(&graph_[g], graph, 0);
      cudaGraphDestroy(graph);
      RSCHOL_CUDA(e);
      graphLaunches_[g] = launches;
    }
    RSCHOL_CUDA(cudaGraphLaunch(graph_[g], stream));
    launches = graphLaunches_[g];
  } else {
    enqueue(timing, false);
  }
  ++runsSincePlan_;
  int flag[2] = {0, 0};
  RSCHOL_CUDA(cudaMemcpyAsync(flag, dFlag.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
  RSCHOL_CUDA(cudaStreamSynchronize(stream));
  if (timing) {
    for (size_t q = 0; q < steps_.size(); ++q) {
      float ms = 0;
      RSCHOL_CUDA(cudaEventElapsedTime(&ms, stepEv_[2 * q], stepEv_[2 * q + 1]));
      // per-kind totals: split-K sums with the GEMMs, the FP64 root's
      // conversions in slot 6, its Cholesky with the fused Cholesky
      const int kd = steps_[q].kind;
      const int k = kd == ST_GEMM_REDUCE ? (int)ST_GEMM : kd == ST_CVT ? 6 : kd == ST_CHOL64 ? (int)ST_CHOL : kd;
      stepMs[k] += ms;
      stepCount[k] += 1;
      stepFlops[k] += steps_[q].flops;
    }
    for (const Step& st : steps_)
      if (st.kind == ST_GEMM)
        for (int k = 0; k < st.count; ++k) {
          const GemmTask<T>& gt = gemm_[st.off + k];
          stepFlops[ST_GEMM] += 2.0 * gt.M * gt.N * (double)gt.K;
        }
    // RSCHOL_STEP_LOG=1: every step of this run on stderr (kind, tasks, grid,
    // device ms; GEMM: flops and largest M / N / K) for tuning the schedule
    const char* sl = std::getenv("RSCHOL_STEP_LOG");
    if (sl && sl[0] == '1') {
      static const char* names[] = {"gemm", "potrf", "trsm", "extadd", "qr", "ident", "reduce", "chol", "cvt", "chol64"};
      for (size_t q = 0; q < steps_.size(); ++q) {
        const Step& st = steps_[q];
        float ms = 0;
        RSCHOL_CUDA(cudaEventElapsedTime(&ms, stepEv_[2 * q], stepEv_[2 * q + 1]));
        double f = 0;
        int mM = 0, mN = 0, mK = 0;
        if (st.kind == ST_GEMM)
          for (int k = 0; k < st.count; ++k) {
            const GemmTask<T>& g = gemm_[st.off + k];
            f += 2.0 * g.M * g.N * (double)g.K;
            mM = std::max(mM, g.M);
            mN = std::max(mN, g.N);
            mK = std::max(mK, g.K);
          }
        std::fprintf(stderr, "step %zu %s tasks %d grid %d aux %d us %.1f gflop %.4f M %d N %d K %d\n", q,
                     names[st.kind], st.count, st.grid, st.aux, 1e3 * ms, f * 1e-9, mM, mN, mK);
      }
    }
  }
  const char* tracePath = std::getenv("RSCHOL_CHOL_TRACE");
  if (dCholTrace_.p && tracePath && tracePath[0]) {   // one line per item of the fused steps of this run
    std::vector<unsigned long long> tr(4 * cholItems_.size());
    RSCHOL_CUDA(cudaMemcpy(tr.data(), dCholTrace_.p, tr.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    if (FILE* fp = std::fopen(tracePath, "w")) {
      for (size_t q = 0; q < steps_.size(); ++q) {
        const Step& st = steps_[q];
        if (st.kind != ST_CHOL) continue;
        for (int t = 0; t < st.count; ++t) {
          const CholItem& it = cholItems_[st.off + t];
          const unsigned long long* r = &tr[4 * (st.off + t)];
          std::fprintf(fp, "%zu %d %d %d %d %d %d %llu %llu %llu %llu\n", q, t, it.job, it.kind, it.p, it.a, it.b,
                       r[0], r[1], r[2], r[3]);
        }
      }
      std::fclose(fp);
    }
  }
  if (flag[1] == 2) throw CudaError("fused Cholesky: ticket counter out of range");
  if (flag[1]) throw FactorWaitTimeout("factor: a bounded wait (tensor-core mbarrier or tile counter) exceeded its limit");
  return flag[0] == INT_MAX ? 0 : flag[0];
}

template class FactorEngine<double>;
template class FactorEngine<float>;

}  // namespace rschol
