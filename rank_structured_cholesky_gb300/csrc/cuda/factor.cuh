// Numeric factorisation on the GPU as a static, level-batched schedule.
//
// Mathematics (the same preconditioner as the reference's
// FactorManager::factorNumeric, src/rschol/solver/FactorManager.cpp:357-804):
//   * interior blocks (maximal runs of uncompressed supernodes) are exact
//     sparse Cholesky factors.  They are computed multifrontally: each front
//     carries all of its supernode's rows, so the root fronts of every
//     interior subtree end with the exact Schur-complement contribution
//     L_{R,I} L_{R,I}^T of that subtree to the compressed supernodes.  The
//     reference applies the same contribution implicitly as
//     A_{R,I} L_I^{-T} L_I^{-1} A_{I,C} (FactorManager.cpp:10792-11088);
//   * each compressed supernode j assembles the dense Schur complement
//     [S11; S21] from A, those interior contributions and its compressed
//     descendants' V (U^T U) V^T, factors S11 (dense or HODLR: explicit
//     builds compress the blocks of the exact factor, recursive builds
//     sketch S_ba L_aa^{-T}), forms L21 = S21 L11^{-T} and runs the
//     reference's randomized range finder on it (Gaussian G from the
//     reseeded Mersenne Twister stream, one power iteration, thin QR,
//     V = L21 U), as blockRandomMultiply_allRows + fixedOffDiagonalDecomposition
//     + fullBasisProject_transpose_allRows (FactorManager.cpp:8193-8297,
//     8717-8780, 5691-5751).
// All supernodes of one level (interior: height in the elimination tree,
// compressed: height among compressed supernodes) are processed by one
// batched launch per phase.  The schedule is built once on the host and
// replayed for every (re)factorisation.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <functional>
#include <map>
#include <vector>

#include "../host/ordering.h"
#include "../host/symbolic.h"
#include "common.cuh"
#include "dense.cuh"

namespace rschol {

enum StepKind : int {
  ST_GEMM = 0,
  ST_POTRF,
  ST_TRSM,
  ST_EXTADD,
  ST_QR,
  ST_IDENT,
  ST_GEMM_REDUCE,   // sum the K-slice partials of the split tensor-core GEMM tasks
  ST_CHOL,          // fused blocked partial Cholesky of a level (POTRF + TRSM + updates, one launch)
  ST_CVT,           // root separator blocks FP32 -> FP64 scratch (aux 1) or back (aux 0); grid: largest block
  ST_CHOL64,        // fused blocked Cholesky of root separator blocks in FP64 (mixed factor with root_fp64)
};

struct Step {
  int kind;
  long long off;    // first task in the kind's task array
  int count;        // number of tasks
  int grid;         // tiles / chunks / columns for the launch
  int aux = 0;      // ST_QR: largest row count of the batch (grid: largest rank);
                    // ST_GEMM: the tile width bn on the tensor cores, 0 on the SIMT kernel
  long long elems = 0;   // ST_GEMM_REDUCE: elements of C summed; ST_CHOL: ints of its counters
  double flops = 0;      // ST_CHOL: algorithmic flops of the launch
  double bytes = 0;      // ST_CHOL: algorithmic bytes (each job's lower region read once and written once)
};

template <class T>
struct CholJob {   // blocked partial Cholesky of F's first nDiag columns
  T* F;
  int ld, nDiag, nRows, nUpd, code;
};

template <class T>
struct TrsmJob {   // B (rows x w) := B L^{-T}
  const T* L;
  T* B;
  int ldl, ldb, rows, w;
};

template <class T>
struct RFJob {     // randomized range finder on the dense block F (rows x cols)
  T* F;
  int ld, rows, cols, r;
  const T* G;      // rows x r Gaussian sketch
  T* Y;            // cols x r: sketch, then the orthonormal basis U
  T* X;            // rows x r scratch
  T* W;            // cols x r + r scratch of the Householder QR
  T* V;            // rows x r
  T* Q;            // r x r: U^T U (may be null)
  bool identity;   // r >= cols: U = I (FactorManager.cpp:9598-9606)
  bool expand;     // overwrite F with V U^T (HODLR block of L11)
};

template <class T>
class FactorEngine {
 public:
  FactorEngine(const Symbolic& S, const CSC& Alower, const Params& prm, cudaStream_t stream);
  ~FactorEngine() {
    drop_graphs();
    for (auto e : stepEv_) cudaEventDestroy(e);
  }

  // (Re)build buffers and schedule for the ranks currently in S.
  void plan();
  // Upload new lower-triangle values (same pattern as Alower).
  void set_values(const double* lowerVals);
  // Run the numeric factorisation; returns 0 or the failing POTRF code.
  int run();

  // --- factor data for the solve and for introspection
  const Symbolic& S;
  const CSC& A;
  Params prm;
  cudaStream_t stream;

  std::vector<long long> frontOff;    // element offset (interior / compressed arena)
  std::vector<int> ld;                // front leading dimension
  std::vector<int> rank;              // off-diagonal rank of compressed supernodes
  std::vector<long long> vOff, uOff, qOff;
  DevBuf dInterior, dCompressed, dVU, dHodlr, dContrib, dGauss, dAvals, dFlag;
  T* interior() const { return dInterior.as<T>(); }
  T* compressed() const { return dCompressed.as<T>(); }
  T* vu() const { return dVU.as<T>(); }

  std::vector<std::vector<int>> interiorLevels, compressedLevels;
  // Work queued on the stream after the last factor step and before the
  // status read (solve-side preprocessing of the factor); returns its launches.
  std::function<int()> post;
  // Per-step CUDA-event timing (off by default): accumulated device time,
  // launches and GEMM flops per step kind over the runs made while on.
  bool timeSteps = false;
  double stepMs[8] = {}, stepCount[8] = {}, stepFlops[8] = {};
  long long launches = 0;            // kernel launches of the last run
  double flops = 0;                  // algorithmic flops of one factorisation
  size_t deviceBytes = 0;

 private:
  void emit_chol(const std::vector<CholJob<T>>& jobs);
  void emit_chol_t(const std::vector<CholJob<T>>& jobs);
  template <class U>
  void emit_fused(const std::vector<CholJob<U>>& jobs, int kind, std::vector<CholFusedJob<U>>& cjobs,
                  std::vector<CholItem>& items, long long& syncMax, long long& wsMax);
  void emit_trsm(const std::vector<TrsmJob<T>>& jobs);
  // L21 = S21 L11^{-T} of large compressed supernodes: column blocks of
  // L21_BLOCK, each a fused TRSM chain against its diagonal block followed by
  // one tensor-core GEMM step for the columns right of it (FP32 with tensor
  // cores; otherwise emit_trsm)
  void emit_l21(const std::vector<TrsmJob<T>>& jobs);
  void emit_rf(const std::vector<RFJob<T>>& jobs);
  struct EaSrc {            // plan-time source of an extend-add
    ExtAddSource<T> s;      // rowRel filled from relOff
    size_t relOff;          // target index of each source row, in ints_
    int aLo, aHi;           // source rows that feed the target
  };
  struct EaTarget {
    T* F;
    int ld, rows;
    std::vector<EaSrc> src;
  };
  void emit_extadd(const std::vector<EaTarget>& tgs);
  void push_gemm(const GemmTask<T>& t, int& tiles, std::vector<GemmTask<T>>& batch);
  void flush_gemm(std::vector<GemmTask<T>>& batch, int tiles);
  void gemm1(const GemmTask<T>& t);   // a single-task GEMM step
  void gemm_launch(const Step& st);    // SIMT kernel, or the tensor cores for FP32
  bool useTc_ = false;
  int tcMinK_ = 128;

 public:
  bool tensor_cores() const { return useTc_; }   // FP32 GEMMs on tcgen05
  // Schedule options timed by the factor tuner (taking effect at the next
  // plan()): FP32 GEMM steps go to the tensor cores from K >= tcMinK
  // (INT_MAX: never); fused level launches for the blocked Cholesky and TRSM
  // chains, or one launch per 64-column panel.
  void set_schedule(int tcMinK, bool fused) {
    tcMinK_ = tcMinK;
    fusedChol_ = fused;
  }
  int tc_min_k() const { return tcMinK_; }
  bool fused_chol() const { return fusedChol_; }

  std::vector<Step> steps_;
  std::vector<cudaEvent_t> stepEv_;
  std::vector<GemmTask<T>> gemm_;
  std::vector<PotrfTask<T>> potrf_;
  std::vector<TrsmTask<T>> trsm_;
  std::vector<ExtAddRow<T>> eaR_;
  std::vector<ExtAddSeg> eaSeg_;
  std::vector<ExtAddSource<T>> eaS_;
  std::vector<QrTask<T>> qr_;
  std::vector<IdentTask<T>> ident_;
  std::vector<int> ints_;
  std::vector<long long> gemmWsOff_;       // per GEMM task: offset of its K-slice partials, or -1
  std::vector<int> splitIds_;              // ST_GEMM_REDUCE: GEMM task ids
  std::vector<long long> splitBase_;       // ST_GEMM_REDUCE: element prefix sums (nIds + 1 per step)
  long long wsCur_ = 0;
  DevBuf dSplitWs_, dSplitIds_, dSplitBase_;
  long long qrWs_ = 0;   // elements of the Householder QR workspace (largest QR step)
  DevBuf dQrWs_;
  // The blocked Cholesky of each emit_chol call, and the blocked TRSM of each
  // emit_trsm call, as one ticketed launch (RSCHOL_FUSED_CHOL=0 keeps the
  // POTRF / TRSM / GEMM steps per panel).
  bool fusedChol_ = false;
  std::vector<CholFusedJob<T>> cholJobs_;
  std::vector<CholItem> cholItems_;
  long long cholSync_ = 0, cholWs_ = 0;   // largest counter array (ints) and inverse workspace (elements) of a step
  DevBuf dCholJobs_, dCholItems_, dCholSync_, dCholWs_, dCholTrace_;
  // Mixed factor with Params::root_fp64: the dense Cholesky of the root
  // separator's blocks runs in FP64 on scratch copies (per root supernode, an
  // n x n FP64 matrix at rootStart_[node] in dRoot64_).
  std::map<int, long long> rootStart_;
  DevBuf dRoot64_, dCvt_;
  std::vector<CvtTask> cvt_;
  std::vector<CholFusedJob<double>> cholJobs64_;
  std::vector<CholItem> cholItems64_;
  long long cholSync64_ = 0, cholWs64_ = 0;
  DevBuf dCholJobs64_, dCholItems64_, dCholSync64_, dCholWs64_;
  std::vector<long long> scatSrc_, scatDst_;
  std::vector<int> scatIsInterior_;
  DevBuf dTmaps_;   // TMA tensor maps of the tensor-core GEMM tasks
  DevBuf dGemm_, dPotrf_, dTrsm_, dEaR_, dEaSeg_, dEaS_, dQr_, dIdent_, dInts_, dScatSrc_, dScatDst_;
  DevBuf dScatSrcC_, dScatDstC_;
  long long nScatI_ = 0, nScatC_ = 0;
  bool planned_ = false;
  // Polls before a bounded wait of the fused Cholesky gives up
  // (RSCHOL_WAIT_LIMIT, default solvedev::SPIN_LIMIT).  The test switch
  // RSCHOL_TEST_DROP_CHOL_ITEM=1 leaves the first POTRF item that TRSM items
  // depend on out of the plan, so that their waits run out: it exercises the
  // give-up path (RSCHOL_E_TIMEOUT, context still usable) and nothing else.
  int waitLimit_ = 0;
  bool dropItemTest_ = false, droppedItem_ = false;
  // The schedule is static per plan: from the second run of a plan on, the
  // whole factorisation (and the solve-side preparation queued by post) is
  // replayed from a CUDA graph captured once; [1] is the variant with the
  // per-step timing events.  Off with RSCHOL_GRAPHS=0.
  bool useGraphs_ = true;
  int runsSincePlan_ = 0;
  cudaGraphExec_t graph_[2] = {nullptr, nullptr};
  long long graphLaunches_[2] = {0, 0};
  void drop_graphs();
  void enqueue(bool timing, bool capturing);
};

}  // namespace rschol
