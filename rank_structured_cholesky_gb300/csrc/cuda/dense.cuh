// Batched dense building blocks of the numeric factorisation.
//
// Every launch carries an array of independent tasks (one per front, per
// tile column, ...) so that all supernodes of one elimination-tree level,
// whatever their sizes, are processed by a single launch.  The reference
// issues one CBLAS/LAPACKE call per supernode instead
// (src/rschol/linearalgebra/MATRIX_FAST.cpp:1758 gemm, 1885 syrk, 2086
// cholesky, 3049 triangularSolve).
#pragma once
#include <type_traits>
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace rschol {

// C (M x N) = alpha * op(A) * op(B) + beta * C, row-major, leading dims.
// lower != 0: tiles strictly above the diagonal of C are skipped (the
// caller only reads C's lower triangle).
template <class T>
struct GemmTask {
  const T* A;
  const T* B;
  T* C;
  int M, N, K;
  int lda, ldb, ldc;
  int tA, tB, lower;
  T alpha, beta;
  int tilesN;
  int tileBase;   // first tile of this task in the launch
  int split;      // tensor-core path: split-precision (3 x TF32) products
  int kSplit;     // tensor-core path: K slices (1: none); slices write partials to ws
  int kLen;       // K per slice (a multiple of 32)
  float* ws;      // kSplit x tiles x 128 x bn partials (kSplit > 1)
  int bn;         // tensor-core path: output tile width of the launch (64 or 128; 0: 64)
  // tensor-core path: device addresses of the TMA tensor maps of A and B
  // (K-major operands, 16-byte aligned), or null for register staging
  const void* tmA;
  const void* tmB;
};

// One TMA tensor map (the driver's 128-byte CUtensorMap, opaque here).
struct alignas(64) TensorMapBytes {
  unsigned char b[128];
};

// In-place lower Cholesky of one diagonal tile (n <= 64).  On a
// non-positive pivot *flag receives min(*flag, code).
template <class T>
struct PotrfTask {
  T* A;
  int ld, n;
  int code;
};

// B (rows x w) := B * L^{-T}, L the w x w (w <= 64) lower tile.  A launch
// block takes trsm_rows<T>() rows; chunkBase counts such blocks.  (FP32
// blocks of 256 rows sharing one tile inverse measured slower than 64: the
// launches lose more parallelism than the repeated inverses cost.)
constexpr int TRSM_ROWS_F32 = 64;
template <class T>
constexpr int trsm_rows() { return std::is_same<T, float>::value ? TRSM_ROWS_F32 : 64; }
template <class T>
struct TrsmTask {
  const T* L;
  T* B;
  int ldl, ldb, w, rows;
  int chunkBase;  // first 64-row chunk of this task in the launch
};

// Blocked partial Cholesky of several fronts in one launch (tile-level
// dependencies, ticketed work items): job = the first nDiag columns of the
// nRows x nRows lower front F; trailing updates reach the columns below nUpd.
// Panels: the first w0 = nDiag - 64 (P - 1) wide, then 64; tile t spans rows
// [b(t), b(t + 1)), b(0) = 0, b(t) = w0 + 64 (t - 1); TR / TU tiles cover
// nRows / nUpd.
// A TRSM job (L != null) is the same launch's B := B L^{-T} for a factored
// w x w lower L (ld ldl) and F = B (nRows x w, ld): "POTRF" items only
// invert L's diagonal tiles (no wait), the updates are X(a) L(b, p)^T, and B's
// rows are cut at 0, r1 = 64, 128, ... (a Cholesky job has r1 = w0).
template <class T>
struct CholFusedJob {
  T* F;
  int ld, nDiag, nRows, nUpd, code;
  int w0, P, TR, TU;
  int cnt;          // offset of the job's TR x TU + TR + P counters after the ticket
  long long inv;    // element offset of the job's P inverse tiles (64 x 64) in the workspace
  const T* L;       // TRSM job: the factored triangle (null for a Cholesky job)
  int ldl, r1;      // r1: height of the first row tile
};
constexpr int CHOL_POTRF = 0, CHOL_TRSM = 1, CHOL_GEMM = 2;
struct CholItem {   // one piece of panel p: POTRF, TRSM of row tile a, update of tile (a, b)
  int job, kind, p, a, b;
};
// sync: syncInts ints (zeroed here, on the stream, before the launch); ws:
// the jobs' inverse tiles; flag[0]: min code of a failed pivot, flag[1]: set
// when a bounded wait gives up, flag[2]: polls before a wait gives up.  trace (diagnostics, may be null): 4 values
// per item -- start, dependencies met, end (ns of the global timer), SM.
template <class T>
void launch_chol_fused(const CholFusedJob<T>* jobs, const CholItem* items, int nItems, int* sync, long long syncInts,
                       T* ws, int* flag, unsigned long long* trace, cudaStream_t s);

// Extend-add "pull" by target row: a warp owns one target row and adds the
// rows of its sources in a fixed order (deterministic, no atomics).  Source
// row a, columns b in [b0, min(b1, a + 1)) (the lower part of a symmetric
// update block), lands on target row rowRel[a], columns rowRel[b]; reads of
// the source row and writes of the target row are both contiguous.
template <class T>
struct ExtAddSource {
  const T* D;          // source block (row-major)
  const int* rowRel;   // target index (row or column) of each source row / column
  int ld;
  int b0, b1;          // source columns that land in the target's columns
  T sign;
};

struct ExtAddSeg {     // one source row feeding a target row
  int src, a;
};

template <class T>
struct ExtAddRow {
  T* Frow;             // target row
  int segBegin, segEnd;
};

template <class T> void launch_gemm(const GemmTask<T>* dTasks, int nTasks, int totalTiles, cudaStream_t s);
// The lower triangle of an n x n FP32 block (leading dimension ld) to FP64
// scratch (leading dimension ldd) when toDouble, else back.
struct CvtTask {
  float* F;
  double* D;
  int ld, ldd, n;
};
void launch_block_convert(const CvtTask* dTasks, int nTasks, int maxN, int toDouble, cudaStream_t s);
// FP32 tasks on the tensor cores (tcgen05, TF32 or split TF32), 128 x bn
// output tiles, bn = 64 or 128 for the whole launch (tileBase / tilesN counted
// for that width; every task's bn equal to it); *dErr is set if an mbarrier
// wait gives up.  bf16: the launch's operands as BF16 (split tasks: hi/lo,
// three kind::f16 MMAs; K slices of split tasks a multiple of 64).
void launch_gemm_tc(const GemmTask<float>* dTasks, int nTasks, int totalTiles, int* dErr, cudaStream_t s,
                    int bn = 64, int bf16 = 0);
// Host: TMA tensor maps for the tasks of one TF32 tensor-core launch of tile
// width bn whose operands allow it (A M x K and B N x K row-major, both
// 16-byte aligned with leading dimensions a multiple of 4 floats).  The maps
// are appended to `maps`; such a task's tmA / tmB are set to 1 + the map's
// index, for the caller to rebase to the maps' device addresses.  Returns how
// many tasks got maps (0 when the driver entry point is missing or
// RSCHOL_TMA=0).
int encode_gemm_tmaps(GemmTask<float>* tasks, int count, int bn, std::vector<TensorMapBytes>& maps);
// The tile width of a tensor-core launch whose widest task has N columns.
inline int tc_tile_n(int maxN) { return maxN > 64 ? 128 : 64; }
// C = alpha * sum of the K-slice partials + beta * C for the split tasks
// ids[0..nIds) (elemBase: prefix sums of their M x N, elemBase[nIds] = elems).
void launch_gemm_splitk_reduce(const GemmTask<float>* dTasks, const int* ids, int nIds, const long long* elemBase,
                               long long elems, cudaStream_t s);
template <class T> void launch_potrf(const PotrfTask<T>* dTasks, int nTasks, int* dFlag, cudaStream_t s);
template <class T> void launch_trsm(const TrsmTask<T>* dTasks, int nTasks, int totalChunks, cudaStream_t s);
template <class T>
void launch_extadd(const ExtAddRow<T>* dRows, int nRows, const ExtAddSeg* dSegs, const ExtAddSource<T>* dSources,
                   cudaStream_t s);
// flag[0] = INT_MAX (no POTRF failure yet), flag[1] = 0 (no tensor-core wait error)
// flag[0] = INT_MAX (no failed pivot), flag[1] = 0 (no wait gave up),
// flag[2] = waitLimit (polls before a fused-Cholesky wait gives up).
void launch_init_flags(int* flag, int waitLimit, cudaStream_t s);
template <class T>
void launch_scatter(const double* Avals, const long long* srcIdx, const long long* dstIdx, long long count,
                    T* dst, cudaStream_t s);
// Thin Householder QR, Y (n x r, row-major, r < n) := Q: the LAPACK
// geqrf + orgqr pair the reference calls (MATRIX::qr / extractQRfactor,
// src/rschol/linearalgebra/MATRIX_FAST.cpp:1095-1180), blocked in panels of
// 16 columns (compact WY).  W is an n x r column-major scratch (the
// reflectors and the panels' T factors).  maxRows / maxR bound n and r over
// the batch.  Returns the number of launches.
template <class T>
struct QrTask {
  T* Y;
  T* W;
  int n, r;
};
template <class T>
int launch_householder_qr(const QrTask<T>* dTasks, int nTasks, int maxRows, int maxR, T* ws, cudaStream_t s);
// elements of the workspace launch_householder_qr needs for such a batch
long long householder_qr_workspace(int nTasks, int maxRows, int maxR);
template <class T>
struct IdentTask {
  T* U;
  int n, ld;
};
template <class T> void launch_set_identity(const IdentTask<T>* dTasks, int nTasks, cudaStream_t s);
// Box-Muller on pairs of raw 32-bit Mersenne Twister draws.
template <class T>
void launch_box_muller(const uint32_t* raw, long long count, T* out, cudaStream_t s);

}  // namespace rschol
