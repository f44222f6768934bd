// Internal interfaces shared by the CUDA translation units of librgf_gb300.
#pragma once

#include <vector>

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace rgf {

// Lives in device memory, one per handle.  Kernels record failures here
// instead of trapping; the host reads it after each stage.
struct DevStatus {
  int not_spd_col;   // smallest global column with a non-positive pivot (INT32_MAX: none)
  int bad_input;     // ingest saw an entry outside the block pattern
  int timeout;       // a bounded device-side wait gave up
  int pad;
};

// ---- programmatic dependent launch -------------------------------------------
// Kernels are launched with programmatic stream serialization (launch_k): the
// next kernel in a stream may be scheduled once every CTA of the running one
// has called pdl_trigger() (placed after each kernel's main loop, so the next
// kernel's CTAs become resident during the tail instead of after it), and
// every kernel calls pdl_wait() before its first global memory access, which
// returns once the previous kernel in the stream has completed and its writes
// are visible.  Both are no-ops in a kernel launched without the attribute.
// RGF_GB300_PDL=0 launches without it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

bool pdl_enabled();

template <typename... KArgs, typename... Args>
inline void launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                     Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  // created streams only: not the default streams (the legacy one synchronizes
  // with every stream)
  cfg.numAttrs =
      pdl_enabled() && s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kern, args...);  // a failure stays the pending launch error
}

enum Tri { TRI_NONE = 0, TRI_LOWER = 1, TRI_UPPER = 2 };

// D = alpha * op(A) * op(B) + beta * C, column-major, op(A) m x k, op(B) k x n.
// triA/triB declare a triangular operand (of op(X)); its other triangle is
// treated as zero whatever memory holds.  outLower writes only r >= c.
// batch > 1 runs independent problems offset by sA/sB/sC/sD elements.
struct GemmDesc {
  int m = 0, n = 0, k = 0;
  const double* A = nullptr; long long lda = 0; int transA = 0;
  // Rows >= mA1 of A come from A2 (row r at A2 + (r - mA1), same lda and
  // batch stride): a stacked operand whose two row blocks are not adjacent
  // in memory.  transA == 0 only; A2 == nullptr means one block.
  const double* A2 = nullptr; int mA1 = 0;
  // Rows >= mD1 of C and D live at C2 / D2 (row r at D2 + (r - mD1), same
  // leading dimensions and batch strides); D2 == nullptr means one block.
  const double* C2 = nullptr; double* D2 = nullptr; int mD1 = 0;
  const double* B = nullptr; long long ldb = 0; int transB = 0;
  const double* C = nullptr; long long ldc = 0;
  double* D = nullptr; long long ldd = 0;
  double alpha = 1.0, beta = 0.0;
  int triA = TRI_NONE, triB = TRI_NONE, outLower = 0;
  int batch = 1;
  long long sA = 0, sB = 0, sC = 0, sD = 0;
  // FP64 kernel only: workspace for split-K partial sums (used when a single
  // problem has too few output tiles to fill the GPU); ksplit is set by the
  // launcher.
  double* ws = nullptr;
  long long ws_elems = 0;
  int ksplit = 1;
  int tile = 0;  // FP64 kernel: output tile 32 or 64; 0 = chosen by the launcher
};

// Algorithmic flops of one GemmDesc (triangular operands and lower-only
// outputs counted at their LAPACK sizes).
double gemm_flops(const GemmDesc& g);

// ---- complex Hermitian matrices (hermitian.cu) -------------------------------
// Lower CSC of the real symmetric embedding [[X, -Y], [Y, X]] of the Hermitian
// A = X + iY given as its lower CSC (a: interleaved re, im), ordered so that it
// is a BTA matrix with (2ns, nt, 2nd).
int hermitian_embed(const size_t* ia, const size_t* ja, const double* a, size_t ns, size_t nt,
                    size_t nd, std::vector<size_t>& ia2, std::vector<size_t>& ja2,
                    std::vector<double>& a2);
// Real index of Re (imag = 0) or Im (imag = 1) of complex unknown k.
size_t hermitian_real_index(size_t ns, size_t nt, size_t nd, size_t k, int imag);

// ---- FP64 kernels (k_fp64.cu) ---------------------------------------------
// Returns the number of kernels launched (2 with split-K).
int launch_gemm_fp64(const GemmDesc& g, cudaStream_t s);

// Cholesky of the nbk x nbk (nbk <= 64) lower tile at T (column-major, ldt),
// in place.  Records the first non-positive pivot (global column col0 + j) in st.
// Each wait of a column for the previous pivot polls at most wait_polls times
// (0 = LEAF_WAIT_POLLS); a wait that runs out records a timeout in st and the
// leaf stops updating.
constexpr int LEAF_WAIT_POLLS = 1 << 26;
void launch_leaf_potrf(double* T, long long ldt, int nbk, int col0, DevStatus* st,
                       cudaStream_t s, int wait_polls = 0);

// Every device allocation of the library goes through here (so that a test
// can make one fail: rgf_debug_fail_alloc_after).  cudaMalloc semantics.
// On a thread that has a device arena set (set_thread_arena), memory comes
// from the arena instead, with no cudaMalloc (and device_free returns it
// there, with no cudaFree and its device-wide wait).
cudaError_t device_malloc(void** p, size_t bytes);
void device_free(void* p);

// A device arena: one cudaMalloc of `bytes` at creation, then first-fit
// sub-allocation (256-byte aligned, neighbours merged on free) under a mutex.
// When it cannot serve a request (full or fragmented) device_malloc falls back
// to cudaMalloc and counts it.
struct DeviceArena;
DeviceArena* arena_create(size_t bytes, int* status);
void arena_destroy(DeviceArena* a);
void set_thread_arena(DeviceArena* a);
long long arena_fallbacks(DeviceArena* a);
size_t arena_in_use(DeviceArena* a);

// Row-parallel triangular solve with an nbk x nbk (nbk <= 64) lower tile L:
//   mode 0: X := X * L^{-T}   (forward,  "R L T N")
//   mode 1: X := X * L^{-1}   (backward, "R L N N")
// X has `rows` independent rows; element (r, j) at X[r*xrs + j*xcs].
// batch > 1: problem b uses X + b*sX, L + b*sL.
void launch_trsm_rows(double* X, long long xrs, long long xcs, int rows, const double* L,
                      long long ldl, int nbk, int mode, int batch, long long sX, long long sL,
                      cudaStream_t s);

// Measured FP64 (DMMA) throughput of the current device in TFLOP/s.
int measure_fp64_peak(double* tflops);

// ---- small kernels (k_misc.cu) ------------------------------------------------
struct BtaShape {
  long long ns, nt, nd, n;
};
long long mf_col_offset(const BtaShape& sh, long long i);
long long mf_lda(const BtaShape& sh, long long i);
long long mf_dense_row(const BtaShape& sh, long long i);

// Scatter the device CSC into the (pre-zeroed) MF layout; one warp per column.
// Columns [c_lo, c_hi) only (c_hi < 0: to the last column): every entry of a
// column lands in its own block column's panel.
void launch_ingest(const BtaShape& sh, const size_t* ia, const size_t* ja, const double* a,
                   double* MF, DevStatus* st, cudaStream_t s, long long c_lo = 0,
                   long long c_hi = -1);
// Sum of nparts partial log sums, times 2, in a fixed order -> *out.
// *out = 2 sum(log diag(L)) over the factor MF: per-block sums into parts
// (logdet_parts(sh) of them), then a fixed-order total.
int logdet_parts(const BtaShape& sh);
void launch_logdet(const BtaShape& sh, const double* MF, double* parts, double* out,
                   cudaStream_t s);
// diag[k] = MS[diag position of k] for all k < n.
void launch_extract_diag(const BtaShape& sh, const double* MS, double* diag, cudaStream_t s);
// batch of identity matrices (m x m, ld) at X + b*stride
void launch_set_identity(double* X, long long ld, int m, int batch, long long stride,
                         cudaStream_t s);
// Y (m x n, ldy) = X (m x n, ldx); batched
// Upper triangle of the symmetric n x n matrix X from its lower triangle.
void launch_mirror_lower(double* X, long long ld, int n, cudaStream_t s);
void launch_copy(const double* X, long long ldx, double* Y, long long ldy, int m, int n,
                 int batch, long long sX, long long sY, cudaStream_t s);
// r = b - A x (symmetric, from the lower CSC) for the first column; then
// out[0] = ||r||_2, out[1] = ||b||_2 (scaled sums of squares, as dnrm2).
// scratch: n doubles.  CSC entries outside the lower triangle or past row n-1
// are skipped; with `bad` (device int, may be null) they set *bad and both
// outputs become NaN.  Returns the first launch error (the caller's pending
// errors are the caller's to check first).
cudaError_t launch_residual(long long n, const size_t* ia, const size_t* ja, const double* a,
                            const double* x, const double* b, double* scratch, double* out,
                            int* bad, cudaStream_t s);
// R = B - A X for nrhs columns (ld n) from the lower CSC; Y is n*nrhs scratch
void launch_residual_vectors(long long n, int nrhs, const size_t* ia, const size_t* ja,
                             const double* a, const double* X, const double* B, double* Y,
                             double* R, cudaStream_t s);
// out[2q] = ||R[:, q]||_2, out[2q + 1] = ||B[:, q]||_2 (columns n apart,
// scaled sums of squares) for q < nrhs.
void launch_rhs_norms(long long n, int nrhs, const double* R, const double* B, double* out,
                      cudaStream_t s);
// right-hand sides per pass of the multi-RHS SpMV of launch_residual_vectors
constexpr int SPMV_MAX_RHS = 16;
// x += d over len entries
void launch_add(long long len, double* x, const double* d, cudaStream_t s);
// out[q*ldo + dd] = sum_i sum_j C_i(dd, j) * R_i(j, q) over block columns,
// computed as per-block partials then an ordered sum: the arrowhead part of
// the forward solve.  y_d -= that.
void launch_arrow_gemv(const BtaShape& sh, const double* MF, const double* rhs, long long ldr,
                       int nrhs, double* partial, cudaStream_t s);
void launch_arrow_reduce(const BtaShape& sh, const double* partial, int nrhs, double* rhs,
                         long long ldr, cudaStream_t s);

}  // namespace rgf
