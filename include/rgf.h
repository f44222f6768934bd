/*
 * rgf.h -- C ABI of the GB300-native RGF solver (sm_103a).
 *
 * Solves with a symmetric positive-definite block-tridiagonal-arrowhead
 * matrix of size n = ns*nt + nd, given as its lower triangle in CSC form
 * with size_t indices (ia: n+1 column pointers, ja: row indices, row >= col,
 * a: values).  This is the input of the reference class
 *     RGF<double>::RGF(size_t *ia, size_t *ja, double *a,
 *                      size_t ns, size_t nt, size_t nd)      (RGF.H:84-146)
 *
 * Every entry point returns an int status (enum rgf_status).  Host pointers
 * are plain host memory (pageable or pinned); device memory is owned by the
 * handle.  One call at a time per handle; different handles may be used from
 * different host threads.  All computation runs on the GPU: there is no CPU
 * fallback, and a missing or unusable device is reported as RGF_ECUDA.
 */
#ifndef RGF_GB300_RGF_H
#define RGF_GB300_RGF_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum rgf_status {
  RGF_OK = 0,
  RGF_EINVAL = 1,    /* bad argument or CSC outside the block pattern        */
  RGF_ENOMEM = 2,    /* device allocation failed                              */
  RGF_ENOTSPD = 3,   /* non-positive pivot: matrix not positive definite      */
  RGF_ECUDA = 4,     /* CUDA runtime error / no usable device                 */
  RGF_ETIMEOUT = 5,  /* a bounded device-side wait gave up                    */
  RGF_ENOTSUP = 6    /* option not supported by this build                    */
};

enum rgf_precision {
  RGF_PREC_FP64 = 0,   /* every operation in FP64                             */
  RGF_PREC_SPLIT = 1   /* bulk GEMMs as bf16 slice products on tcgen05 tensor
                          cores (Ozaki scheme), FP64 elsewhere                */
};

enum rgf_selinv_mode {
  RGF_SELINV_EXACT = 0,  /* exact block selected inversion                    */
  RGF_SELINV_COMPAT = 1  /* the reference's recursion (RGF.H:422-506), which
                            omits the arrowhead cross terms when nd > 0       */
};

typedef struct rgf_opts {
  int precision;    /* enum rgf_precision (default RGF_PREC_FP64)             */
  int slices;       /* split precision: 8-bit slices per operand (1..8),
                       0 = default 5 (40-bit operands)                        */
  int selinv_mode;  /* enum rgf_selinv_mode (default RGF_SELINV_EXACT)        */
  int device;       /* CUDA device ordinal, -1 = the current device           */
  int use_graphs;   /* 1 = replay each stage as a captured CUDA graph         */
  int fp64_diag;    /* split precision, Cholesky and inverse of the diagonal
                       blocks: 1 (default) FP64 accuracy, their inner products
                       emulated with 7 slices (56-bit operands); 2 native FP64
                       units; 0 the bulk slice count                          */
  int async_upload; /* 1: rgf_create queues the CSC upload and returns; the
                       copies overlap the first factorization, which waits for
                       each block column just before using it.  Applies to
                       page-locked arrays (cudaHostAlloc / cudaHostRegister);
                       pageable ones are copied before rgf_create returns, as
                       with 0 (the host stages such copies anyway).  The caller's
                       ia/ja/a must then stay valid and unchanged until the
                       first call that factorizes (rgf_factorize / rgf_logdet /
                       rgf_diag / rgf_solve) or rgf_residual_norm returns, or
                       until rgf_destroy -- the reference's own contract
                       (RGF.H:87-89 keeps the pointers), and pattern errors
                       are reported by that call.  0 (default): copied and
                       validated before rgf_create returns                    */
  int reserved[9];
} rgf_opts;

typedef struct rgf_handle rgf_handle;

/* Sizes of one instance (RGF.H:94-95). */
typedef struct rgf_info_t {
  size_t n;          /* ns*nt + nd                                           */
  size_t nnz;        /* stored lower non-zeros (ia[n])                       */
  size_t mf_size;    /* doubles in the block-column factor layout MF         */
  size_t device_bytes; /* device memory held by the handle                   */
  int not_spd_column;  /* first column with a non-positive pivot, or -1      */
  int reserved0;
  long long kernels_launched; /* GPU kernels launched by this handle so far   */
  int reserved[4];
} rgf_info_t;

/* Human-readable name of a status code. */
const char* rgf_status_string(int status);

/* Fill *opts with defaults. */
int rgf_default_opts(rgf_opts* opts);

/* Replaces RGF<double>::RGF (RGF.H:84-146).  Validates the CSC against the
 * block-tridiagonal-arrowhead pattern and copies it to the device, so the
 * caller's arrays may be freed after the call (with opts->async_upload = 0,
 * the default; see async_upload for the overlapped form).  opts may be NULL. */
int rgf_create(const size_t* ia, const size_t* ja, const double* a,
               size_t ns, size_t nt, size_t nd,
               const rgf_opts* opts, rgf_handle** out);

/* RGF<complex<double>> (RGF.H:756-774) for a Hermitian positive-definite
 * A = X + iY: ia/ja as for rgf_create, a holds nnz complex values as
 * interleaved (re, im) doubles.  The instance is held as the real symmetric
 * embedding [[X, -Y], [Y, X]] ordered per block, itself a BTA matrix with
 * (2ns, nt, 2nd), so every kernel and option of the real path applies.  On
 * such a handle rgf_logdet returns log det A (= log det of the embedding / 2),
 * and rgf_solve (x, b: n x nrhs complex), rgf_diag (diag: n complex, zero
 * imaginary parts) and rgf_residual_norm[_normalized] take complex
 * interleaved arrays; rgf_get_info, the exports and the device pointers
 * describe the real embedding.  (The reference's RGF<CPX> pairs a Hermitian
 * POTRF with plain transposes, which is consistent only for real data; this
 * is the Hermitian factorization.) */
int rgf_create_hermitian(const size_t* ia, const size_t* ja, const double* a,
                         size_t ns, size_t nt, size_t nd,
                         const rgf_opts* opts, rgf_handle** out);

/* The embedding itself, on the host: the lower CSC (2n + 1 column pointers,
 * *nnz2 entries) of the real matrix rgf_create_hermitian factors.  With ia2,
 * ja2 and a2 NULL only *nnz2 is set (then call again with arrays of that size). */
int rgf_hermitian_embed(const size_t* ia, const size_t* ja, const double* a,
                        size_t ns, size_t nt, size_t nd,
                        size_t* ia2, size_t* ja2, double* a2, size_t* nnz2);

/* Replaces RGF<double>::~RGF (RGF.H:150-170). */
int rgf_destroy(rgf_handle* h);

/* Replaces RGF<double>::factorize (RGF.H:510-546, FirstStageFactor
 * RGF.H:233-340).  The factor stays resident on the device. */
int rgf_factorize(rgf_handle* h);

/* Replaces RGF<double>::logDet (RGF.H:616-627): 2*sum(log L_kk).
 * Factorizes first if needed. */
int rgf_logdet(rgf_handle* h, double* logdet);

/* Replaces RGF<double>::solve(x, b, nrhs) (RGF.H:559-578,
 * SecondStageSolve RGF.H:344-418).  b and x are n x nrhs column-major
 * (ld = n) host arrays; x may equal b (RGF.H:550-554).  Factorizes first if
 * needed. */
int rgf_solve(rgf_handle* h, double* x, const double* b, size_t nrhs);

/* Replaces RGF<double>::RGFdiag (RGF.H:582-612, ThirdStageRGF
 * RGF.H:422-506): diag(A^{-1}) into the host array diag[n].  Unlike the
 * reference, the factor is not invalidated. */
int rgf_diag(rgf_handle* h, double* diag);

/* Replaces RGF<double>::residualNorm (RGF.H:631-655): ||b - A x||_2 of the
 * first right-hand side, computed on the device from the stored CSC. */
int rgf_residual_norm(rgf_handle* h, const double* x, const double* b, double* norm);

/* Replaces RGF<double>::residualNormNormalized (RGF.H:659-663). */
int rgf_residual_norm_normalized(rgf_handle* h, const double* x, const double* b,
                                 double* norm);

/* Copy the factor, in the reference's block-column layout MF (RGF.H:95,
 * 114-138), to the host array mf[mf_size].  Only the lower triangles of the
 * diagonal blocks are defined; the strict upper triangles are zero. */
int rgf_export_factor(rgf_handle* h, double* mf);

/* Copy the selected inverse to the host in the MF layout: Sigma_ii (full
 * block), Sigma_{i+1,i}, Sigma_{d,i} and Sigma_dd in the positions of
 * L_ii, L_{i+1,i}, C_i and L_dd.  Runs the selected inversion if needed.
 * Only RGF_SELINV_EXACT defines the off-diagonal blocks. */
int rgf_export_selinv(rgf_handle* h, double* ms);

/* Sizes and last-failure details. */
int rgf_get_info(rgf_handle* h, rgf_info_t* info);

/* Device-resident results (for callers that keep data on the GPU):
 * the selected-inverse diagonal, n doubles owned by the handle. */
int rgf_diag_device(rgf_handle* h, const double** d_diag);

/* The CUDA stream (cudaStream_t) all work of this handle is issued on. */
int rgf_get_stream(rgf_handle* h, void** stream);

/* Kernel timer: while enabled, every launch of the bulk GEMM kernels of this
 * handle is bracketed by CUDA events on the handle's stream.  For kind
 * 0 (all bulk GEMMs), 1 (FP64 DMMA GEMM) or 2 (split tensor-core GEMM, including
 * its slicing kernels) *ms receives the summed device time, *launches their
 * number and *flops their algorithmic FP64-equivalent flops since the last
 * reset; kind 3 reports the split GEMMs with *flops = executed bf16
 * slice-product flops.  While it is enabled stages run without CUDA graphs
 * and every timed product runs alone (the handle's streams are drained before
 * it), so the times are those of the kernels themselves.
 * enable = 2 also prints per-shape totals to stderr at each reset. */
int rgf_kernel_timer_enable(rgf_handle* h, int enable);
int rgf_kernel_timer_read(rgf_handle* h, int reset, int kind, double* ms, long long* launches,
                          double* flops);

/* C := alpha op(A) op(B) + beta C on device memory (column-major, BLAS
 * argument conventions, transa/transb 'N' or 'T'), queued on `stream` and
 * completed before return.  precision RGF_PREC_FP64 runs the FP64 DMMA
 * kernel; RGF_PREC_SPLIT runs the split-precision tensor-core kernel with
 * `slices` bf16 digits per operand (0 = default) when k is large enough, else
 * FP64.  These are the kernels of the solver's bulk updates. */
int rgf_dgemm_device(int precision, int slices, char transa, char transb, int m, int n, int k,
                     double alpha, const double* A, int lda, const double* B, int ldb,
                     double beta, double* C, int ldc, void* stream);

/* Failure handling.  Every device-side wait is bounded; a wait that runs out
 * makes the stage return RGF_ETIMEOUT and leaves the handle usable (the next
 * call recomputes).  rgf_set_wait_limit sets how many times the leaf
 * Cholesky's wait for the previous column's pivot polls before it gives up
 * (0 = the default, 2^26 polls); a small limit makes that wait run out, which
 * is how the timeout path is tested.  Changing it drops the handle's captured
 * stage graphs and its results. */
int rgf_set_wait_limit(rgf_handle* h, int polls);

/* Process-wide cache of device memory, off by default (max_bytes = 0).  With
 * max_bytes > 0, the buffers of a destroyed handle (and of the library's other
 * non-arena allocations) are kept, up to max_bytes in all, and handed to later
 * allocations of exactly their size on their device: a process that creates
 * and destroys handles of one shape in a loop (one per hyperparameter
 * evaluation, say) then pays no cudaMalloc/cudaFree per handle.  The memory
 * stays reserved for this library until a smaller limit (0 returns all of it)
 * or until an allocation the driver cannot serve, which first returns the
 * device's cached blocks.  rgf_device_cache_bytes reports the bytes held. */
int rgf_set_device_cache(size_t max_bytes);
int rgf_device_cache_bytes(size_t* held);

/* Failure injection for tests, process-wide: the next `after` device
 * allocations of the library succeed, the one after that fails as if the
 * device were out of memory (the call returns RGF_ENOMEM), and later ones
 * succeed again.  after < 0 switches it off. */
int rgf_debug_fail_alloc_after(long long after);

/* Measured FP64 (DMMA m8n8k4) throughput of the current device in TFLOP/s:
 * the denominator of the FP64 roofline.  Runs about 100 ms of GPU work. */
int rgf_measure_fp64_peak(double* tflops);

/* Largest n accepted by rgf_residual_norm_noalloc (8 MiB of doubles). */
#define RGF_NOALLOC_MAX_N ((size_t)1 << 20)

/* Allocation-free residual: d_out[0] = ||b - A x||_2, d_out[1] = ||b||_2 for
 * the symmetric matrix given by its lower CSC (n+1 column pointers d_ia, row
 * indices d_ja, values d_a), first right-hand side only.  Every pointer is
 * DEVICE memory on the current device and the work is queued on `stream`
 * (a cudaStream_t, NULL = legacy default stream); read d_out after that
 * stream has finished.
 * This entry point has no counterpart in the reference.  It exists for
 * callers that cannot call cudaMalloc: frameworks whose allocator already
 * holds nearly all device memory, serving loops that keep cudaMalloc and
 * cudaFree (which waits for the whole device) out of their steady state, and
 * embeddings that forbid hidden allocations.  It allocates nothing: its
 * scratch (n doubles) is a fixed 8 MiB device array that every GPU loading
 * this library holds until the process exits, so n must not exceed
 * RGF_NOALLOC_MAX_N (RGF_EINVAL otherwise).
 * The array belongs to this library's device code, which CUDA loads on a
 * device at the first call there (lazy module loading): that first call
 * reserves the 8 MiB and should be made during set-up, before the caller's
 * allocator takes the rest of the memory and before any stream capture.
 * Later calls reserve nothing.  Each call looks up the array's device
 * address in the current context.
 * The CSC must be a valid lower CSC (d_ia non-decreasing from 0, every row
 * index in [c, n) for column c), for example one that rgf_create accepted.
 * Row indices outside that range are skipped, never written through, and
 * make both outputs NaN; d_ia itself is not checked.
 * An error already pending on the calling thread is reported as RGF_ECUDA
 * and left pending.  All calls share the array: calls whose work overlaps on
 * the GPU race and give wrong results, so serialize them (one stream, or
 * events). */
int rgf_residual_norm_noalloc(size_t n, const size_t* d_ia, const size_t* d_ja,
                              const double* d_a, const double* d_x, const double* d_b,
                              double* d_out, void* stream);

/* ---- batches of independent instances --------------------------------------
 * Many factorizations of uneven (ns, nt, nd), as in a hyper-parameter search.
 * The reference handles one instance per RGF object (RGF.H:84); a batch holds
 * `count` instances, each created as by rgf_create from its own CSC. */
typedef struct rgf_batch rgf_batch;

int rgf_batch_create(size_t count, const size_t* const* ia, const size_t* const* ja,
                     const double* const* a, const size_t* ns, const size_t* nt,
                     const size_t* nd, const rgf_opts* opts, rgf_batch** out);
int rgf_batch_destroy(rgf_batch* b);
int rgf_batch_size(rgf_batch* b, size_t* count);
/* Instance i as an ordinary handle (solve, export, ... ); owned by the batch. */
int rgf_batch_handle(rgf_batch* b, size_t i, rgf_handle** h);
int rgf_batch_get_stream(rgf_batch* b, void** stream);
/* factorize + logDet + RGFdiag of every instance.  mode 0: all instances at
 * once, one concurrent branch (stream pair) per instance; the first run
 * launches the kernels directly, the second captures them into one CUDA graph
 * that later runs replay with a single launch.  mode 1: instance after
 * instance, each with its own stage launches (the per-instance baseline).  logdet[count] and
 * diag[i] (n_i doubles; diag or diag[i] may be NULL) receive the results. */
int rgf_batch_run(rgf_batch* b, int mode, double* logdet, double* const* diag);
/* GPU kernels launched by the batch's runs so far. */
int rgf_batch_kernels(rgf_batch* b, long long* kernels);

/* ---- tuning -----------------------------------------------------------------
 * Knobs of one handle's factorize + selected inversion (no counterpart in the
 * reference, whose MAGMA calls pick their own blocking).  None changes the
 * algorithm or the operation count; each changes how it is cut into kernels:
 *   leaf_nb     column width of the FP64 leaf Cholesky / triangular solves
 *               the recursive panel factorization bottoms out in: 16, 32, 64;
 *   lookahead   1 = the rows below each diagonal block are solved and updated
 *               on a second, lower-priority stream; 0 = one stream;
 *   split_bias  split precision: a product runs on the tensor cores when its
 *               estimated split time times split_bias is below its estimated
 *               FP64 time (1.0 = the fitted cost model; > 1 moves products to
 *               the FP64 kernels).  In [1/16, 16].
 * Results under different knobs agree to rounding; under the same knobs they
 * are bitwise identical, alone, batched or served. */
typedef struct rgf_tuning {
  int leaf_nb;
  int lookahead;
  double split_bias;
  double ms;        /* out: factorize + RGFdiag time measured by the autotuner
                       for this choice (0 when not measured)                 */
  int splitk_max;   /* tile shapes: largest split-K degree of the tensor-core
                       products (0 = default 16, 1 = no split K; 2, 4, 8)    */
  int fp64_tile;    /* output tile of the FP64 products: 0 = chosen per
                       product (32 or 64), 32 or 64 = always that           */
  int reserved[2];
} rgf_tuning;

enum rgf_tune_flags {
  RGF_TUNE_FORCE = 1  /* measure again even when the process-wide cache holds
                         a choice for this class                            */
};

int rgf_get_tuning(rgf_handle* h, rgf_tuning* t);
/* Set the knobs (t->ms is ignored).  Stage graphs captured with the old knobs
 * are dropped, the factor and selected inverse are recomputed on next use,
 * and a batch holding the handle recaptures its graph on its next run. */
int rgf_set_tuning(rgf_handle* h, const rgf_tuning* t);
/* Autotuner: times factorize + selected inversion (graph-replayed, best of two
 * after a direct run and a capture) for candidate knobs by coordinate
 * descent (leaf width, then look-ahead, then, in split precision, the routing
 * bias), keeps a candidate only when it is at least 2% faster, and sets the
 * best on h.  Choices are cached per process by (device, ns, nd, options);
 * a cached class is not measured again unless flags has RGF_TUNE_FORCE.
 * Allocates the selected-inversion buffers; leaves h unfactored.  The matrix
 * must be positive definite (the status of a failed run is returned, with
 * the knobs left as they were).  RGF_EINVAL while the kernel timer is on
 * (timed stages run launch by launch).  chosen may be NULL. */
int rgf_autotune(rgf_handle* h, int flags, rgf_tuning* chosen);
/* Autotune a batch: instances are grouped by (ns, nd); each group's knobs
 * are tuned (or taken from the cache) on its instance of median nt and set on
 * every member.  *classes (may be NULL) receives the number of groups. */
int rgf_batch_autotune(rgf_batch* b, int flags, size_t* classes);

/* ---- request loop (serving) -------------------------------------------------
 * Continuous batching on one GPU: `slots` workers take requests as soon as
 * they are free and, for a new factorization, as soon as its HBM footprint
 * fits `hbm_budget_bytes` (least-recently-used idle factors are evicted to make
 * room); admitted requests run concurrently on their own streams.  Factors
 * stay resident for follow-up solve / RGFdiag requests until released or
 * evicted; a factor that a submitted, not yet run request names is never
 * evicted, so such a request fails only if the factor id was unknown at
 * submission or released in between.  Built on the lazy-factorize, resident-factor semantics of the
 * class (RGF.H:561, 585, 619); the reference has no request loop. */
enum rgf_request_kind {
  RGF_REQ_FACTOR = 0,   /* create + factorize + logDet; returns factor_id    */
  RGF_REQ_SOLVE = 1,    /* x = A^{-1} b with a resident factor              */
  RGF_REQ_DIAG = 2,     /* diag(A^{-1}) with a resident factor              */
  RGF_REQ_RELEASE = 3   /* drop a resident factor                           */
};

/* Caller-owned; every pointer it holds must stay valid until the request is
 * done.  The server writes factor_id (FACTOR), logdet, status and latency. */
typedef struct rgf_request {
  int kind;
  int status;            /* out: rgf_status, -1 while pending                */
  long long factor_id;   /* in: SOLVE/DIAG/RELEASE; out: FACTOR               */
  const size_t* ia;      /* FACTOR: lower CSC and sizes                        */
  const size_t* ja;
  const double* a;
  size_t ns, nt, nd;
  const double* b;       /* SOLVE: n x nrhs column-major                       */
  double* x;
  size_t nrhs;
  double* diag;          /* DIAG: n doubles                                    */
  double logdet;         /* out: FACTOR                                        */
  double latency_ms;     /* out: submit to completion                          */
  size_t reserved_bytes; /* internal                                           */
} rgf_request;

typedef struct rgf_server_stats_t {
  long long submitted, admitted, completed, failed, evicted;
  long long resident_factors, queued;
  size_t used_bytes;        /* HBM reserved for admitted requests (estimates) */
  size_t arena_bytes;       /* device memory pre-reserved at creation          */
  size_t arena_in_use;      /* of which held by resident factors and requests  */
  long long arena_fallbacks;/* allocations the arena could not serve (cudaMalloc) */
} rgf_server_stats_t;

typedef struct rgf_server rgf_server;
/* The whole HBM budget is reserved at creation as one device arena: every
 * handle a request creates takes its memory from it and eviction returns it
 * there, so the steady state calls neither cudaMalloc nor cudaFree (whose
 * device-wide wait would stall every request in flight).  RGF_ENOMEM if the
 * budget cannot be reserved. */
int rgf_server_create(const rgf_opts* opts, size_t hbm_budget_bytes, int slots,
                      rgf_server** out);
int rgf_server_submit(rgf_server* s, rgf_request* req, long long* ticket);
/* Wait up to timeout_s for a ticket; *status receives the request's status.
 * Returns RGF_ETIMEOUT if it is still running. */
int rgf_server_wait(rgf_server* s, long long ticket, double timeout_s, int* status);
int rgf_server_stats(rgf_server* s, rgf_server_stats_t* stats);
/* Stops the workers (requests still queued are not run) and frees factors. */
int rgf_server_destroy(rgf_server* s);

#ifdef __cplusplus
}
#endif

#endif /* RGF_GB300_RGF_H */
