// Host engine and C ABI of librgf_gb300.
//
// A handle owns, in device memory: the CSC (uploaded once), the factor in the
// reference's block-column layout MF, the selected inverse in the same
// layout, and workspaces.  Each stage (factorize, selected inversion, solve
// with a given nrhs) is issued once on the handle's stream under CUDA graph
// capture and replayed afterwards, so the launch sequence costs one graph
// launch per call.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/rgf.h"
#include "rgf_internal.h"
#include "rgf_split.h"

using namespace rgf;

namespace {
constexpr int NB = 64;  // leaf tile of the FP64 panel Cholesky / triangular solves
// FP64 refinement of split-precision solves: at most this many correction
// steps; refinement stops as soon as every right-hand side's normalized
// residual ||b - A x|| / ||b|| is at or below RGF_REFINE_TOL (one step
// suffices when the factor is accurate to ~1e-10: the error contracts by
// about that factor per step)
constexpr int RGF_REFINE_STEPS = 3;
constexpr double RGF_REFINE_TOL = 1e-14;
}

struct rgf_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  // Second stream of the panel factorization: the rows below a diagonal block
  // (off the column-to-column critical path) are solved and updated there.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool on_side = false;  // launch wrappers issue to `side`
  bool lookahead = true;
  // complex Hermitian instance held as its real embedding (2ns, nt, 2nd):
  // x, b and diag of the C ABI are then complex (interleaved re, im) of size nc
  bool hermitian = false;
  size_t hns = 0, hnt = 0, hnd = 0, nc = 0;
  BtaShape sh{};
  long long nnz = 0, mf_size = 0;
  rgf_opts opts{};

  size_t* d_ia = nullptr;
  size_t* d_ja = nullptr;
  double* d_a = nullptr;
  double* d_MF = nullptr;
  double* d_MS = nullptr;
  double* d_U = nullptr;     // Linv^T of every diagonal block (ns x ns each), then the corner
  double* d_T1 = nullptr;    // (ns + nd) x ns
  double* d_T2 = nullptr;    // ns x ns
  double* d_T3 = nullptr;    // nd x ns
  double* d_logpart = nullptr;
  int nparts = 0;
  double* d_scalars = nullptr;  // [0] logdet, [1] ||r||, [2] ||b||
  double* d_diag = nullptr;
  DevStatus* d_status = nullptr;
  double* d_rhs = nullptr;
  double* d_rhs2 = nullptr;  // y of the block substitution (rhs_cap doubles)
  size_t rhs_cap = 0;           // doubles
  double* d_partial = nullptr;  // arrowhead partial sums, nt * nrhs * nd
  size_t partial_cap = 0;
  double* d_res = nullptr;      // residual scratch: x, b, y (3n)
  double* d_ref = nullptr;      // refinement of split solves: x, b, y (3 n nrhs)
  double* d_norms = nullptr;    // refinement: ||r_q||, ||b_q|| per right-hand side (2 x 4096)
  size_t ref_cap = 0;           // doubles
  double* d_gemm_ws = nullptr;  // split-K partial sums of small FP64 GEMMs
  double* d_gemm_ws_side = nullptr;  // the same for the side stream
  long long gemm_ws_elems = 0;

  bool factored = false;
  bool selinv_done = false;
  bool inv_done = false;  // U holds the inverses of the current factor's blocks
  int not_spd_col = -1;
  size_t device_bytes = 0;

  cudaGraphExec_t g_factor = nullptr, g_selinv = nullptr, g_inv = nullptr;
  long long k_factor = 0, k_selinv = 0, k_inv = 0;
  std::map<size_t, std::pair<cudaGraphExec_t, long long>> g_solve;
  int runs_factor = 0, runs_selinv = 0, runs_inv = 0;  // stage runs so far (the first is not captured)
  bool mf_holds_a = false;  // MF holds the ingested A (create's validation), not yet factored
  // Asynchronous upload (rgf_opts.async_upload): create queues the CSC copies
  // and the ingest of every block column on `upload` and returns; ev_chunk[i]
  // marks block column i of MF holding A (i = nt: the arrowhead corner).  The
  // first factorization waits for each block column just before using it.
  cudaStream_t upload = nullptr;
  std::vector<cudaEvent_t> ev_chunk;
  bool upload_pending = false;
  std::map<size_t, int> runs_solve;
  long long kernels_issued = 0;   // kernels of the stage being recorded
  long long kernels_total = 0;    // kernels launched over the handle's life

  SplitEngine* split = nullptr;
  SplitEngine* split_side = nullptr;  // own slice workspace for the side stream
  // tuning knobs (rgf_set_tuning / rgf_autotune); knob_gen counts changes so
  // that a batch graph captured with older knobs is captured again
  int leaf_wait_polls = 0;   // poll limit of the leaf's pivot waits (0 = default)
  int nb = 32;               // leaf width of the panel Cholesky (16, 32 or 64)
  double split_bias = 1.0;   // the estimated split-product time is scaled by it
  int splitk_max = 0;        // tile shapes: split-K cap of the tensor-core products (0 = 16)
  int fp64_tile = 0;         // and the FP64 output tile (0 = per product; split: 32)
  double tuned_ms = 0.0;     // factorize + RGFdiag time measured by the autotuner
  long long knob_gen = 0;

  // kernel timer: per class (1 = FP64 DMMA GEMM, 2 = split tensor-core GEMM)
  struct TimedLaunch {
    cudaEvent_t e0, e1;
    int kind;
    double flops;         // algorithmic FP64-equivalent flops
    double tensor_flops;  // executed bf16 slice-product flops (split only)
    int m, n, k, batch, cls;
  };
  std::map<std::string, std::pair<long long, double>> timer_detail;  // shape -> (launches, ms)
  bool timer_on = false;
  bool timer_detail_on = false;  // per-shape totals printed to stderr on timer reset
  std::vector<TimedLaunch> ev_used;
  // launch trace (RGF_GB300_TRACE=<csv path>): stages run launch by launch and
  // an event follows every launch on its stream
  struct TraceRec {
    std::string label;
    int side;
    cudaEvent_t ev;
  };
  std::string trace_path;
  std::vector<TraceRec> trace;
  cudaEvent_t trace_t0 = nullptr;
  int trace_stage = 0;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
  double timer_ms[3] = {0, 0, 0}, timer_flops[3] = {0, 0, 0}, timer_tflops = 0.0;
  long long timer_launches[3] = {0, 0, 0};
};

namespace rgf {
// allocations left before the injected failure; < 0: injection off
static std::atomic<long long> g_fail_alloc_after{-1};

struct DeviceArena {
  char* base = nullptr;
  size_t size = 0;
  std::mutex mu;
  std::map<size_t, size_t> free_blocks;  // offset -> bytes
  std::map<size_t, size_t> used_blocks;  // offset -> bytes
  size_t in_use = 0;
  long long fallbacks = 0;
};

static std::mutex g_arenas_mu;
static std::vector<DeviceArena*> g_arenas;
static thread_local DeviceArena* t_arena = nullptr;

DeviceArena* arena_create(size_t bytes, int* status) {
  *status = RGF_OK;
  DeviceArena* a = new (std::nothrow) DeviceArena();
  if (!a) {
    *status = RGF_ENOMEM;
    return nullptr;
  }
  bytes = (bytes + 255) & ~size_t(255);
  if (cudaMalloc((void**)&a->base, bytes) != cudaSuccess) {
    cudaGetLastError();
    delete a;
    *status = RGF_ENOMEM;
    return nullptr;
  }
  a->size = bytes;
  a->free_blocks[0] = bytes;
  std::lock_guard<std::mutex> lk(g_arenas_mu);
  g_arenas.push_back(a);
  return a;
}

void arena_destroy(DeviceArena* a) {
  if (!a) return;
  {
    std::lock_guard<std::mutex> lk(g_arenas_mu);
    g_arenas.erase(std::remove(g_arenas.begin(), g_arenas.end(), a), g_arenas.end());
  }
  cudaFree(a->base);
  delete a;
}

void set_thread_arena(DeviceArena* a) { t_arena = a; }
long long arena_fallbacks(DeviceArena* a) {
  if (!a) return 0;
  std::lock_guard<std::mutex> lk(a->mu);
  return a->fallbacks;
}
size_t arena_in_use(DeviceArena* a) {
  if (!a) return 0;
  std::lock_guard<std::mutex> lk(a->mu);
  return a->in_use;
}

static void* arena_alloc(DeviceArena* a, size_t bytes) {
  bytes = (std::max<size_t>(bytes, 1) + 255) & ~size_t(255);
  std::lock_guard<std::mutex> lk(a->mu);
  for (auto it = a->free_blocks.begin(); it != a->free_blocks.end(); ++it) {
    if (it->second < bytes) continue;
    const size_t off = it->first, rest = it->second - bytes;
    a->free_blocks.erase(it);
    if (rest) a->free_blocks[off + bytes] = rest;
    a->used_blocks[off] = bytes;
    a->in_use += bytes;
    return a->base + off;
  }
  a->fallbacks++;
  return nullptr;
}

// true when p belonged to an arena (and is now free there)
static bool arena_release(void* p) {
  std::lock_guard<std::mutex> lk(g_arenas_mu);
  for (DeviceArena* a : g_arenas) {
    char* c = static_cast<char*>(p);
    if (c < a->base || c >= a->base + a->size) continue;
    std::lock_guard<std::mutex> la(a->mu);
    size_t off = (size_t)(c - a->base);
    auto u = a->used_blocks.find(off);
    if (u == a->used_blocks.end()) return true;  // not a live block: ignore
    size_t len = u->second;
    a->used_blocks.erase(u);
    a->in_use -= len;
    auto next = a->free_blocks.lower_bound(off);
    if (next != a->free_blocks.end() && next->first == off + len) {  // merge right
      len += next->second;
      next = a->free_blocks.erase(next);
    }
    if (next != a->free_blocks.begin()) {  // merge left
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        prev->second += len;
        return true;
      }
    }
    a->free_blocks[off] = len;
    return true;
  }
  return false;
}

bool pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("RGF_GB300_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

// Process-wide cache of freed device blocks (rgf_set_device_cache; off by
// default).  A block freed outside an arena is kept, while the cache holds at
// most `limit` bytes, for a later allocation of exactly its size on its
// device -- a handle of the same shape gets its buffers back without a
// cudaMalloc, and destroying one costs no cudaFree (whose unmapping of tens of
// GB takes ~20 ms).  Blocks are freed only after the streams that used them
// are synchronized (release(), the workspace resizes), so a cached block is
// idle when it is handed out again.  An allocation that cudaMalloc cannot
// serve returns the device's cached blocks to the driver and tries again.
struct DeviceCache {
  std::mutex mu;
  size_t limit = 0, held = 0;
  std::multimap<std::pair<int, size_t>, void*> free_blocks;  // (device, bytes) -> block
  std::map<void*, std::pair<int, size_t>> sizes;             // live cudaMalloc blocks
};
static DeviceCache g_cache;

static void cache_trim(size_t keep, int device) {  // g_cache.mu held
  int cur = -1;
  cudaGetDevice(&cur);
  for (auto it = g_cache.free_blocks.begin();
       it != g_cache.free_blocks.end() && g_cache.held > keep;) {
    if (device >= 0 && it->first.first != device) {
      ++it;
      continue;
    }
    g_cache.held -= it->first.second;
    cudaSetDevice(it->first.first);  // the block's own device
    cudaFree(it->second);
    it = g_cache.free_blocks.erase(it);
  }
  if (cur >= 0) cudaSetDevice(cur);
}

cudaError_t device_malloc(void** p, size_t bytes) {
  long long left = g_fail_alloc_after.load();
  while (left >= 0) {
    if (g_fail_alloc_after.compare_exchange_weak(left, left - 1)) {
      if (left == 0) {  // this allocation fails, later ones succeed again
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  if (t_arena) {
    *p = arena_alloc(t_arena, bytes);
    if (*p) return cudaSuccess;
  }
  std::lock_guard<std::mutex> lk(g_cache.mu);
  if (g_cache.limit == 0 && g_cache.held == 0) return cudaMalloc(p, bytes);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cudaErrorInvalidDevice;
  auto it = g_cache.free_blocks.find({dev, bytes});
  if (it != g_cache.free_blocks.end()) {
    *p = it->second;
    g_cache.held -= bytes;
    g_cache.free_blocks.erase(it);
  } else {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaErrorMemoryAllocation && g_cache.held > 0) {
      cudaGetLastError();
      cache_trim(0, dev);
      e = cudaMalloc(p, bytes);
    }
    if (e != cudaSuccess) return e;
  }
  g_cache.sizes[*p] = {dev, bytes};
  return cudaSuccess;
}

void device_free(void* p) {
  if (!p || arena_release(p)) return;
  {
    std::lock_guard<std::mutex> lk(g_cache.mu);
    auto it = g_cache.sizes.find(p);
    if (it != g_cache.sizes.end()) {
      const std::pair<int, size_t> key = it->second;
      g_cache.sizes.erase(it);
      if (g_cache.held + key.second <= g_cache.limit) {
        g_cache.free_blocks.emplace(key, p);
        g_cache.held += key.second;
        return;
      }
    }
  }
  cudaFree(p);
}
}  // namespace rgf

namespace {

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return RGF_OK;
  if (e == cudaErrorMemoryAllocation) return RGF_ENOMEM;
  return RGF_ECUDA;
}

#define RGF_CK(call)                       \
  do {                                     \
    cudaError_t e_ = (call);               \
    if (e_ != cudaSuccess) {               \
      return cuda_status(e_);              \
    }                                      \
  } while (0)

__global__ void status_init_kernel(DevStatus* st) {
  st->not_spd_col = INT_MAX;
  st->bad_input = 0;
  st->timeout = 0;
}

template <class T>
int dalloc(rgf_handle* h, T** p, size_t count) {
  if (count == 0) count = 1;
  cudaError_t e = device_malloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RGF_ENOMEM : RGF_ECUDA;
  }
  h->device_bytes += count * sizeof(T);
  return RGF_OK;
}

void dfree(void* p) { device_free(p); }

// ---- launch wrappers (count kernels; optional event timer on bulk GEMMs) ----
// GEMM classes: SMALL always runs in FP64; BULK may run as split products;
// DIAG (updates inside a diagonal block's Cholesky or inverse) runs split
// only when the handle does not keep diagonal blocks in FP64.
enum GemmClass { SMALL = 0, BULK = 1, DIAG = 2 };

cudaStream_t cur_stream(const rgf_handle* h) { return h->on_side ? h->side : h->stream; }

// Work issued to the side stream after fork_side waits for everything issued
// to the main stream before it; join_side makes the main stream wait for the
// side stream.  Both are plain event dependencies (graph edges when captured).
void fork_side(rgf_handle* h) {
  cudaEventRecord(h->ev_fork, h->stream);
  cudaStreamWaitEvent(h->side, h->ev_fork, 0);
}
void join_side(rgf_handle* h) {
  cudaEventRecord(h->ev_join, h->side);
  cudaStreamWaitEvent(h->stream, h->ev_join, 0);
}

// Launch trace: an event on the current stream after the launch just issued.
void trace(rgf_handle* h, const char* label) {
  if (h->trace_path.empty()) return;
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, cur_stream(h));
  h->trace.push_back({label, h->on_side ? 1 : 0, e});
}

// Append the stage's trace to the CSV file: stage, launch, stream (0 main,
// 1 side), label, ms from the stage start to the end of the launch.
void trace_flush(rgf_handle* h) {
  if (h->trace.empty()) return;
  FILE* f = std::fopen(h->trace_path.c_str(), "a");
  int i = 0;
  for (auto& t : h->trace) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->trace_t0, t.ev);
    if (f) std::fprintf(f, "%d,%d,%d,%s,%.4f\n", h->trace_stage, i++, t.side, t.label.c_str(), ms);
    cudaEventDestroy(t.ev);
  }
  if (f) std::fclose(f);
  h->trace.clear();
  h->trace_stage++;
}

void gemm(rgf_handle* h, const GemmDesc& g, int cls) {
  if (g.m <= 0 || g.n <= 0 || g.batch <= 0) return;
  const bool bulk = cls != SMALL;
  // fp64_diag: 0 = diagonal blocks at the bulk slice count, 1 = at 7 slices
  // (56-bit operands: FP64-accurate emulation), 2 = native FP64 DMMA
  const int fd = h->opts.fp64_diag;
  const bool may_split = cls == BULK || (cls == DIAG && fd != 2);
  const int slices = (cls == DIAG && fd == 1) ? 7 : 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (h->timer_on && bulk) {
    if (h->ev_pool.empty()) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
    } else {
      e0 = h->ev_pool.back().first;
      e1 = h->ev_pool.back().second;
      h->ev_pool.pop_back();
    }
    // each timed product runs alone: both streams drained before it starts,
    // so its events measure the kernels themselves, not queueing or overlap
    cudaStreamSynchronize(h->stream);
    cudaStreamSynchronize(h->side);
    cudaEventRecord(e0, cur_stream(h));
  }
  long long launched = 1;
  double tflops = 0.0;
  SplitEngine* eng = h->on_side ? h->split_side : h->split;
  bool split = eng && may_split && eng->supports(g);
  if (split) {
    // Route by estimated time: the split engine's estimate (its launches,
    // slicing, MMA streams and split K) against the FP64 DMMA kernel at
    // ~9 us of launches and ~0.9 TFLOP/s.  Small or thin products are faster
    // in FP64 (which is also FP64-accurate).
    const double t_split = eng->estimate_seconds(g, slices);
    const double t_fp64 = 9e-6 + gemm_flops(g) / 0.9e12;
    split = t_split * h->split_bias < t_fp64;
  }
  if (split) {
    launched = eng->gemm(g, cur_stream(h), h->d_status, &tflops, slices);
  } else {
    GemmDesc gw = g;
    gw.ws = h->on_side ? h->d_gemm_ws_side : h->d_gemm_ws;
    gw.ws_elems = h->gemm_ws_elems;
    gw.tile = h->fp64_tile;
    launched = launch_gemm_fp64(gw, cur_stream(h));
  }
  h->kernels_issued += launched;
  if (!h->trace_path.empty()) {
    char lab[96];
    std::snprintf(lab, sizeof(lab), "%s cls%d m%d n%d k%d b%d", split ? "split" : "fp64", cls, g.m,
                  g.n, g.k, g.batch);
    trace(h, lab);
  }
  if (e0) {
    cudaEventRecord(e1, cur_stream(h));
    h->ev_used.push_back({e0, e1, split ? 2 : 1, gemm_flops(g), tflops, g.m, g.n, g.k, g.batch, cls});
  }
}

void leaf_potrf(rgf_handle* h, double* T, long long ldt, int nbk, int col0) {
  launch_leaf_potrf(T, ldt, nbk, col0, h->d_status, cur_stream(h), h->leaf_wait_polls);
  h->kernels_issued++;
  trace(h, "leaf");
}

void trsm_rows(rgf_handle* h, double* X, long long xrs, long long xcs, int rows,
               const double* L, long long ldl, int nbk, int mode, int batch = 1,
               long long sX = 0, long long sL = 0) {
  if (rows <= 0) return;
  launch_trsm_rows(X, xrs, xcs, rows, L, ldl, nbk, mode, batch, sX, sL, cur_stream(h));
  h->kernels_issued++;
  if (!h->trace_path.empty()) {
    char lab[64];
    std::snprintf(lab, sizeof(lab), "trsm rows%d nb%d b%d", rows, nbk, batch);
    trace(h, lab);
  }
}

// ---- panel Cholesky: [D; B; C] (rows x cols, lda) -> [L; B L^-T; C L^-T] ----
// Recursive (left half first) Cholesky of the top cols x cols block with the
// TRSM of the rows below folded in (RGF.H:254-260, 284-287, 312-317, 335 as
// one pass).  Halving the column range makes every trailing update one GEMM
// with an inner dimension of half the range, so most of the work runs in a
// few large products; 64-column leaves are factored in FP64 in one CTA and
// solved against row-parallel.
//
// Rows [0, dr) belong to the diagonal block being factored (the column-to-
// column critical path); rows [dr, rows) are the block rows below it, which
// nothing on that path reads.  With look-ahead on, their solves and updates
// go to the side stream, ordered after the main-stream work they read, so the
// critical path only carries the diagonal block.
void panel_potrf(rgf_handle* h, double* P, long long lda, int rows, int cols, int dr, int col0) {
  const int nb = h->nb;
  const bool la = h->lookahead && h->side;
  const int split_row = la ? dr : rows;  // rows at or past this go to the side stream
  if (cols <= nb) {
    leaf_potrf(h, P, lda, cols, col0);
    if (split_row > cols) trsm_rows(h, P + cols, 1, lda, split_row - cols, P, lda, cols, 0);
    if (rows > split_row) {
      fork_side(h);
      h->on_side = true;
      trsm_rows(h, P + split_row, 1, lda, rows - split_row, P, lda, cols, 0);
      h->on_side = false;
    }
    return;
  }
  const int c1 = ((cols / 2 + nb - 1) / nb) * nb;
  panel_potrf(h, P, lda, rows, c1, dr, col0);
  // trailing update: P[c1:rows, c1:cols] -= P[c1:rows, 0:c1] P[c1:cols, 0:c1]^T
  auto upd = [&](int r0, int m, int cls) {
    if (m <= 0) return;
    GemmDesc g;
    g.m = m; g.n = cols - c1; g.k = c1;
    g.A = P + r0; g.lda = lda; g.transA = 0;
    g.B = P + c1; g.ldb = lda; g.transB = 1;
    g.C = g.D = P + r0 + (long long)c1 * lda;
    g.ldc = g.ldd = lda;
    g.alpha = -1.0; g.beta = 1.0;
    // lower-only when the block starts on the diagonal (rows below it are full)
    g.outLower = r0 < cols ? 1 : 0;
    gemm(h, g, cls);
  };
  if (rows > split_row) {
    fork_side(h);
    h->on_side = true;
    upd(split_row, rows - split_row, BULK);
    h->on_side = false;
  }
  if (h->split && h->opts.fp64_diag && cols - c1 > 256) {
    upd(c1, cols - c1, DIAG);              // inside the diagonal block: FP64 accuracy
    upd(cols, split_row - cols, BULK);
  } else if (h->split && h->opts.fp64_diag) {
    // a narrow node: one launch covers the diagonal block and the rows below
    // it on the critical path, at FP64 accuracy (7-slice split products or
    // FP64, whichever the cost model finds faster)
    upd(c1, split_row - c1, DIAG);
  } else {
    upd(c1, split_row - c1, BULK);
  }
  panel_potrf(h, P + c1 + (long long)c1 * lda, lda, rows - c1, cols - c1, dr - c1, col0 + c1);
}

// ---- stage 1: factorize (RGF.H:233-340) ----
void issue_factor(rgf_handle* h) {
  const BtaShape& sh = h->sh;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd;
  cudaStream_t s = h->stream;
  // first factorization after an asynchronous create: block column i is
  // waited for just before its first use (the corner, uploaded first, now);
  // the status was initialized before the uploads' ingests, which record
  // pattern errors in it
  const bool streamed = h->upload_pending;
  const long long corner_chunk = nd > 0 ? nt : -1;
  if (streamed) {
    if (corner_chunk >= 0) cudaStreamWaitEvent(s, h->ev_chunk[corner_chunk], 0);
  } else {
    status_init_kernel<<<1, 1, 0, s>>>(h->d_status);
    h->kernels_issued += 1;
  }
  // The first factorization after create launched directly finds A already
  // ingested into MF by create's validation; a captured stage ingests on
  // every replay.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusActive;
  if (!h->mf_holds_a || cap != cudaStreamCaptureStatusNone) {
    cudaMemsetAsync(h->d_MF, 0, sizeof(double) * h->mf_size, s);
    launch_ingest(sh, h->d_ia, h->d_ja, h->d_a, h->d_MF, h->d_status, s);
    h->kernels_issued += 1;
    trace(h, "ingest");
  }
  h->mf_holds_a = false;
  double* corner = h->d_MF + mf_col_offset(sh, nt);
  for (long long i = 0; i < nt; ++i) {
    double* P = h->d_MF + mf_col_offset(sh, i);
    const long long lda = mf_lda(sh, i);
    if (streamed) cudaStreamWaitEvent(s, h->ev_chunk[i], 0);
    if (i > 0) {
      const double* Pm = h->d_MF + mf_col_offset(sh, i - 1);
      const long long ldm = mf_lda(sh, i - 1);
      // [D_i; C_i] -= [L_{i,i-1}; C_{i-1}] L_{i,i-1}^T  (RGF.H:276, 279, 304, 307): the
      // rows [L_{i,i-1}; C_{i-1}] are adjacent in block column i-1, so both
      // updates run as one product (lower part only for D_i)
      GemmDesc g;
      g.m = (int)(ns + nd); g.n = g.k = (int)ns;
      g.A = Pm + ns; g.lda = ldm; g.B = Pm + ns; g.ldb = ldm; g.transB = 1;
      g.C = g.D = P; g.ldc = g.ldd = lda;
      if (nd > 0) {
        g.C2 = g.D2 = P + mf_dense_row(sh, i);
        g.mD1 = (int)ns;
      }
      g.alpha = -1.0; g.beta = 1.0; g.outLower = 1;
      gemm(h, g, BULK);
      if (nd > 0) {
        const double* Cm = Pm + mf_dense_row(sh, i - 1);
        GemmDesc c;  // corner -= C_{i-1} C_{i-1}^T  (RGF.H:280, 308)
        c.m = c.n = (int)nd; c.k = (int)ns;
        c.A = Cm; c.lda = ldm; c.B = Cm; c.ldb = ldm; c.transB = 1;
        c.C = c.D = corner; c.ldc = c.ldd = nd;
        c.alpha = -1.0; c.beta = 1.0; c.outLower = 1;
        // With look-ahead, on the side stream, where C_{i-1} was computed
        // (no fork needed): nothing else touches the corner until the last
        // block's join, so the update leaves the critical path.
        h->on_side = h->lookahead && h->side;
        gemm(h, c, SMALL);
        h->on_side = false;
      }
    }
    panel_potrf(h, P, lda, (int)lda, (int)ns, (int)ns, (int)(i * ns));
    if (h->lookahead && h->side && lda > ns) join_side(h);
    trace(h, "block end");
  }
  if (nd > 0) {
    const double* Pl = h->d_MF + mf_col_offset(sh, nt - 1);
    const double* Cl = Pl + mf_dense_row(sh, nt - 1);
    GemmDesc c;  // corner -= C_{nt-1} C_{nt-1}^T  (RGF.H:332)
    c.m = c.n = (int)nd; c.k = (int)ns;
    c.A = Cl; c.lda = mf_lda(sh, nt - 1); c.B = Cl; c.ldb = mf_lda(sh, nt - 1); c.transB = 1;
    c.C = c.D = corner; c.ldc = c.ldd = nd;
    c.alpha = -1.0; c.beta = 1.0; c.outLower = 1;
    gemm(h, c, SMALL);
    panel_potrf(h, corner, nd, (int)nd, (int)nd, (int)nd, (int)(nt * ns));  // RGF.H:335
  }
  launch_logdet(sh, h->d_MF, h->d_logpart, h->d_scalars, s);
  h->kernels_issued += 2;
}

// For every diagonal block at once: U_i = L_ii^{-T} (upper triangular).
// Right-looking RLTN solve U L^T = I by 64-column blocks; only rows above the
// current block are non-zero, so the work is ns^3/3 per block.  The
// nt-1 blocks of leading dimension 2ns+nd run as one batch, the last block
// (leading dimension ns+nd) and the corner separately.
// For `batch` diagonal blocks at once: U = L^{-T} (upper triangular).
// Recursive halving: with L = [L11 0; L21 L22], U = [U11 U12; 0 U22] where
// U11 = L11^{-T}, U22 = L22^{-T} and U12 = -U11 (L21^T U22).  The two halves
// are independent; each level adds two GEMMs with an inner dimension of half
// the range, batched over all blocks, so the inverse runs as a few large
// products (DIAG class: FP64 or FP64-accurate split).  Leaves (<= 64) solve
// X L^T = I row-parallel.  T (the product L21^T U22) lives in Tmp at the
// position of U12.
void issue_trtri(rgf_handle* h, double* U, long long ldu, long long n, const double* L,
                 long long ldl, double* Tmp, long long ldt, int batch, long long sU, long long sL,
                 long long sT) {
  if (batch <= 0 || n <= 0) return;
  if (n <= NB) {
    launch_set_identity(U, ldu, (int)n, batch, sU, h->stream);
    h->kernels_issued++;
    trsm_rows(h, U, 1, ldu, (int)n, L, ldl, (int)n, 0, batch, sU, sL);
    return;
  }
  const long long n1 = ((n / 2 + NB - 1) / NB) * NB, n2 = n - n1;
  issue_trtri(h, U, ldu, n1, L, ldl, Tmp, ldt, batch, sU, sL, sT);
  issue_trtri(h, U + n1 + n1 * ldu, ldu, n2, L + n1 + n1 * ldl, ldl, Tmp + n1 + n1 * ldt, ldt,
              batch, sU, sL, sT);
  double* T = Tmp + n1 * ldt;
  GemmDesc a;  // T = L21^T U22
  a.m = (int)n1; a.n = (int)n2; a.k = (int)n2;
  a.A = L + n1; a.lda = ldl; a.transA = 1;
  a.B = U + n1 + n1 * ldu; a.ldb = ldu; a.triB = TRI_UPPER;
  a.D = T; a.ldd = ldt; a.alpha = 1.0; a.beta = 0.0;
  a.batch = batch; a.sA = sL; a.sB = sU; a.sD = sT;
  gemm(h, a, DIAG);
  GemmDesc b;  // U12 = -U11 T
  b.m = (int)n1; b.n = (int)n2; b.k = (int)n1;
  b.A = U; b.lda = ldu; b.triA = TRI_UPPER;
  b.B = T; b.ldb = ldt;
  b.D = U + n1 * ldu; b.ldd = ldu; b.alpha = -1.0; b.beta = 0.0;
  b.batch = batch; b.sA = sU; b.sB = sT; b.sD = sU;
  gemm(h, b, DIAG);
}

GemmDesc mk(int m, int n, int k, const double* A, long long lda, int tA, const double* B,
            long long ldb, int tB, const double* C, long long ldc, double* D, long long ldd,
            double alpha, double beta) {
  GemmDesc g;
  g.m = m; g.n = n; g.k = k;
  g.A = A; g.lda = lda; g.transA = tA;
  g.B = B; g.ldb = ldb; g.transB = tB;
  g.C = C; g.ldc = ldc; g.D = D; g.ldd = ldd;
  g.alpha = alpha; g.beta = beta;
  return g;
}

// U_i = L_ii^{-T} of every diagonal block and of the corner, as one batched
// recursive TRTRI (the blocks are independent once the factor exists); MS is
// the recursion's scratch.
void issue_inverses(rgf_handle* h) {
  const BtaShape& sh = h->sh;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd;
  const long long ss = ns * ns;
  // The inverses are upper triangular and are read as full blocks
  // (W^T = U_i - ...); the recursion writes only their upper part, so the
  // strictly lower part must be zero.
  cudaMemsetAsync(h->d_U, 0, sizeof(double) * (nt * ss + nd * nd), h->stream);
  if (nt > 1)
    issue_trtri(h, h->d_U, ns, ns, h->d_MF, 2 * ns + nd, h->d_MS, 2 * ns + nd, (int)(nt - 1), ss,
                ns * (2 * ns + nd), ns * (2 * ns + nd));
  issue_trtri(h, h->d_U + (nt - 1) * ss, ns, ns, h->d_MF + mf_col_offset(sh, nt - 1), ns + nd,
              h->d_MS + mf_col_offset(sh, nt - 1), ns + nd, 1, 0, 0, 0);
  if (nd > 0)
    issue_trtri(h, h->d_U + nt * ss, nd, nd, h->d_MF + mf_col_offset(sh, nt), nd,
                h->d_MS + mf_col_offset(sh, nt), nd, 1, 0, 0, 0);
}

// ---- stage 3: selected inversion ----
void issue_selinv(rgf_handle* h) {
  const BtaShape& sh = h->sh;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd;
  const int ins = (int)ns, ind = (int)nd;
  cudaStream_t s = h->stream;
  const long long ss = ns * ns;
  double* Ud = h->d_U + nt * ss;
  double* Sdd = h->d_MS + mf_col_offset(sh, nt);
  issue_inverses(h);
  if (nd > 0) {
    // Sigma_dd = L_dd^{-T} L_dd^{-1} = U_d U_d^T   (RGF.H:439-442)
    gemm(h, mk(ind, ind, ind, Ud, nd, 0, Ud, nd, 1, nullptr, 0, Sdd, nd, 1.0, 0.0), SMALL);
  }
  const bool compat = h->opts.selinv_mode == RGF_SELINV_COMPAT;
  for (long long i = nt - 1; i >= 0; --i) {
    const double* P = h->d_MF + mf_col_offset(sh, i);
    double* Q = h->d_MS + mf_col_offset(sh, i);
    const long long lda = mf_lda(sh, i);
    const double* Ui = h->d_U + i * ss;
    const double* Bi = P + ns;                      // L_{i+1,i}
    const double* Ci = P + mf_dense_row(sh, i);     // C_i
    const bool has_next = i < nt - 1;
    const double* Sn = has_next ? h->d_MS + mf_col_offset(sh, i + 1) : nullptr;  // Sigma_{i+1,i+1}
    const long long ldn = has_next ? mf_lda(sh, i + 1) : 0;
    const double* Sdn = has_next ? Sn + mf_dense_row(sh, i + 1) : nullptr;       // Sigma_{d,i+1}
    if (!compat) {
      // Rows below the diagonal block are [L_{i+1,i}; C_i] = P + ns and
      // [Sigma_{i+1,i}; Sigma_{d,i}] = Q + ns (adjacent), so the products that
      // produce or consume them run once over ns + nd rows instead of as a
      // square product plus a thin nd-row one.
      if (has_next) {
        const int m2 = ins + ind;
        const long long ldt = m2;
        // [X; Y] = [Sigma_{i+1,i+1}; Sigma_{d,i+1}] L_{i+1,i}
        //          + [Sigma_{d,i+1}^T C_i; Sigma_dd C_i]
        GemmDesc x = mk(m2, ins, ins, Sn, ldn, 0, Bi, lda, 0, nullptr, 0, h->d_T1, ldt, 1.0, 0.0);
        if (nd > 0) {
          x.A2 = Sdn;
          x.mA1 = ins;
        }
        gemm(h, x, BULK);
        if (nd > 0) {
          gemm(h, mk(ins, ins, ind, Sdn, ldn, 1, Ci, lda, 0, h->d_T1, ldt, h->d_T1, ldt, 1.0, 1.0),
               SMALL);
          gemm(h, mk(ind, ins, ind, Sdd, nd, 0, Ci, lda, 0, h->d_T1 + ns, ldt, h->d_T1 + ns, ldt,
                     1.0, 1.0), SMALL);
        }
        // [Sigma_{i+1,i}; Sigma_{d,i}] = -[X; Y] L_ii^{-1} = -[X; Y] U_i^T
        GemmDesc g = mk(m2, ins, ins, h->d_T1, ldt, 0, Ui, ns, 1, nullptr, 0, Q + ns, lda, -1.0, 0.0);
        g.triB = TRI_LOWER;
        gemm(h, g, BULK);
        // W^T = U_i - [Sigma_{i+1,i}; Sigma_{d,i}]^T [L_{i+1,i}; C_i]
        gemm(h, mk(ins, ins, m2, Q + ns, lda, 1, Bi, lda, 0, Ui, ns, h->d_T2, ns, -1.0, 1.0), BULK);
      } else {
        if (nd > 0) {
          // Y = Sigma_dd C_i;  Sigma_{d,i} = -Y U_i^T
          gemm(h, mk(ind, ins, ind, Sdd, nd, 0, Ci, lda, 0, nullptr, 0, h->d_T3, nd, 1.0, 0.0),
               SMALL);
          GemmDesc g = mk(ind, ins, ins, h->d_T3, nd, 0, Ui, ns, 1, nullptr, 0,
                          Q + mf_dense_row(sh, i), lda, -1.0, 0.0);
          g.triB = TRI_LOWER;
          gemm(h, g, BULK);
          // W^T = U_i - Sigma_{d,i}^T C_i
          gemm(h, mk(ins, ins, ind, Q + mf_dense_row(sh, i), lda, 1, Ci, lda, 0, Ui, ns, h->d_T2,
                     ns, -1.0, 1.0), SMALL);
        } else {
          launch_copy(Ui, ns, h->d_T2, ns, ins, ins, 1, 0, 0, s);
          h->kernels_issued++;
        }
      }
      // Sigma_ii = L_ii^{-T} W = U_i (W^T)^T, symmetric: only its lower
      // triangle is computed (the output tiles above the diagonal, nearly
      // half, are skipped), then mirrored
      GemmDesc g = mk(ins, ins, ins, Ui, ns, 0, h->d_T2, ns, 1, nullptr, 0, Q, lda, 1.0, 0.0);
      g.triA = TRI_UPPER;
      g.outLower = 1;
      gemm(h, g, BULK);
      launch_mirror_lower(Q, lda, ins, s);
      h->kernels_issued++;
    } else {
      // the reference's recursion (RGF.H:444-502):
      // Sigma_ii = L^{-T} (I + B^T Sigma_{i+1,i+1} B + C^T Sigma_dd C) L^{-1}
      launch_set_identity(h->d_T2, ns, ins, 1, 0, s);
      h->kernels_issued++;
      if (has_next) {
        gemm(h, mk(ins, ins, ins, Sn, ldn, 0, Bi, lda, 0, nullptr, 0, h->d_T1, ns, 1.0, 0.0), BULK);
        gemm(h, mk(ins, ins, ins, Bi, lda, 1, h->d_T1, ns, 0, h->d_T2, ns, h->d_T2, ns, 1.0, 1.0),
             BULK);
      }
      if (nd > 0) {
        gemm(h, mk(ind, ins, ind, Sdd, nd, 0, Ci, lda, 0, nullptr, 0, h->d_T3, nd, 1.0, 0.0), SMALL);
        gemm(h, mk(ins, ins, ind, Ci, lda, 1, h->d_T3, nd, 0, h->d_T2, ns, h->d_T2, ns, 1.0, 1.0),
             SMALL);
      }
      GemmDesc g1 = mk(ins, ins, ins, h->d_T2, ns, 0, Ui, ns, 1, nullptr, 0, h->d_T1, ns, 1.0, 0.0);
      g1.triB = TRI_LOWER;
      gemm(h, g1, BULK);
      GemmDesc g2 = mk(ins, ins, ins, Ui, ns, 0, h->d_T1, ns, 0, nullptr, 0, Q, lda, 1.0, 0.0);
      g2.triA = TRI_UPPER;
      gemm(h, g2, BULK);
    }
  }
  launch_extract_diag(sh, h->d_MS, h->d_diag, s);
  h->kernels_issued++;
}

// L X = R (left, lower, no transpose) for the ns x nrhs block R (ld ldr).
void trsv_lower(rgf_handle* h, const double* L, long long ldl, int m, double* R, long long ldr,
                int nrhs) {
  for (int k0 = 0; k0 < m; k0 += NB) {
    const int nbk = std::min(NB, m - k0);
    const double* Lkk = L + k0 + (long long)k0 * ldl;
    trsm_rows(h, R + k0, ldr, 1, nrhs, Lkk, ldl, nbk, 0);
    const int rem = m - k0 - nbk;
    if (rem > 0)
      gemm(h, mk(rem, nrhs, nbk, Lkk + nbk, ldl, 0, R + k0, ldr, 0, R + k0 + nbk, ldr,
                 R + k0 + nbk, ldr, -1.0, 1.0), SMALL);
  }
}

// L^T X = R (left, lower, transposed).
void trsv_lower_t(rgf_handle* h, const double* L, long long ldl, int m, double* R, long long ldr,
                  int nrhs) {
  const int nblk = (m + NB - 1) / NB;
  for (int b = nblk - 1; b >= 0; --b) {
    const int k0 = b * NB;
    const int nbk = std::min(NB, m - k0);
    const double* Lkk = L + k0 + (long long)k0 * ldl;
    trsm_rows(h, R + k0, ldr, 1, nrhs, Lkk, ldl, nbk, 1);
    if (k0 > 0)
      gemm(h, mk(k0, nrhs, nbk, L + k0, ldl, 1, R + k0, ldr, 0, R, ldr, R, ldr, -1.0, 1.0), SMALL);
  }
}

// ---- stage 2: solve (RGF.H:344-418) on the device buffer d_rhs ----
// Block substitution with the inverted diagonal blocks U_i = L_ii^{-T}: every
// step is a product (FP64, spread over the GPU by split K) instead of a chain
// of small triangular solves.  y lives in d_rhs2, b and then x in d_rhs.
void issue_solve(rgf_handle* h, int nrhs) {
  const BtaShape& sh = h->sh;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd, n = sh.n;
  const int ins = (int)ns, ind = (int)nd;
  const long long ss = ns * ns;
  double* R = h->d_rhs;
  double* Y = h->d_rhs2;
  const double* corner = h->d_MF + mf_col_offset(sh, nt);
  for (long long i = 0; i < nt; ++i) {
    if (i > 0) {  // b_i -= L_{i,i-1} y_{i-1}   (RGF.H:365)
      const double* Pm = h->d_MF + mf_col_offset(sh, i - 1);
      gemm(h, mk(ins, nrhs, ins, Pm + ns, mf_lda(sh, i - 1), 0, Y + (i - 1) * ns, n, 0,
                 R + i * ns, n, R + i * ns, n, -1.0, 1.0), SMALL);
    }
    // y_i = L_ii^{-1} b_i = U_i^T b_i   (RGF.H:356, 367)
    GemmDesc g = mk(ins, nrhs, ins, h->d_U + i * ss, ns, 1, R + i * ns, n, 0, nullptr, 0,
                    Y + i * ns, n, 1.0, 0.0);
    g.triA = TRI_LOWER;
    gemm(h, g, SMALL);
  }
  if (nd > 0) {
    // b_d -= sum_i C_i y_i; y_d, then x_d, by the corner factor   (RGF.H:377-393)
    launch_arrow_gemv(sh, h->d_MF, Y, n, nrhs, h->d_partial, h->stream);
    launch_arrow_reduce(sh, h->d_partial, nrhs, R, n, h->stream);
    h->kernels_issued += 2;
    trsv_lower(h, corner, nd, ind, R + nt * ns, n, nrhs);
    trsv_lower_t(h, corner, nd, ind, R + nt * ns, n, nrhs);
    // y_i -= C_i^T x_d for every block column (RGF.H:396-399)
    if (nt > 1) {
      GemmDesc g = mk(ins, nrhs, ind, h->d_MF + 2 * ns, 2 * ns + nd, 1, R + nt * ns, n, 0, Y, n, Y,
                      n, -1.0, 1.0);
      g.batch = (int)(nt - 1); g.sA = ns * (2 * ns + nd); g.sB = 0; g.sC = g.sD = ns;
      gemm(h, g, SMALL);
    }
    const double* Pl = h->d_MF + mf_col_offset(sh, nt - 1);
    gemm(h, mk(ins, nrhs, ind, Pl + ns, ns + nd, 1, R + nt * ns, n, 0, Y + (nt - 1) * ns, n,
               Y + (nt - 1) * ns, n, -1.0, 1.0), SMALL);
  }
  for (long long i = nt - 1; i >= 0; --i) {
    if (i < nt - 1) {  // y_i -= L_{i+1,i}^T x_{i+1}   (RGF.H:410)
      const double* P = h->d_MF + mf_col_offset(sh, i);
      gemm(h, mk(ins, nrhs, ins, P + ns, mf_lda(sh, i), 1, R + (i + 1) * ns, n, 0, Y + i * ns, n,
                 Y + i * ns, n, -1.0, 1.0), SMALL);
    }
    // x_i = L_ii^{-T} y_i = U_i y_i   (RGF.H:408, 417)
    GemmDesc g = mk(ins, nrhs, ins, h->d_U + i * ss, ns, 0, Y + i * ns, n, 0, nullptr, 0,
                    R + i * ns, n, 1.0, 0.0);
    g.triA = TRI_UPPER;
    gemm(h, g, SMALL);
  }
}

// ---- asynchronous upload ----
// Queue the CSC on the upload stream in block-column chunks (the arrowhead
// corner first, then block columns 0, 1, ... in factorization order): each
// chunk's rows and values are copied, its MF panel cleared and its columns
// ingested, then ev_chunk[i] is recorded.  Nothing waits here; the caller's
// arrays are read until the first factorization (or finish_upload) returns,
// as the reference reads them during factorize (RGF.H:87-89, 689-698).
int start_upload(rgf_handle* h, const size_t* ia, const size_t* ja, const double* a) {
  const BtaShape& sh = h->sh;
  const long long nblk = sh.nt + (sh.nd > 0 ? 1 : 0);
  RGF_CK(cudaStreamCreateWithFlags(&h->upload, cudaStreamNonBlocking));
  h->ev_chunk.assign((size_t)nblk, nullptr);
  for (auto& e : h->ev_chunk) RGF_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaStream_t u = h->upload;
  // after what create queued on the main stream (workspace clears)
  RGF_CK(cudaEventRecord(h->ev_fork, h->stream));
  RGF_CK(cudaStreamWaitEvent(u, h->ev_fork, 0));
  status_init_kernel<<<1, 1, 0, u>>>(h->d_status);
  RGF_CK(cudaMemcpyAsync(h->d_ia, ia, sizeof(size_t) * (sh.n + 1), cudaMemcpyHostToDevice, u));
  h->upload_pending = true;  // from here on release() waits for the stream
  for (long long q = 0; q < nblk; ++q) {
    const long long i = sh.nd > 0 ? (q == 0 ? sh.nt : q - 1) : q;
    const long long c0 = i * sh.ns, c1 = i < sh.nt ? c0 + sh.ns : sh.n;
    const size_t e0 = ia[c0], e1 = ia[c1];
    if (e1 > e0) {
      RGF_CK(cudaMemcpyAsync(h->d_ja + e0, ja + e0, sizeof(size_t) * (e1 - e0),
                             cudaMemcpyHostToDevice, u));
      RGF_CK(cudaMemcpyAsync(h->d_a + e0, a + e0, sizeof(double) * (e1 - e0),
                             cudaMemcpyHostToDevice, u));
    }
    const long long o0 = mf_col_offset(sh, i);
    const long long o1 = i < sh.nt ? mf_col_offset(sh, i + 1) : h->mf_size;
    RGF_CK(cudaMemsetAsync(h->d_MF + o0, 0, sizeof(double) * (o1 - o0), u));
    launch_ingest(sh, h->d_ia, h->d_ja, h->d_a, h->d_MF, h->d_status, u, c0, c1);
    RGF_CK(cudaGetLastError());
    RGF_CK(cudaEventRecord(h->ev_chunk[(size_t)i], u));
  }
  h->mf_holds_a = true;
  return RGF_OK;
}

// Wait (on the host) until the asynchronous upload is complete; afterwards
// nothing reads the caller's arrays.  With check, a pattern error that the
// ingests recorded is reported now, as a synchronous create would have.
int finish_upload(rgf_handle* h, bool check) {
  if (!h->upload_pending) return RGF_OK;
  h->upload_pending = false;
  RGF_CK(cudaStreamSynchronize(h->upload));
  RGF_CK(cudaGetLastError());
  if (!check) return RGF_OK;
  DevStatus st;
  RGF_CK(cudaMemcpy(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st.bad_input) {
    h->mf_holds_a = false;  // the next factorization ingests (and reports) again
    return RGF_EINVAL;
  }
  return RGF_OK;
}

// ---- graph capture / replay ----
// The first run of a stage launches its kernels directly; from the second run
// on, the stage is captured once into a CUDA graph and replayed.  A handle
// used once (create, factorize, RGFdiag, destroy) never pays for a capture
// and instantiation of tens of thousands of nodes.  With the kernel timer on
// the stage runs launch by launch.
template <class F>
int run_stage(rgf_handle* h, cudaGraphExec_t* exec, long long* nk, int* runs, F issue) {
  const bool direct =
      h->timer_on || !h->trace_path.empty() || !h->opts.use_graphs || (!*exec && (*runs)++ == 0);
  // a run that waits for an asynchronous upload is launched directly (its
  // waits are on events recorded outside any capture)
  if (direct || h->upload_pending) {
    h->kernels_issued = 0;
    if (!h->trace_path.empty()) {
      if (!h->trace_t0) cudaEventCreate(&h->trace_t0);
      cudaEventRecord(h->trace_t0, h->stream);
    }
    issue();
    h->kernels_total += h->kernels_issued;
    RGF_CK(cudaGetLastError());
    return RGF_OK;
  }
  if (!*exec) {
    cudaGraph_t graph = nullptr;
    h->kernels_issued = 0;
    RGF_CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    issue();
    cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (e != cudaSuccess) return cuda_status(e);
    e = cudaGraphInstantiateWithFlags(exec, graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      *exec = nullptr;
      return cuda_status(e);
    }
    *nk = h->kernels_issued;
  }
  RGF_CK(cudaGraphLaunch(*exec, h->stream));
  h->kernels_total += *nk;
  return RGF_OK;
}

int collect_timer(rgf_handle* h) {
  for (const auto& t : h->ev_used) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t.e0, t.e1);
    for (int k : {0, t.kind}) {
      h->timer_ms[k] += ms;
      h->timer_flops[k] += t.flops;
      h->timer_launches[k]++;
    }
    h->timer_tflops += t.tensor_flops;
    if (h->timer_detail_on) {
      char key[128];
      std::snprintf(key, sizeof(key), "%s cls%d m%5d n%5d k%5d b%4d", t.kind == 2 ? "split" : "fp64 ",
                    t.cls, t.m, t.n, t.k, t.batch);
      auto& e = h->timer_detail[key];
      e.first++;
      e.second += ms;
    }
    h->ev_pool.push_back({t.e0, t.e1});
  }
  h->ev_used.clear();
  return RGF_OK;
}

int sync_and_check(rgf_handle* h) {
  RGF_CK(cudaStreamSynchronize(h->stream));
  RGF_CK(cudaGetLastError());
  if (h->timer_on) collect_timer(h);
  trace_flush(h);
  DevStatus st;
  RGF_CK(cudaMemcpy(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost));
  if (st.timeout) {
    // a split product that gave up may have left its split-K workspace dirty
    for (SplitEngine* e : {h->split, h->split_side})
      if (e) e->reset_splitk(h->stream);
    cudaStreamSynchronize(h->stream);
    return RGF_ETIMEOUT;
  }
  if (st.bad_input) return RGF_EINVAL;
  if (st.not_spd_col != INT_MAX) {
    h->not_spd_col = st.not_spd_col;
    return RGF_ENOTSPD;
  }
  h->not_spd_col = -1;
  return RGF_OK;
}

int ensure_factored(rgf_handle* h) {
  if (h->factored) return RGF_OK;
  const bool streamed = h->upload_pending;
  int st = run_stage(h, &h->g_factor, &h->k_factor, &h->runs_factor, [&] { issue_factor(h); });
  if (streamed) {  // the stage waited for every block column; the copies are done too
    const int su = finish_upload(h, false);
    if (!st) st = su;
  }
  if (st) return st;
  st = sync_and_check(h);
  if (st) return st;
  h->factored = true;
  h->selinv_done = false;
  h->inv_done = false;
  return RGF_OK;
}

int alloc_selinv(rgf_handle* h) {
  if (h->d_MS) return RGF_OK;
  const long long ns = h->sh.ns, nt = h->sh.nt, nd = h->sh.nd;
  int st;
  if ((st = dalloc(h, &h->d_MS, h->mf_size))) return st;
  if ((st = dalloc(h, &h->d_U, nt * ns * ns + nd * nd))) return st;
  if ((st = dalloc(h, &h->d_T1, (ns + nd) * ns))) return st;
  if ((st = dalloc(h, &h->d_T2, ns * ns))) return st;
  if ((st = dalloc(h, &h->d_T3, std::max<long long>(1, nd * ns)))) return st;
  RGF_CK(cudaMemsetAsync(h->d_MS, 0, sizeof(double) * h->mf_size, h->stream));
  return RGF_OK;
}

int ensure_selinv(rgf_handle* h) {
  int st = ensure_factored(h);
  if (st) return st;
  if (h->selinv_done) return RGF_OK;
  if ((st = alloc_selinv(h))) return st;
  st = run_stage(h, &h->g_selinv, &h->k_selinv, &h->runs_selinv, [&] { issue_selinv(h); });
  if (st) return st;
  st = sync_and_check(h);
  if (st) return st;
  h->selinv_done = true;
  h->inv_done = true;
  return RGF_OK;
}

// The diagonal-block inverses the solve uses (computed by the selected
// inversion too).
int ensure_inverses(rgf_handle* h) {
  int st = ensure_factored(h);
  if (st) return st;
  if (h->inv_done) return RGF_OK;
  if ((st = alloc_selinv(h))) return st;
  st = run_stage(h, &h->g_inv, &h->k_inv, &h->runs_inv, [&] { issue_inverses(h); });
  if (st) return st;
  st = sync_and_check(h);
  if (st) return st;
  h->inv_done = true;
  return RGF_OK;
}

// Whether host memory is page-locked (cudaHostAlloc / cudaHostRegister), so
// that an asynchronous copy from it returns at once; from pageable memory the
// calling thread stages every copy itself, and a chunked upload only adds
// copies (measured much slower under concurrent requests).
bool page_locked(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

int validate_host_csc(const size_t* ia, long long n) {
  if (ia[0] != 0) return RGF_EINVAL;
  for (long long c = 0; c < n; ++c)
    if (ia[c + 1] < ia[c]) return RGF_EINVAL;
  return RGF_OK;
}

void release(rgf_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  // nothing may still use a buffer when it goes back to an arena (no
  // implicit synchronization there, unlike cudaFree)
  if (h->upload) cudaStreamSynchronize(h->upload);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->g_factor) cudaGraphExecDestroy(h->g_factor);
  if (h->g_selinv) cudaGraphExecDestroy(h->g_selinv);
  if (h->g_inv) cudaGraphExecDestroy(h->g_inv);
  for (auto& kv : h->g_solve) cudaGraphExecDestroy(kv.second.first);
  for (auto& e : h->ev_used) { cudaEventDestroy(e.e0); cudaEventDestroy(e.e1); }
  for (auto& e : h->ev_pool) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto& t : h->trace) cudaEventDestroy(t.ev);
  if (h->trace_t0) cudaEventDestroy(h->trace_t0);
  delete h->split;
  delete h->split_side;
  void* bufs[] = {h->d_ia, h->d_ja, h->d_a, h->d_MF, h->d_MS, h->d_U, h->d_T1, h->d_T2, h->d_T3,
                  h->d_logpart, h->d_scalars, h->d_diag, h->d_status, h->d_rhs, h->d_partial,
                  h->d_res, h->d_gemm_ws, h->d_gemm_ws_side, h->d_ref, h->d_rhs2,
                  h->d_norms};
  for (void* p : bufs) dfree(p);
  if (h->ev_fork) cudaEventDestroy(h->ev_fork);
  if (h->ev_join) cudaEventDestroy(h->ev_join);
  for (cudaEvent_t e : h->ev_chunk)
    if (e) cudaEventDestroy(e);
  if (h->upload) cudaStreamDestroy(h->upload);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

// Discard the captured stage graphs (their kernels were cut with the old
// knobs) and the results computed so far: the next run of every stage
// launches directly, the one after captures again.
int drop_graphs(rgf_handle* h) {
  RGF_CK(cudaStreamSynchronize(h->stream));
  RGF_CK(cudaStreamSynchronize(h->side));
  for (cudaGraphExec_t* g : {&h->g_factor, &h->g_selinv, &h->g_inv}) {
    if (*g) cudaGraphExecDestroy(*g);
    *g = nullptr;
  }
  for (auto& kv : h->g_solve) cudaGraphExecDestroy(kv.second.first);
  h->g_solve.clear();
  h->runs_solve.clear();
  h->runs_factor = h->runs_selinv = h->runs_inv = 0;
  h->k_factor = h->k_selinv = h->k_inv = 0;
  h->factored = h->selinv_done = h->inv_done = false;
  return RGF_OK;
}

}  // namespace

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

const char* rgf_status_string(int status) {
  switch (status) {
    case RGF_OK: return "RGF_OK";
    case RGF_EINVAL: return "RGF_EINVAL: invalid argument or CSC outside the block pattern";
    case RGF_ENOMEM: return "RGF_ENOMEM: device allocation failed";
    case RGF_ENOTSPD: return "RGF_ENOTSPD: matrix is not positive definite";
    case RGF_ECUDA: return "RGF_ECUDA: CUDA error or no usable device";
    case RGF_ETIMEOUT: return "RGF_ETIMEOUT: a bounded device wait gave up";
    case RGF_ENOTSUP: return "RGF_ENOTSUP: option not supported";
    default: return "unknown rgf status";
  }
}

int rgf_default_opts(rgf_opts* o) {
  if (!o) return RGF_EINVAL;
  std::memset(o, 0, sizeof(*o));
  o->precision = RGF_PREC_FP64;
  o->slices = 0;
  o->selinv_mode = RGF_SELINV_EXACT;
  o->device = -1;
  o->use_graphs = 1;
  o->fp64_diag = 1;
  o->async_upload = 0;
  return RGF_OK;
}

int rgf_create(const size_t* ia, const size_t* ja, const double* a, size_t ns, size_t nt,
               size_t nd, const rgf_opts* opts, rgf_handle** out) {
  if (!out) return RGF_EINVAL;
  *out = nullptr;
  if (!ia || !ja || !a || ns < 1 || nt < 1) return RGF_EINVAL;
  if (ns > (1u << 20) || nd > (1u << 20) || nt > (1u << 24)) return RGF_EINVAL;
  const long long n = (long long)(ns * nt + nd);
  if (n >= INT_MAX) return RGF_EINVAL;
  if (validate_host_csc(ia, n)) return RGF_EINVAL;
  rgf_opts o;
  rgf_default_opts(&o);
  if (opts) o = *opts;
  if (o.precision != RGF_PREC_FP64 && o.precision != RGF_PREC_SPLIT) return RGF_EINVAL;
  if (o.selinv_mode != RGF_SELINV_EXACT && o.selinv_mode != RGF_SELINV_COMPAT) return RGF_EINVAL;
  if (o.slices < 0 || o.slices > 8) return RGF_EINVAL;
  if (o.fp64_diag < 0 || o.fp64_diag > 2) return RGF_EINVAL;
  if (o.async_upload < 0 || o.async_upload > 1) return RGF_EINVAL;

  int dev = o.device;
  if (dev < 0) {
    if (cudaGetDevice(&dev) != cudaSuccess) return RGF_ECUDA;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0 || dev >= ndev) {
    cudaGetLastError();
    return RGF_ECUDA;
  }
  if (cudaSetDevice(dev) != cudaSuccess) return RGF_ECUDA;
  // the asynchronous upload needs page-locked arrays (else: copied now)
  const bool async = o.async_upload && page_locked(ia) && page_locked(ja) && page_locked(a);

  rgf_handle* h = new (std::nothrow) rgf_handle();
  if (!h) return RGF_ENOMEM;
  h->device = dev;
  h->opts = o;
  // Split precision leaves the FP64 kernel the small, latency-bound products of
  // the diagonal-block chain and the batched inverses, which run faster cut
  // into 32 x 32 tiles (more CTAs) whatever their size: measured 3.5% on
  // factorize + RGFdiag at ns = 2000.
  if (o.precision == RGF_PREC_SPLIT) h->fp64_tile = 32;
  h->sh = {(long long)ns, (long long)nt, (long long)nd, n};
  h->nnz = (long long)ia[n];
  h->mf_size = 2 * (long long)(nt - 1) * ns * ns + (long long)ns * ns + n * (long long)nd;
  int st = RGF_OK;
  do {
    // the main stream carries the critical path: give it the higher priority
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio_lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess) {
      st = RGF_ECUDA;
      break;
    }
    if (const char* e = std::getenv("RGF_GB300_LOOKAHEAD")) h->lookahead = std::atoi(e) != 0;
    if (const char* e = std::getenv("RGF_GB300_TRACE")) h->trace_path = e;
    if ((st = dalloc(h, &h->d_ia, n + 1))) break;
    if ((st = dalloc(h, &h->d_ja, h->nnz))) break;
    if ((st = dalloc(h, &h->d_a, h->nnz))) break;
    if ((st = dalloc(h, &h->d_MF, h->mf_size))) break;
    if (const char* e = std::getenv("RGF_GB300_LEAF_NB")) {
      const int v = std::atoi(e);
      if (v == 16 || v == 32 || v == 64) h->nb = v;
    }
    h->nparts = logdet_parts(h->sh);
    if ((st = dalloc(h, &h->d_logpart, h->nparts))) break;
    if ((st = dalloc(h, &h->d_scalars, 8))) break;
    if ((st = dalloc(h, &h->d_diag, n))) break;
    if ((st = dalloc(h, &h->d_status, 1))) break;
    h->gemm_ws_elems = std::min<long long>(20ll << 20, 8ll * (2 * (long long)ns + (long long)nd) *
                                                           std::max<long long>(ns, nd));
    if ((st = dalloc(h, &h->d_gemm_ws, h->gemm_ws_elems))) break;
    if ((st = dalloc(h, &h->d_gemm_ws_side, h->gemm_ws_elems))) break;
    // the CSC goes up in two halves on the two streams, so that two copy
    // engines move it at once; the main stream joins before anything reads it
    // (asynchronous upload: below, in block-column chunks)
    if (!async) {
      const size_t h1 = (size_t)h->nnz / 2, h2 = (size_t)h->nnz - h1;
      if (cudaMemcpyAsync(h->d_ia, ia, sizeof(size_t) * (n + 1), cudaMemcpyHostToDevice,
                          h->stream) ||
          cudaMemcpyAsync(h->d_ja, ja, sizeof(size_t) * h1, cudaMemcpyHostToDevice, h->stream) ||
          cudaMemcpyAsync(h->d_a, a, sizeof(double) * h1, cudaMemcpyHostToDevice, h->stream) ||
          cudaMemcpyAsync(h->d_ja + h1, ja + h1, sizeof(size_t) * h2, cudaMemcpyHostToDevice,
                          h->side) ||
          cudaMemcpyAsync(h->d_a + h1, a + h1, sizeof(double) * h2, cudaMemcpyHostToDevice,
                          h->side)) {
        st = RGF_ECUDA;
        break;
      }
      join_side(h);
    }
    if (o.precision == RGF_PREC_SPLIT) {
      h->split = SplitEngine::create(o.slices, &st);
      if (st) break;
      // operands have at most 2ns+nd rows and ns+nd terms
      st = h->split->prepare((int)(2 * ns + nd), (int)(ns + nd), (int)nt, h->stream);
      if (st) break;
      h->split_side = SplitEngine::create(o.slices, &st);
      if (st) break;
      st = h->split_side->prepare((int)(ns + nd), (int)ns, 1, h->stream);
      if (st) break;
    }
    if (async) {  // copies and ingests overlap the first factorization
      st = start_upload(h, ia, ja, a);
      break;
    }
    // validate the pattern once on the device
    status_init_kernel<<<1, 1, 0, h->stream>>>(h->d_status);
    cudaMemsetAsync(h->d_MF, 0, sizeof(double) * h->mf_size, h->stream);
    launch_ingest(h->sh, h->d_ia, h->d_ja, h->d_a, h->d_MF, h->d_status, h->stream);
    st = sync_and_check(h);
    if (!st) h->mf_holds_a = true;
  } while (0);
  if (st) {
    release(h);
    return st;
  }
  *out = h;
  return RGF_OK;
}

int rgf_create_hermitian(const size_t* ia, const size_t* ja, const double* a, size_t ns,
                         size_t nt, size_t nd, const rgf_opts* opts, rgf_handle** out) {
  if (!out) return RGF_EINVAL;
  *out = nullptr;
  if (!ia || !ja || !a || ns < 1 || nt < 1) return RGF_EINVAL;
  if (ns > (1u << 19) || nd > (1u << 19) || nt > (1u << 24)) return RGF_EINVAL;
  if (validate_host_csc(ia, (long long)(ns * nt + nd))) return RGF_EINVAL;
  std::vector<size_t> ia2, ja2;
  std::vector<double> a2;
  int st = hermitian_embed(ia, ja, a, ns, nt, nd, ia2, ja2, a2);
  if (st) return st;
  rgf_opts o;
  rgf_default_opts(&o);
  if (opts) o = *opts;
  o.async_upload = 0;  // the embedding is freed on return: copy it now
  st = rgf_create(ia2.data(), ja2.data(), a2.data(), 2 * ns, nt, 2 * nd, &o, out);
  if (st) return st;
  rgf_handle* h = *out;
  h->hermitian = true;
  h->hns = ns; h->hnt = nt; h->hnd = nd;
  h->nc = ns * nt + nd;
  return RGF_OK;
}

int rgf_destroy(rgf_handle* h) {
  if (!h) return RGF_EINVAL;
  release(h);
  return RGF_OK;
}

int rgf_factorize(rgf_handle* h) {
  if (!h) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  h->factored = false;
  h->selinv_done = false;
  return ensure_factored(h);
}

int rgf_logdet(rgf_handle* h, double* logdet) {
  if (!h || !logdet) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  int st = ensure_factored(h);
  if (st) return st;
  RGF_CK(cudaMemcpy(logdet, h->d_scalars, sizeof(double), cudaMemcpyDeviceToHost));
  if (h->hermitian) *logdet *= 0.5;  // det M = det(A)^2
  return RGF_OK;
}

int rgf_diag(rgf_handle* h, double* diag) {
  if (!h || !diag) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  int st = ensure_selinv(h);
  if (st) return st;
  if (h->hermitian) {  // diag(A^{-1})_k = (M^{-1})_{Re k, Re k}, imaginary part 0
    std::vector<double> d((size_t)h->sh.n);
    RGF_CK(cudaMemcpy(d.data(), h->d_diag, sizeof(double) * d.size(), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < h->nc; ++k) {
      diag[2 * k] = d[hermitian_real_index(h->hns, h->hnt, h->hnd, k, 0)];
      diag[2 * k + 1] = 0.0;
    }
    return RGF_OK;
  }
  RGF_CK(cudaMemcpy(diag, h->d_diag, sizeof(double) * h->sh.n, cudaMemcpyDeviceToHost));
  return RGF_OK;
}

int rgf_diag_device(rgf_handle* h, const double** d_diag) {
  if (!h || !d_diag) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  int st = ensure_selinv(h);
  if (st) return st;
  *d_diag = h->d_diag;
  return RGF_OK;
}

// complex (interleaved) n_c x nrhs <-> real embedded 2 n_c x nrhs
static void hermitian_to_real(const rgf_handle* h, const double* z, size_t nrhs, double* r) {
  const size_t nc = h->nc, n2 = 2 * nc;
  for (size_t q = 0; q < nrhs; ++q)
    for (size_t k = 0; k < nc; ++k) {
      r[q * n2 + hermitian_real_index(h->hns, h->hnt, h->hnd, k, 0)] = z[2 * (q * nc + k)];
      r[q * n2 + hermitian_real_index(h->hns, h->hnt, h->hnd, k, 1)] = z[2 * (q * nc + k) + 1];
    }
}
static void real_to_hermitian(const rgf_handle* h, const double* r, size_t nrhs, double* z) {
  const size_t nc = h->nc, n2 = 2 * nc;
  for (size_t q = 0; q < nrhs; ++q)
    for (size_t k = 0; k < nc; ++k) {
      z[2 * (q * nc + k)] = r[q * n2 + hermitian_real_index(h->hns, h->hnt, h->hnd, k, 0)];
      z[2 * (q * nc + k) + 1] = r[q * n2 + hermitian_real_index(h->hns, h->hnt, h->hnd, k, 1)];
    }
}

static int solve_real(rgf_handle* h, double* x, const double* b, size_t nrhs);

int rgf_solve(rgf_handle* h, double* x, const double* b, size_t nrhs) {
  if (!h || !x || !b) return RGF_EINVAL;
  if (nrhs == 0) return RGF_OK;
  if (nrhs > 4096) return RGF_EINVAL;
  if (!h->hermitian) return solve_real(h, x, b, nrhs);
  std::vector<double> br(2 * h->nc * nrhs), xr(2 * h->nc * nrhs);
  hermitian_to_real(h, b, nrhs, br.data());
  const int st = solve_real(h, xr.data(), br.data(), nrhs);
  if (st) return st;
  real_to_hermitian(h, xr.data(), nrhs, x);
  return RGF_OK;
}

static int solve_real(rgf_handle* h, double* x, const double* b, size_t nrhs) {
  if (nrhs == 0) return RGF_OK;
  if (nrhs > 4096) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  int st = ensure_inverses(h);
  if (st) return st;
  const long long n = h->sh.n;
  const size_t need = (size_t)n * nrhs;
  if (need > h->rhs_cap) {
    for (auto& kv : h->g_solve) cudaGraphExecDestroy(kv.second.first);
    h->g_solve.clear();
    dfree(h->d_rhs);
    dfree(h->d_rhs2);
    h->d_rhs2 = nullptr;
    h->device_bytes -= 2 * h->rhs_cap * sizeof(double);
    h->rhs_cap = 0;
    if ((st = dalloc(h, &h->d_rhs, need))) return st;
    if ((st = dalloc(h, &h->d_rhs2, need))) return st;
    h->rhs_cap = need;
  }
  const size_t pneed = (size_t)h->sh.nt * nrhs * std::max<long long>(1, h->sh.nd);
  if (pneed > h->partial_cap) {
    for (auto& kv : h->g_solve) cudaGraphExecDestroy(kv.second.first);
    h->g_solve.clear();
    dfree(h->d_partial);
    h->device_bytes -= h->partial_cap * sizeof(double);
    h->partial_cap = 0;
    if ((st = dalloc(h, &h->d_partial, pneed))) return st;
    h->partial_cap = pneed;
  }
  // Split precision: the factor is accurate to ~1e-10, so the solve is
  // refined in FP64: r = b - A x from the resident CSC (one pass over it for
  // up to 16 right-hand sides), and while some normalized residual is above
  // RGF_REFINE_TOL, x += A~^{-1} r with the same factor (at most
  // RGF_REFINE_STEPS times).
  const bool refine = h->opts.precision == RGF_PREC_SPLIT;
  if (refine && !h->d_norms && (st = dalloc(h, &h->d_norms, 2 * 4096))) return st;
  if (refine && need * 3 > h->ref_cap) {
    for (auto& kv : h->g_solve) cudaGraphExecDestroy(kv.second.first);  // they name d_ref
    h->g_solve.clear();
    dfree(h->d_ref);
    h->device_bytes -= h->ref_cap * sizeof(double);
    h->ref_cap = 0;
    if ((st = dalloc(h, &h->d_ref, need * 3))) return st;
    h->ref_cap = need * 3;
  }
  double* xr = h->d_ref;
  double* br = refine ? h->d_ref + need : nullptr;
  double* yr = refine ? h->d_ref + 2 * need : nullptr;
  RGF_CK(cudaMemcpyAsync(h->d_rhs, b, sizeof(double) * need, cudaMemcpyHostToDevice, h->stream));
  if (refine)
    RGF_CK(cudaMemcpyAsync(br, h->d_rhs, sizeof(double) * need, cudaMemcpyDeviceToDevice,
                           h->stream));
  auto it = h->g_solve.find(nrhs);
  cudaGraphExec_t exec = it == h->g_solve.end() ? nullptr : it->second.first;
  long long nk = it == h->g_solve.end() ? 0 : it->second.second;
  const int passes = refine ? 1 + RGF_REFINE_STEPS : 1;
  std::vector<double> norms(refine ? 2 * nrhs : 0);
  for (int pass = 0; pass < passes; ++pass) {
    if (pass > 0) {  // d_rhs = b - A x; done when every residual is small
      launch_residual_vectors(n, (int)nrhs, h->d_ia, h->d_ja, h->d_a, xr, br, yr, h->d_rhs,
                              h->stream);
      launch_rhs_norms(n, (int)nrhs, h->d_rhs, br, h->d_norms, h->stream);
      RGF_CK(cudaMemcpyAsync(norms.data(), h->d_norms, sizeof(double) * 2 * nrhs,
                             cudaMemcpyDeviceToHost, h->stream));
      RGF_CK(cudaStreamSynchronize(h->stream));
      bool done = true;
      for (size_t q = 0; q < nrhs; ++q)
        if (!(norms[2 * q] <= RGF_REFINE_TOL * norms[2 * q + 1])) done = false;
      if (done) break;
    }
    st = run_stage(h, &exec, &nk, &h->runs_solve[nrhs], [&] { issue_solve(h, (int)nrhs); });
    if (st) return st;
    if (exec) h->g_solve[nrhs] = {exec, nk};
    if (refine) {
      if (pass == 0)
        RGF_CK(cudaMemcpyAsync(xr, h->d_rhs, sizeof(double) * need, cudaMemcpyDeviceToDevice,
                               h->stream));
      else
        launch_add((long long)need, xr, h->d_rhs, h->stream);
    }
  }
  RGF_CK(cudaMemcpyAsync(x, refine ? xr : h->d_rhs, sizeof(double) * need,
                         cudaMemcpyDeviceToHost, h->stream));
  return sync_and_check(h);
}

int rgf_residual_norm(rgf_handle* h, const double* x, const double* b, double* norm) {
  if (!h || !x || !b || !norm) return RGF_EINVAL;
  if (h->hermitian) {  // ||b - A x|| = ||b' - M x'|| for the embedded vectors
    std::vector<double> xr(2 * h->nc), br(2 * h->nc);
    hermitian_to_real(h, x, 1, xr.data());
    hermitian_to_real(h, b, 1, br.data());
    h->hermitian = false;
    const int st = rgf_residual_norm(h, xr.data(), br.data(), norm);
    h->hermitian = true;
    return st;
  }
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  const long long n = h->sh.n;
  int st = finish_upload(h, true);  // the product reads the device CSC
  if (st) return st;
  if (!h->d_res && (st = dalloc(h, &h->d_res, 3 * n))) return st;
  RGF_CK(cudaMemcpyAsync(h->d_res, x, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  RGF_CK(cudaMemcpyAsync(h->d_res + n, b, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
  RGF_CK(launch_residual(n, h->d_ia, h->d_ja, h->d_a, h->d_res, h->d_res + n, h->d_res + 2 * n,
                         h->d_scalars + 1, nullptr, h->stream));
  double out[2];
  RGF_CK(cudaMemcpyAsync(out, h->d_scalars + 1, sizeof(out), cudaMemcpyDeviceToHost, h->stream));
  RGF_CK(cudaStreamSynchronize(h->stream));
  RGF_CK(cudaGetLastError());
  *norm = out[0];
  return RGF_OK;
}

int rgf_residual_norm_normalized(rgf_handle* h, const double* x, const double* b, double* norm) {
  if (!h || !x || !b || !norm) return RGF_EINVAL;
  double r;
  int st = rgf_residual_norm(h, x, b, &r);
  if (st) return st;
  double out[2];
  RGF_CK(cudaMemcpy(out, h->d_scalars + 1, sizeof(out), cudaMemcpyDeviceToHost));
  *norm = out[0] / out[1];
  return RGF_OK;
}

int rgf_export_factor(rgf_handle* h, double* mf) {
  if (!h || !mf) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  int st = ensure_factored(h);
  if (st) return st;
  RGF_CK(cudaMemcpy(mf, h->d_MF, sizeof(double) * h->mf_size, cudaMemcpyDeviceToHost));
  return RGF_OK;
}

int rgf_export_selinv(rgf_handle* h, double* ms) {
  if (!h || !ms) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  int st = ensure_selinv(h);
  if (st) return st;
  RGF_CK(cudaMemcpy(ms, h->d_MS, sizeof(double) * h->mf_size, cudaMemcpyDeviceToHost));
  return RGF_OK;
}

int rgf_get_info(rgf_handle* h, rgf_info_t* info) {
  if (!h || !info) return RGF_EINVAL;
  std::memset(info, 0, sizeof(*info));
  info->n = (size_t)h->sh.n;
  info->nnz = (size_t)h->nnz;
  info->mf_size = (size_t)h->mf_size;
  info->device_bytes = h->device_bytes;
  info->not_spd_column = h->not_spd_col;
  info->kernels_launched = h->kernels_total;
  return RGF_OK;
}

int rgf_get_stream(rgf_handle* h, void** stream) {
  if (!h || !stream) return RGF_EINVAL;
  *stream = (void*)h->stream;
  return RGF_OK;
}

int rgf_kernel_timer_enable(rgf_handle* h, int enable) {
  if (!h) return RGF_EINVAL;
  h->timer_on = enable != 0;
  h->timer_detail_on = enable > 1;
  return RGF_OK;
}

int rgf_kernel_timer_read(rgf_handle* h, int reset, int kind, double* ms, long long* launches,
                          double* flops) {
  if (!h || kind < 0 || kind > 3) return RGF_EINVAL;
  const int k = kind == 3 ? 2 : kind;
  if (ms) *ms = h->timer_ms[k];
  if (launches) *launches = h->timer_launches[k];
  if (flops) *flops = kind == 3 ? h->timer_tflops : h->timer_flops[k];
  if (reset && h->timer_detail_on && !h->timer_detail.empty()) {
    std::vector<std::pair<double, std::string>> rows;
    for (auto& kv : h->timer_detail) {
      char line[200];
      std::snprintf(line, sizeof(line), "%s  x%6lld  %9.3f ms", kv.first.c_str(), kv.second.first,
                    kv.second.second);
      rows.push_back({kv.second.second, line});
    }
    std::sort(rows.rbegin(), rows.rend());
    std::fprintf(stderr, "[rgf timer] per GEMM shape (top 40)\n");
    for (size_t i = 0; i < rows.size() && i < 40; ++i) std::fprintf(stderr, "  %s\n", rows[i].second.c_str());
    h->timer_detail.clear();
  }
  if (reset) {
    for (int i = 0; i < 3; ++i) {
      h->timer_ms[i] = 0.0;
      h->timer_flops[i] = 0.0;
      h->timer_launches[i] = 0;
    }
    h->timer_tflops = 0.0;
  }
  return RGF_OK;
}

int rgf_dgemm_device(int precision, int slices, char transa, char transb, int m, int n, int k,
                     double alpha, const double* A, int lda, const double* B, int ldb,
                     double beta, double* C, int ldc, void* stream) {
  if (m < 0 || n < 0 || k < 0 || !C || (k > 0 && (!A || !B))) return RGF_EINVAL;
  if (precision != RGF_PREC_FP64 && precision != RGF_PREC_SPLIT) return RGF_EINVAL;
  if (slices < 0 || slices > 8) return RGF_EINVAL;
  const bool ta = transa == 'T' || transa == 't', tb = transb == 'T' || transb == 't';
  if (lda < std::max(1, ta ? k : m) || ldb < std::max(1, tb ? n : k) || ldc < std::max(1, m))
    return RGF_EINVAL;
  if (m == 0 || n == 0) return RGF_OK;
  GemmDesc g;
  g.m = m; g.n = n; g.k = k;
  g.A = A; g.lda = lda; g.transA = ta;
  g.B = B; g.ldb = ldb; g.transB = tb;
  g.C = C; g.ldc = ldc; g.D = C; g.ldd = ldc;
  g.alpha = alpha; g.beta = beta;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DevStatus* st = nullptr;
  RGF_CK(cudaMalloc(&st, sizeof(DevStatus)));
  RGF_CK(cudaMemsetAsync(st, 0, sizeof(DevStatus), s));
  int status = RGF_OK;
  SplitEngine* eng = nullptr;
  if (precision == RGF_PREC_SPLIT) {
    eng = SplitEngine::create(slices, &status);
    if (!status) status = eng->prepare(std::max(m, n), k, 1, s);
  }
  if (!status) {
    if (eng && eng->supports(g)) eng->gemm(g, s, st);
    else launch_gemm_fp64(g, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) status = cuda_status(e);
  }
  if (!status) {
    DevStatus hs;
    if (cudaMemcpy(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost) != cudaSuccess) status = RGF_ECUDA;
    else if (hs.timeout) status = RGF_ETIMEOUT;
  }
  delete eng;
  cudaFree(st);
  return status;
}

int rgf_set_device_cache(size_t max_bytes) {
  std::lock_guard<std::mutex> lk(rgf::g_cache.mu);
  rgf::g_cache.limit = max_bytes;
  rgf::cache_trim(max_bytes, -1);
  return RGF_OK;
}

int rgf_device_cache_bytes(size_t* held) {
  if (!held) return RGF_EINVAL;
  std::lock_guard<std::mutex> lk(rgf::g_cache.mu);
  *held = rgf::g_cache.held;
  return RGF_OK;
}

int rgf_debug_fail_alloc_after(long long after) {
  rgf::g_fail_alloc_after.store(after < 0 ? -1 : after);
  return RGF_OK;
}

int rgf_set_wait_limit(rgf_handle* h, int polls) {
  if (!h || polls < 0) return RGF_EINVAL;
  if (polls == h->leaf_wait_polls) return RGF_OK;
  const int st = drop_graphs(h);  // the limit is a kernel argument of the captured stages
  if (st) return st;
  h->leaf_wait_polls = polls;
  return RGF_OK;
}

int rgf_measure_fp64_peak(double* tflops) {
  if (!tflops) return RGF_EINVAL;
  return measure_fp64_peak(tflops);
}

}  // extern "C"

// ============================================================================
// Batches of independent instances (many factorizations of uneven (ns, nt, nd)
// as in a hyper-parameter search).  Every instance keeps its own handle,
// stream and workspaces; the whole batch's factorize + selected inversion is
// captured once as ONE CUDA graph whose branches (one per instance) run
// concurrently, and replayed with a single graph launch.
// ============================================================================
struct rgf_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<rgf_handle*> h;
  std::vector<cudaEvent_t> ev;
  cudaGraphExec_t g_all = nullptr;
  long long k_all = 0;
  long long kernels_total = 0;
  int runs = 0;  // graph-mode runs so far (the first one is not captured)
  long long knob_sum = 0;  // sum of the instances' knob_gen when g_all was captured
};

namespace {
long long batch_knob_sum(const rgf_batch* b) {
  long long s = 0;
  for (const rgf_handle* h : b->h) s += h->knob_gen;
  return s;
}
}  // namespace

namespace {

void batch_release(rgf_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->g_all) cudaGraphExecDestroy(b->g_all);
  for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
  for (rgf_handle* h : b->h) release(h);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// Every instance's factorize + selected inversion, each on its own streams,
// forked from and joined back into the batch stream.  capture = true records
// it as one CUDA graph (b->g_all); otherwise the kernels are launched directly
// (the first run: a batch used once never pays for capturing and
// instantiating a graph of hundreds of thousands of nodes).
int batch_issue(rgf_batch* b, bool capture) {
  for (rgf_handle* h : b->h) {
    int st = alloc_selinv(h);
    if (st) return st;
  }
  RGF_CK(cudaStreamSynchronize(b->stream));
  for (rgf_handle* h : b->h) RGF_CK(cudaStreamSynchronize(h->stream));
  const size_t n = b->h.size();
  if (b->ev.empty()) {
    b->ev.resize(n + 1);
    for (auto& e : b->ev) RGF_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  cudaGraph_t graph = nullptr;
  if (capture) RGF_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaEventRecord(b->ev[0], b->stream);
  long long nk = 0;
  for (size_t i = 0; i < n; ++i) {
    rgf_handle* h = b->h[i];
    cudaStreamWaitEvent(h->stream, b->ev[0], 0);
    h->kernels_issued = 0;
    issue_factor(h);
    issue_selinv(h);
    nk += h->kernels_issued;
    cudaEventRecord(b->ev[i + 1], h->stream);
    cudaStreamWaitEvent(b->stream, b->ev[i + 1], 0);
  }
  if (!capture) {
    b->kernels_total += nk;
    RGF_CK(cudaGetLastError());
    return RGF_OK;
  }
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaGraphInstantiate(&b->g_all, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->g_all = nullptr;
    return cuda_status(e);
  }
  b->k_all = nk;
  b->knob_sum = batch_knob_sum(b);
  return RGF_OK;
}

}  // namespace

extern "C" {

int rgf_batch_create(size_t count, const size_t* const* ia, const size_t* const* ja,
                     const double* const* a, const size_t* ns, const size_t* nt, const size_t* nd,
                     const rgf_opts* opts, rgf_batch** out) {
  if (!out || count == 0 || !ia || !ja || !a || !ns || !nt || !nd) return RGF_EINVAL;
  *out = nullptr;
  rgf_batch* b = new (std::nothrow) rgf_batch();
  if (!b) return RGF_ENOMEM;
  rgf_opts o;
  rgf_default_opts(&o);
  if (opts) o = *opts;
  o.async_upload = 0;  // a batch graph is captured over all instances: upload now
  int st = RGF_OK;
  for (size_t i = 0; i < count && !st; ++i) {
    rgf_handle* h = nullptr;
    st = rgf_create(ia[i], ja[i], a[i], ns[i], nt[i], nd[i], &o, &h);
    if (!st) b->h.push_back(h);
  }
  if (!st) {
    b->device = b->h[0]->device;
    cudaSetDevice(b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) st = RGF_ECUDA;
  }
  if (st) {
    batch_release(b);
    return st;
  }
  *out = b;
  return RGF_OK;
}

int rgf_batch_destroy(rgf_batch* b) {
  if (!b) return RGF_EINVAL;
  batch_release(b);
  return RGF_OK;
}

int rgf_batch_size(rgf_batch* b, size_t* count) {
  if (!b || !count) return RGF_EINVAL;
  *count = b->h.size();
  return RGF_OK;
}

int rgf_batch_handle(rgf_batch* b, size_t i, rgf_handle** h) {
  if (!b || !h || i >= b->h.size()) return RGF_EINVAL;
  *h = b->h[i];
  return RGF_OK;
}

int rgf_batch_get_stream(rgf_batch* b, void** stream) {
  if (!b || !stream) return RGF_EINVAL;
  *stream = (void*)b->stream;
  return RGF_OK;
}

int rgf_batch_run(rgf_batch* b, int mode, double* logdet, double* const* diag) {
  if (!b || (mode != 0 && mode != 1)) return RGF_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess) return RGF_ECUDA;
  int st = RGF_OK;
  if (mode == 0) {
    if (b->g_all && b->knob_sum != batch_knob_sum(b)) {
      // an instance's knobs changed since the capture: launch directly once,
      // then capture again
      RGF_CK(cudaStreamSynchronize(b->stream));
      cudaGraphExecDestroy(b->g_all);
      b->g_all = nullptr;
      b->runs = 0;
    }
    if (b->runs++ == 0) {
      if ((st = batch_issue(b, false))) return st;
    } else {
      if (!b->g_all && (st = batch_issue(b, true))) return st;
      RGF_CK(cudaGraphLaunch(b->g_all, b->stream));
      b->kernels_total += b->k_all;
    }
    RGF_CK(cudaStreamSynchronize(b->stream));
    for (rgf_handle* h : b->h) {
      h->factored = false;
      h->selinv_done = false;
      if ((st = sync_and_check(h))) return st;
      h->factored = true;
      h->selinv_done = true;
      h->inv_done = true;
    }
  } else {
    for (rgf_handle* h : b->h) {
      const long long k0 = h->kernels_total;
      if ((st = rgf_factorize(h))) return st;
      if ((st = ensure_selinv(h))) return st;
      b->kernels_total += h->kernels_total - k0;
    }
  }
  for (size_t i = 0; i < b->h.size(); ++i) {
    rgf_handle* h = b->h[i];
    if (logdet) RGF_CK(cudaMemcpy(&logdet[i], h->d_scalars, sizeof(double), cudaMemcpyDeviceToHost));
    if (diag && diag[i])
      RGF_CK(cudaMemcpy(diag[i], h->d_diag, sizeof(double) * h->sh.n, cudaMemcpyDeviceToHost));
  }
  return RGF_OK;
}

int rgf_batch_kernels(rgf_batch* b, long long* kernels) {
  if (!b || !kernels) return RGF_EINVAL;
  *kernels = b->kernels_total;
  return RGF_OK;
}

}  // extern "C"

// ============================================================================
// Tuning knobs and the autotuner.  The knobs change how the factorization and
// selected inversion are cut into kernels (leaf width, look-ahead stream,
// split/FP64 routing), never the operation count; the autotuner measures the
// candidates on the instance itself and caches the choice per class.
// ============================================================================
namespace {

bool valid_tuning(const rgf_tuning& t) {
  return (t.leaf_nb == 16 || t.leaf_nb == 32 || t.leaf_nb == 64) &&
         (t.lookahead == 0 || t.lookahead == 1) && std::isfinite(t.split_bias) &&
         t.split_bias >= 1.0 / 16 && t.split_bias <= 16.0 &&
         (t.splitk_max == 0 || t.splitk_max == 1 || t.splitk_max == 2 || t.splitk_max == 4 ||
          t.splitk_max == 8 || t.splitk_max == 16) &&
         (t.fp64_tile == 0 || t.fp64_tile == 32 || t.fp64_tile == 64);
}

rgf_tuning knobs_of(const rgf_handle* h) {
  rgf_tuning t{};
  t.leaf_nb = h->nb;
  t.lookahead = h->lookahead ? 1 : 0;
  t.split_bias = h->split_bias;
  t.splitk_max = h->splitk_max;
  t.fp64_tile = h->fp64_tile;
  t.ms = h->tuned_ms;
  return t;
}

int set_knobs(rgf_handle* h, const rgf_tuning& t) {
  const int st = drop_graphs(h);
  if (st) return st;
  h->nb = t.leaf_nb;
  h->lookahead = t.lookahead != 0;
  h->split_bias = t.split_bias;
  h->splitk_max = t.splitk_max;
  h->fp64_tile = t.fp64_tile;
  for (SplitEngine* e : {h->split, h->split_side})
    if (e) e->set_splitk_max(t.splitk_max);
  h->tuned_ms = t.ms;
  h->knob_gen++;
  return RGF_OK;
}

// Wall time of one factorize + selected inversion under the handle's current
// knobs as a steady-state caller sees it: one direct run and one run that
// captures the stage graphs (both untimed), then the best of `reps` graph
// replays.  Every stage ends with a synchronisation, so the host clock
// brackets the device work.
int time_factor_selinv(rgf_handle* h, int reps, double* ms) {
  double best = 1e300;
  for (int r = 0; r < 2 + reps; ++r) {
    h->factored = false;
    const auto t0 = std::chrono::steady_clock::now();
    const int st = ensure_selinv(h);
    if (st) return st;
    const double t =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (r >= 2) best = std::min(best, t);
  }
  *ms = best;
  return RGF_OK;
}

// Coordinate descent from the current knobs: leaf width, then look-ahead,
// then (split precision) the routing bias.  A candidate replaces the best so
// far only when it is at least 2% faster, so timing noise does not move the
// choice away from the defaults.
int tune_handle(rgf_handle* h, rgf_tuning* out) {
  rgf_tuning best = knobs_of(h);
  int st = set_knobs(h, best);
  if (st) return st;
  if ((st = time_factor_selinv(h, 2, &best.ms))) return st;
  auto trial = [&](rgf_tuning t) -> int {
    if (t.leaf_nb == best.leaf_nb && t.lookahead == best.lookahead &&
        t.split_bias == best.split_bias && t.splitk_max == best.splitk_max &&
        t.fp64_tile == best.fp64_tile)
      return RGF_OK;
    int e = set_knobs(h, t);
    if (e) return e;
    if ((e = time_factor_selinv(h, 2, &t.ms))) return e;
    if (t.ms < 0.98 * best.ms) best = t;
    return RGF_OK;
  };
  for (int nb : {16, 32, 64}) {
    rgf_tuning t = best;
    t.leaf_nb = nb;
    if ((st = trial(t))) return st;
  }
  {
    rgf_tuning t = best;
    t.lookahead = !best.lookahead;
    if ((st = trial(t))) return st;
  }
  if (h->split) {
    for (double bias : {0.5, 2.0}) {
      rgf_tuning t = best;
      t.split_bias = bias;
      if ((st = trial(t))) return st;
    }
    for (int k : {1, 4}) {  // tile shapes: split-K degree of the tensor-core products
      rgf_tuning t = best;
      t.splitk_max = k;
      if ((st = trial(t))) return st;
    }
  }
  for (int tile : {0, 32, 64}) {  // and the FP64 products' output tile
    rgf_tuning t = best;
    t.fp64_tile = tile;
    if ((st = trial(t))) return st;
  }
  if ((st = set_knobs(h, best))) return st;
  *out = best;
  return RGF_OK;
}

// Process-wide choices, keyed by everything that changes what is timed.
struct TuneKey {
  int device;
  long long ns, nd;
  int precision, slices, fp64_diag, selinv_mode, use_graphs;
  bool operator<(const TuneKey& o) const {
    return std::tie(device, ns, nd, precision, slices, fp64_diag, selinv_mode, use_graphs) <
           std::tie(o.device, o.ns, o.nd, o.precision, o.slices, o.fp64_diag, o.selinv_mode,
                    o.use_graphs);
  }
};
std::mutex g_tune_mu;
std::map<TuneKey, rgf_tuning> g_tune_cache;

TuneKey tune_key(const rgf_handle* h) {
  const rgf_opts& o = h->opts;
  return {h->device, h->sh.ns, h->sh.nd, o.precision, o.slices, o.fp64_diag, o.selinv_mode,
          o.use_graphs};
}

}  // namespace

extern "C" {

int rgf_get_tuning(rgf_handle* h, rgf_tuning* t) {
  if (!h || !t) return RGF_EINVAL;
  *t = knobs_of(h);
  return RGF_OK;
}

int rgf_set_tuning(rgf_handle* h, const rgf_tuning* t) {
  if (!h || !t || !valid_tuning(*t)) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  rgf_tuning k = *t;
  k.ms = 0.0;
  return set_knobs(h, k);
}

int rgf_autotune(rgf_handle* h, int flags, rgf_tuning* chosen) {
  if (!h || (flags & ~RGF_TUNE_FORCE) || h->timer_on) return RGF_EINVAL;
  if (cudaSetDevice(h->device) != cudaSuccess) return RGF_ECUDA;
  const TuneKey key = tune_key(h);
  rgf_tuning t{};
  bool cached = false;
  if (!(flags & RGF_TUNE_FORCE)) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      t = it->second;
      cached = true;
    }
  }
  int st;
  if (cached) {
    st = set_knobs(h, t);
  } else {
    const rgf_tuning orig = knobs_of(h);
    st = tune_handle(h, &t);
    if (st) {
      set_knobs(h, orig);  // a failed run leaves the knobs as they were
      return st;
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = t;
  }
  if (st) return st;
  if (chosen) *chosen = t;
  return RGF_OK;
}

int rgf_batch_autotune(rgf_batch* b, int flags, size_t* classes) {
  if (!b || (flags & ~RGF_TUNE_FORCE)) return RGF_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess) return RGF_ECUDA;
  RGF_CK(cudaStreamSynchronize(b->stream));
  std::map<std::pair<long long, long long>, std::vector<size_t>> groups;
  for (size_t i = 0; i < b->h.size(); ++i) groups[{b->h[i]->sh.ns, b->h[i]->sh.nd}].push_back(i);
  for (auto& kv : groups) {
    std::vector<size_t> idx = kv.second;
    std::stable_sort(idx.begin(), idx.end(),
                     [&](size_t x, size_t y) { return b->h[x]->sh.nt < b->h[y]->sh.nt; });
    rgf_handle* rep = b->h[idx[idx.size() / 2]];
    rgf_tuning t{};
    int st = rgf_autotune(rep, flags, &t);
    if (st) return st;
    for (size_t i : idx)
      if (b->h[i] != rep && (st = set_knobs(b->h[i], t))) return st;
  }
  if (b->g_all) {
    cudaGraphExecDestroy(b->g_all);
    b->g_all = nullptr;
  }
  b->runs = 0;
  if (classes) *classes = groups.size();
  return RGF_OK;
}

}  // extern "C"
