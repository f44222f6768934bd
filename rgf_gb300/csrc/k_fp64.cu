// FP64 kernels of the RGF recursion for sm_103a.
//
// On GB300 the FP64 rate is the same for DMMA (mma.sync .f64) and DFMA
// (about 1 TFLOP/s per GPU), so the FP64 GEMM below is bound by the FP64
// pipe, not by memory: 64x64 output tiles, 4 warps of 32x32 built from
// m8n8k4 DMMA fragments, operands staged through shared memory with a
// register prefetch of the next K slice.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>

#include "rgf_internal.h"

namespace rgf {

namespace {

__device__ __forceinline__ void dmma_8x8x4(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

struct GemmTileRange {
  int klo, khi;
};

template <int TM, int TK>
__device__ __forceinline__ GemmTileRange k_range(const GemmDesc& g, int m0, int n0) {
  int klo = 0, khi = g.k;
  if (g.triA == TRI_LOWER) khi = min(khi, m0 + TM);
  if (g.triA == TRI_UPPER) klo = max(klo, m0);
  if (g.triB == TRI_LOWER) klo = max(klo, n0);
  if (g.triB == TRI_UPPER) khi = min(khi, n0 + TM);
  klo = (klo / TK) * TK;
  return {klo, khi};
}

// TM x TM output tiles, 4 warps of (TM/2) x (TM/2) built from m8n8k4 DMMA
// fragments, K staged TK at a time.  TM = 64, TK = 16 for large products;
// TM = 32, TK = 8 spreads small products over four times as many CTAs (each
// SM retires only ~3.5 FP64 flops per cycle, so a small product on few SMs
// is slow however short it is).
template <int TM, int TK>
__global__ void __launch_bounds__(128) gemm_fp64_kernel(GemmDesc g) {
  constexpr int F = TM / 16;             // 8 x 8 fragments per warp side
  constexpr int LPT = TM * TK / 128;     // elements per thread per operand and stage
  constexpr int PAD = TM + 4;
  pdl_wait();
  const int m0 = blockIdx.x * TM;
  const int n0 = blockIdx.y * TM;
  if (g.outLower && m0 + TM <= n0) return;  // tile entirely above the diagonal
  const bool splitk = g.ksplit > 1;              // blockIdx.z is the K slice, batch == 1
  const long long bz = splitk ? 0 : blockIdx.z;
  const double* __restrict__ A = g.A + bz * g.sA;
  const double* A2 = g.A2 ? g.A2 + bz * g.sA - g.mA1 : nullptr;
  const int mA1 = g.A2 ? g.mA1 : g.m;
  const double* __restrict__ B = g.B + bz * g.sB;
  const double* C = g.C ? g.C + bz * g.sC : nullptr;
  double* D = g.D + bz * g.sD;
  const double* C2 = g.C2 ? g.C2 + bz * g.sC - g.mD1 : nullptr;
  double* D2 = g.D2 ? g.D2 + bz * g.sD - g.mD1 : nullptr;
  const int mD1 = g.D2 ? g.mD1 : g.m;

  __shared__ double As[TK][PAD];
  __shared__ double Bs[TK][PAD];

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * (TM / 2), wn = (warp >> 1) * (TM / 2);
  GemmTileRange kr = k_range<TM, TK>(g, m0, n0);
  if (splitk) {
    const int len = max(0, kr.khi - kr.klo);
    const int chunk = ((len + g.ksplit - 1) / g.ksplit + TK - 1) / TK * TK;
    const int lo = kr.klo + (int)blockIdx.z * chunk;
    kr.khi = min(kr.khi, lo + chunk);
    kr.klo = lo;
  }

  double acc[F][F][2];
#pragma unroll
  for (int i = 0; i < F; ++i)
#pragma unroll
    for (int j = 0; j < F; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  double ra[LPT], rb[LPT];
  auto load = [&](int kt) {
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
      int rr, kk;
      if (!g.transA) { rr = tid % TM; kk = tid / TM + (128 / TM) * j; }
      else           { kk = tid % TK; rr = tid / TK + (128 / TK) * j; }
      const int r = m0 + rr, kg = kt + kk;
      bool ok = r < g.m && kg < kr.khi;
      if (g.triA == TRI_LOWER) ok = ok && kg <= r;
      if (g.triA == TRI_UPPER) ok = ok && kg >= r;
      double v = 0.0;
      if (ok) v = g.transA ? A[(long long)kg + (long long)r * g.lda]
                           : (r < mA1 ? A : A2)[(long long)r + (long long)kg * g.lda];
      ra[j] = v;
    }
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
      int cc, kk;
      if (!g.transB) { kk = tid % TK; cc = tid / TK + (128 / TK) * j; }
      else           { cc = tid % TM; kk = tid / TM + (128 / TM) * j; }
      const int c = n0 + cc, kg = kt + kk;
      bool ok = c < g.n && kg < kr.khi;
      if (g.triB == TRI_LOWER) ok = ok && kg >= c;
      if (g.triB == TRI_UPPER) ok = ok && kg <= c;
      double v = 0.0;
      if (ok) v = g.transB ? B[(long long)c + (long long)kg * g.ldb] : B[(long long)kg + (long long)c * g.ldb];
      rb[j] = v;
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int j = 0; j < LPT; ++j) {
      if (!g.transA) As[tid / TM + (128 / TM) * j][tid % TM] = ra[j];
      else           As[tid % TK][tid / TK + (128 / TK) * j] = ra[j];
      if (!g.transB) Bs[tid % TK][tid / TK + (128 / TK) * j] = rb[j];
      else           Bs[tid / TM + (128 / TM) * j][tid % TM] = rb[j];
    }
  };

  if (kr.klo < kr.khi) {
    load(kr.klo);
    for (int kt = kr.klo; kt < kr.khi; kt += TK) {
      store();
      __syncthreads();
      if (kt + TK < kr.khi) load(kt + TK);
#pragma unroll
      for (int ks = 0; ks < TK; ks += 4) {
        if (kt + ks >= kr.khi) break;  // a short last K tile: no products of the zero padding
        double af[F], bf[F];
#pragma unroll
        for (int i = 0; i < F; ++i) af[i] = As[ks + (lane & 3)][wm + i * 8 + (lane >> 2)];
#pragma unroll
        for (int j = 0; j < F; ++j) bf[j] = Bs[ks + (lane & 3)][wn + j * 8 + (lane >> 2)];
#pragma unroll
        for (int i = 0; i < F; ++i)
#pragma unroll
          for (int j = 0; j < F; ++j) dmma_8x8x4(acc[i][j], af[i], bf[j]);
      }
      __syncthreads();
    }
  }
  pdl_trigger();

  if (splitk) {  // raw partial sums of this K slice; reduced in fixed order later
    double* W = g.ws + (long long)blockIdx.z * g.m * g.n;
#pragma unroll
    for (int i = 0; i < F; ++i) {
      const int r = m0 + wm + i * 8 + (lane >> 2);
#pragma unroll
      for (int j = 0; j < F; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int c = n0 + wn + j * 8 + (lane & 3) * 2 + e;
          if (r < g.m && c < g.n) W[(long long)r + (long long)c * g.m] = acc[i][j][e];
        }
    }
    return;
  }
#pragma unroll
  for (int i = 0; i < F; ++i) {
    const int r = m0 + wm + i * 8 + (lane >> 2);
    if (r >= g.m) continue;
    const double* Cr = r < mD1 ? C : C2;
    double* Dr = r < mD1 ? D : D2;
#pragma unroll
    for (int j = 0; j < F; ++j) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int c = n0 + wn + j * 8 + (lane & 3) * 2 + e;
        if (c >= g.n) continue;
        if (g.outLower && r < c) continue;
        double v = g.alpha * acc[i][j][e];
        if (g.beta != 0.0) v += g.beta * Cr[(long long)r + (long long)c * g.ldc];
        Dr[(long long)r + (long long)c * g.ldd] = v;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Leaf Cholesky of one <= 64 x 64 diagonal tile in shared memory.
// On GB300 each SM sub-partition has its own FP64 unit; one FP64 warp
// instruction occupies it ~76 cycles whatever the number of active lanes, and
// a dependent FP64 op waits ~63 (measured), so the column-to-column pivot
// chain (the next pivot's update, its reciprocal square root, the column's
// scaling) is the critical path.  The log-determinant is summed later from
// the factor's diagonal, off this path.
// ---------------------------------------------------------------------------
// float -> double by bit manipulation (no FP64 conversion instruction);
// zero and subnormal floats give zero
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int ex = (u >> 23) & 0xffu;
  if (ex == 0) return 0.0;
  return __longlong_as_double((long long)((unsigned long long)(u >> 31) << 63 |
                                          (unsigned long long)(ex - 127 + 1023) << 52 |
                                          (unsigned long long)(u & 0x7fffffu) << 29));
}

// Reciprocal square root of a normal positive double with few dependent FP64
// operations (they are the slow link of the leaf's pivot chain): d = m 4^k
// with m in [1, 4) by integer ops; an FP32 seed y0 = rsqrt(m_hi) is refined
// once in double-float arithmetic on the FP32 units (m = m_hi + m_lo split
// exactly from the bit pattern; e = 1 - m y0^2 with FMA-exact products), which
// gives ~44 bits; one FP64 Newton step then gives full precision.  FP64 ops on
// the chain: one add, one multiply, two FMAs; the 4^-k scale is an exponent
// shift.
__device__ __forceinline__ double rsqrt_fast(double d) {
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e == -1023) return 1.0 / sqrt(d);                   // subnormal pivot
  const int k = e >> 1;                                   // d = m * 4^k, m in [1, 4)
  const long long mb = b - ((long long)(2 * k) << 52);
  const double m = __longlong_as_double(mb);
  const int em = (int)((mb >> 52) & 0x7ff) - 1023;        // 0 or 1
  // m_hi: the top 24 significant bits as a float; m_lo: the remaining 29 bits
  const float mh = __uint_as_float((unsigned int)(((mb >> 52) - 1023 + 127) << 23) |
                                   (unsigned int)((mb >> 29) & 0x7fffff));
  const float ml = (float)(unsigned int)(mb & ((1ll << 29) - 1)) *
                   __uint_as_float((unsigned int)(127 + em - 52) << 23);
  const float y0 = rsqrtf(mh);
  const float p = y0 * y0;
  const float pe = fmaf(y0, y0, -p);                      // y0^2 = p + pe exactly
  float t = fmaf(-mh, p, 1.0f);
  t = fmaf(-mh, pe, t);
  t = fmaf(-ml, p, t);                                    // e = 1 - m y0^2
  const double y1 = f2d_bits(y0) + f2d_bits(0.5f * y0 * t);
  const double hm = __longlong_as_double(mb - (1ll << 52));  // m / 2, exact
  const double y2 = fma(y1, fma(-hm, y1 * y1, 0.5), y1);    // y1 (1.5 - m y1^2 / 2)
  return __longlong_as_double(__double_as_longlong(y2) - ((long long)k << 52));
}


// ---------------------------------------------------------------------------
// Leaf Cholesky, data-flow form: warps hand columns to each other through
// release/acquire on a shared-memory counter (no CTA-wide barrier per
// column); see leaf_chol below.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void st_release_cta(int* p, int v) {
  asm volatile("st.release.cta.shared::cta.b32 [%0], %1;"
               :: "r"((unsigned)__cvta_generic_to_shared(p)), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_cta(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];"
               : "=r"(v) : "r"((unsigned)__cvta_generic_to_shared(p)) : "memory");
  return v;
}

// The leaf Cholesky proper, on the tile held in shared memory S (lower part).
// Column c belongs to warp c % 8.  Step j applies the final column j of L to
// every later column (one FMA per column and 32 rows: L_cj is a broadcast
// read); the owner of column j + 1 does that column first, then takes its
// pivot d from shared memory in every lane (rsqrt on all lanes costs the same
// warp instruction as on one), scales the column to its final value
// (L_rc = S_rc d^{-1/2}, L_cc = d d^{-1/2}) and publishes it with a release
// store.  FP64 ops on the pivot chain per column: FMA, the four of rsqrt_fast,
// one multiply.  Columns are written only by their owner; column j is
// read-only once published.  Waits are bounded by wait_polls polls, after
// which the leaf records a timeout and stops.
__device__ __forceinline__ void leaf_finalize(double (*S)[65], int nbk, int c, int lane,
                                              int* ready, int* fail) {
  __syncwarp();
  const double d = S[c][c];
  const bool ok = d > 0.0;
  const double y = ok ? rsqrt_fast(d) : __longlong_as_double(0x7ff8000000000000LL);
  for (int r = c + lane; r < nbk; r += 32) S[r][c] = (r == c ? d : S[r][c]) * y;
  if (!ok && lane == 0) atomicMin(fail, c);
  __syncwarp();
  if (lane == 0) st_release_cta(ready, c);
}

__device__ void leaf_chol(double (*S)[65], int nbk, DevStatus* st, int wait_polls, int* ready,
                          int* abort_, int* fail) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) leaf_finalize(S, nbk, 0, lane, ready, fail);
  for (int j = 0; j + 1 < nbk; ++j) {
    if (ld_acquire_cta(ready) < j) {
      int it = 0;
      while (ld_acquire_cta(ready) < j && !*(volatile int*)abort_ && ++it < wait_polls) {
      }
      if (it >= wait_polls) {
        *(volatile int*)abort_ = 1;
        if (lane == 0) atomicExch(&st->timeout, 1);
      }
      if (*(volatile int*)abort_) break;
    }
    int c = j + 1 + ((warp - (j + 1)) % 8 + 8) % 8;  // first owned column > j
    for (; c < nbk; c += 8) {
      const double lcj = S[c][j];
      for (int r = c + lane; r < nbk; r += 32) S[r][c] = fma(-S[r][j], lcj, S[r][c]);
      if (c == j + 1) leaf_finalize(S, nbk, c, lane, ready, fail);
    }
  }
}

// Row-parallel solve X := X L^{-T} (MODE 0) or X := X L^{-1} (MODE 1) of the
// rows [r0, r0 + nthreads/8) of X against the nbk x nbk lower tile in Ls.
// Eight lanes share one row: lane q of the group keeps the unknowns
// l = q, q + 8, ... in registers.  Step j: the owner of x_j scales it, one
// shuffle hands it to the other seven lanes, and each applies it to its own
// unknowns -- no CTA barrier per column, so the column-to-column chain is a
// multiply, a shuffle and a fused multiply-add.
// MODE 0: x_j = (b_j - sum_{l<j} x_l L_jl) / L_jj   (X L^T = B)
// MODE 1: x_j = (b_j - sum_{l>j} x_l L_lj) / L_jj   (X L = B)
template <int MODE>
__device__ __forceinline__ void trsm_rows_body(double* X, long long xrs, long long xcs, int rows,
                                               double (*Ls)[65], const double* rinv, int nbk,
                                               long long r0) {
  const int lane = threadIdx.x & 31, q = lane & 7, gbase = lane & ~7;
  const long long r = r0 + (threadIdx.x >> 3);
  const bool live = r < rows;
  double u[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const int l = t * 8 + q;
    u[t] = (live && l < nbk) ? X[r * xrs + (long long)l * xcs] : 0.0;
  }
  for (int s = 0; s < nbk; ++s) {
    const int j = MODE == 0 ? s : nbk - 1 - s;
    const int jt = j >> 3;
    double uj = 0.0;
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (t == jt) uj = u[t];
    const double xj = __shfl_sync(0xffffffffu, uj * rinv[j], gbase | (j & 7));
    // slots that can hold a live unknown: a warp-uniform range, so FP64
    // instructions with no live lane are not issued
    const int tlo = MODE == 0 ? jt : 0, thi = MODE == 0 ? (nbk - 1) >> 3 : jt;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      if (t < tlo || t > thi) continue;
      const int l = t * 8 + q;
      if (l == j) u[t] = xj;
      if (MODE == 0 ? (l > j && l < nbk) : (l < j)) u[t] = fma(-xj, MODE == 0 ? Ls[l][j] : Ls[j][l], u[t]);
    }
  }
  pdl_trigger();
  if (live) {
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int l = t * 8 + q;
      if (l < nbk) X[r * xrs + (long long)l * xcs] = u[t];
    }
  }
}

// Leaf Cholesky of the nbk x nbk lower tile T in one CTA (leaf_chol).  The
// rows below the leaf are solved by a separate trsm_rows launch: folding that
// solve into this launch (CTAs that wait for the leaf) was measured slower at
// ns=2000, as the waiting CTAs hold SMs that the concurrent side-stream
// products need.
__global__ void __launch_bounds__(256) leaf_potrf_kernel(double* T, long long ldt, int nbk,
                                                         int col0, DevStatus* st, int wait_polls) {
  __shared__ double S[64][65];
  __shared__ int ready, abort_, fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  pdl_wait();
  for (int c = warp; c < nbk; c += 8)
    for (int r = c + lane; r < nbk; r += 32) S[r][c] = T[(long long)r + (long long)c * ldt];
  if (tid == 0) {
    fail = 0x7fffffff;
    abort_ = 0;
    ready = -1;
  }
  __syncthreads();
  leaf_chol(S, nbk, st, wait_polls, &ready, &abort_, &fail);
  __syncthreads();
  pdl_trigger();
  for (int c = warp; c < nbk; c += 8)
    for (int r = c + lane; r < nbk; r += 32) T[(long long)r + (long long)c * ldt] = S[r][c];
  if (tid == 0 && fail != 0x7fffffff) atomicMin(&st->not_spd_col, col0 + fail);
}

// Row-parallel triangular solve with a <= 64 x 64 lower tile (trsm_rows_body):
// a warp holds four rows and a CTA of 4 warps 16 rows, so the FP64 work
// spreads over many SMs (each SM retires only ~3.5 FP64 flops per cycle).
template <int MODE>
__global__ void __launch_bounds__(128) trsm_rows_kernel(double* X, long long xrs, long long xcs,
                                                         int rows, const double* L, long long ldl,
                                                         int nbk, long long sX, long long sL) {
  __shared__ double Ls[64][65];
  __shared__ double rinv[64];
  pdl_wait();
  X += (long long)blockIdx.y * sX;
  L += (long long)blockIdx.y * sL;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 128) {
    const int c = idx >> 6, r = idx & 63;
    double v = 0.0;
    if (r < nbk && c < nbk && r >= c) v = L[(long long)r + (long long)c * ldl];
    Ls[r][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 64) rinv[threadIdx.x] = (threadIdx.x < nbk) ? 1.0 / Ls[threadIdx.x][threadIdx.x] : 0.0;
  __syncthreads();
  trsm_rows_body<MODE>(X, xrs, xcs, rows, Ls, rinv, nbk, (long long)blockIdx.x * 16);
}

// Thin products (m <= 16, op(B) = B^T): lane = output column, the 4 warps of
// a CTA split a K chunk, blockIdx.y selects the chunk.  Partial sums go to
// the split-K workspace in the GEMM kernel's layout.
__global__ void __launch_bounds__(128) gemm_thin_m_kernel(GemmDesc g, int kchunk) {
  __shared__ double red[4][16][33];
  pdl_wait();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + lane;
  const int k0 = blockIdx.y * kchunk, k1 = min(g.k, k0 + kchunk);
  double acc[16];
#pragma unroll
  for (int r = 0; r < 16; ++r) acc[r] = 0.0;
  if (c < g.n) {
    for (int k = k0 + w; k < k1; k += 4) {
      if (g.triB == TRI_LOWER && k < c) continue;   // op(B)(k, c) = 0 above
      if (g.triB == TRI_UPPER && k > c) continue;
      const double b = g.B[(long long)c + (long long)k * g.ldb];
      const double* a = g.transA ? g.A + (long long)k : g.A + (long long)k * g.lda;
#pragma unroll
      for (int r = 0; r < 16; ++r)
        if (r < g.m) acc[r] = fma(g.transA ? a[(long long)r * g.lda] : a[r], b, acc[r]);
    }
  }
  pdl_trigger();
#pragma unroll
  for (int r = 0; r < 16; ++r) red[w][r][lane] = acc[r];
  __syncthreads();
  if (w == 0 && c < g.n) {
    double* W = g.ws + (long long)blockIdx.y * g.m * g.n;
#pragma unroll
    for (int r = 0; r < 16; ++r)
      if (r < g.m) W[(long long)r + (long long)c * g.m] =
          ((red[0][r][lane] + red[1][r][lane]) + red[2][r][lane]) + red[3][r][lane];
  }
}

// Thin products (n <= 16, op(B) = B): thread = output row; the CTA's 128 rows
// share 32-term K tiles of op(A) and op(B) staged through shared memory (read
// along A's contiguous dimension either way), so every FP64 instruction has
// all lanes busy.  The next tile is loaded into registers while the current
// one is multiplied.  blockIdx.y selects a K chunk; partial sums go to the
// split-K workspace in the GEMM kernel's layout.  op(A) may be triangular.
__global__ void __launch_bounds__(128) gemm_thin_n_kernel(GemmDesc g, int kchunk) {
  __shared__ double As[32][129];
  __shared__ double Bs[32][17];
  pdl_wait();
  const int tid = threadIdx.x;
  const int r0 = blockIdx.x * 128, r = r0 + tid;
  int k0 = blockIdx.y * kchunk, k1 = min(g.k, k0 + kchunk);
  if (g.triA == TRI_LOWER) k1 = min(k1, r0 + 128);  // op(A)(r, kk) = 0 for kk > r
  if (g.triA == TRI_UPPER) k0 = max(k0, r0);        // op(A)(r, kk) = 0 for kk < r
  double acc[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) acc[c] = 0.0;
  double ra[32], rb[4];
  auto load = [&](int kt) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int idx = tid + 128 * j;
      int i, kk;
      if (!g.transA) { i = idx & 127; kk = idx >> 7; }
      else           { kk = idx & 31; i = idx >> 5; }
      const int row = r0 + i, kg = kt + kk;
      bool ok = row < g.m && kg < k1;
      if (g.triA == TRI_LOWER) ok = ok && kg <= row;
      if (g.triA == TRI_UPPER) ok = ok && kg >= row;
      double v = 0.0;
      if (ok) v = g.transA ? g.A[(long long)kg + (long long)row * g.lda]
                           : g.A[(long long)row + (long long)kg * g.lda];
      ra[j] = v;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int idx = tid + 128 * j, kk = idx & 31, c = idx >> 5, kg = kt + kk;
      rb[j] = (c < g.n && kg < k1) ? g.B[(long long)kg + (long long)c * g.ldb] : 0.0;
    }
  };
  auto store = [&]() {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int idx = tid + 128 * j;
      if (!g.transA) As[idx >> 7][idx & 127] = ra[j];
      else           As[idx & 31][idx >> 5] = ra[j];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int idx = tid + 128 * j;
      Bs[idx & 31][idx >> 5] = rb[j];
    }
  };
  if (k0 < k1) {
    load(k0);
    for (int kt = k0; kt < k1; kt += 32) {
      store();
      __syncthreads();
      if (kt + 32 < k1) load(kt + 32);
#pragma unroll 4
      for (int kk = 0; kk < 32; ++kk) {
        const double a = As[kk][tid];
#pragma unroll
        for (int c = 0; c < 16; ++c)
          if (c < g.n) acc[c] = fma(a, Bs[kk][c], acc[c]);
      }
      __syncthreads();
    }
  }
  pdl_trigger();
  if (r < g.m) {
    double* W = g.ws + (long long)blockIdx.y * g.m * g.n;
#pragma unroll
    for (int c = 0; c < 16; ++c)
      if (c < g.n) W[(long long)r + (long long)c * g.m] = acc[c];
  }
}

// D = alpha * sum_s W_s + beta * C over the split-K partials, in slice order.
__global__ void splitk_reduce_kernel(GemmDesc g) {
  pdl_wait();
  pdl_trigger();
  const int r = blockIdx.x * 32 + threadIdx.x, c = blockIdx.y * 8 + threadIdx.y;
  if (r >= g.m || c >= g.n || (g.outLower && r < c)) return;
  const long long mn = (long long)g.m * g.n, o = (long long)r + (long long)c * g.m;
  double v = 0.0;
  for (int s = 0; s < g.ksplit; ++s) v += g.ws[s * mn + o];
  v *= g.alpha;
  const bool hi = g.D2 && r >= g.mD1;
  const long long ro = hi ? r - g.mD1 : r;
  if (g.beta != 0.0) v += g.beta * (hi ? g.C2 : g.C)[ro + (long long)c * g.ldc];
  (hi ? g.D2 : g.D)[ro + (long long)c * g.ldd] = v;
}

}  // namespace

double gemm_flops(const GemmDesc& g) {
  double m = g.m, n = g.n, k = g.k;
  double f = 2.0 * m * n * k;
  if (g.triA != TRI_NONE) f = m * (m + 1.0) * n;
  if (g.triB != TRI_NONE) f = m * n * (n + 1.0);
  if (g.outLower && g.m >= g.n && g.n > 0) f = 2.0 * k * (n * (n + 1.0) / 2.0 + (m - n) * n);
  return f * g.batch;
}

int launch_gemm_fp64(const GemmDesc& g0, cudaStream_t s) {
  if (g0.m <= 0 || g0.n <= 0 || g0.batch <= 0) return 0;
  GemmDesc g = g0;
  if (g.m <= 16 && g.transB && g.triA == TRI_NONE && g.batch == 1 && g.ws && !g.outLower &&
      !g.A2) {
    const int cx = (g.n + 31) / 32;
    int kchunks = std::max(1, std::min((2 * 152 + cx - 1) / cx, (g.k + 63) / 64));
    while (kchunks > 1 && (long long)kchunks * g.m * g.n > g.ws_elems) --kchunks;
    if ((long long)kchunks * g.m * g.n <= g.ws_elems) {
      const int kchunk = (g.k + kchunks - 1) / kchunks;
      g.ksplit = kchunks;
      launch_k(gemm_thin_m_kernel, dim3(cx, kchunks), dim3(128), 0, s, g, kchunk);
      dim3 rg((g.m + 31) / 32, (g.n + 7) / 8);
      launch_k(splitk_reduce_kernel, rg, dim3(32, 8), 0, s, g);
      return 2;
    }
  }
  if (g.n <= 16 && !g.transB && g.triB == TRI_NONE && g.batch == 1 && g.ws && !g.outLower &&
      !g.A2) {
    const int rb = (g.m + 127) / 128;
    // about two CTAs per SM, each with at least 2 K tiles to pipeline
    int kchunks = std::max(1, std::min((2 * 152 + rb - 1) / rb, (g.k + 63) / 64));
    while (kchunks > 1 && (long long)kchunks * g.m * g.n > g.ws_elems) --kchunks;
    if ((long long)kchunks * g.m * g.n <= g.ws_elems) {
      const int kchunk = ((g.k + kchunks - 1) / kchunks + 31) / 32 * 32;
      kchunks = (g.k + kchunk - 1) / kchunk;
      g.ksplit = kchunks;
      launch_k(gemm_thin_n_kernel, dim3(rb, kchunks), dim3(128), 0, s, g, kchunk);
      dim3 rg((g.m + 31) / 32, (g.n + 7) / 8);
      launch_k(splitk_reduce_kernel, rg, dim3(32, 8), 0, s, g);
      return 2;
    }
  }
  // tiles of 64 when they (with split K) cover the SMs, else tiles of 32
  auto count_tiles = [&](int tm) {
    const int tx = (g.m + tm - 1) / tm, ty = (g.n + tm - 1) / tm;
    long long tiles = 0;
    for (int bx = 0; bx < tx; ++bx)
      for (int by = 0; by < ty; ++by)
        if (!(g.outLower && bx * tm + tm <= by * tm)) ++tiles;
    return tiles;
  };
  const long long t64 = count_tiles(64);
  const bool small = g.tile == 32 || (g.tile != 64 && g.batch == 1 && g.ws &&
                                       t64 * std::min(16, std::max(1, g.k / 16)) < 152);
  const int tm = small ? 32 : 64, tk = small ? 8 : 16;
  const long long tiles = small ? count_tiles(32) : t64;
  // too few output tiles for 152 SMs (each SM retires only ~3.5 FP64 flops
  // per cycle, so one 64x64x64 tile is tens of microseconds): split K
  int ksplit = 1;
  if (g.batch == 1 && g.ws && g.k >= 2 * tk) {
    if (tiles > 0 && tiles < 2 * 152) {
      ksplit = (int)std::min<long long>(16, (3 * 152 + tiles - 1) / tiles);
      ksplit = std::min(ksplit, g.k / tk);
      while (ksplit > 1 && (long long)ksplit * g.m * g.n > g.ws_elems) --ksplit;
    }
  }
  g.ksplit = ksplit;
  const int tx = (g.m + tm - 1) / tm, ty = (g.n + tm - 1) / tm;
  dim3 grid(tx, ty, ksplit > 1 ? ksplit : g.batch);
  if (small) launch_k(gemm_fp64_kernel<32, 8>, grid, dim3(128), 0, s, g);
  else launch_k(gemm_fp64_kernel<64, 16>, grid, dim3(128), 0, s, g);
  if (ksplit > 1) {
    dim3 rg((g.m + 31) / 32, (g.n + 7) / 8);
    launch_k(splitk_reduce_kernel, rg, dim3(32, 8), 0, s, g);
    return 2;
  }
  return 1;
}

void launch_leaf_potrf(double* T, long long ldt, int nbk, int col0, DevStatus* st,
                       cudaStream_t s, int wait_polls) {
  if (nbk <= 0) return;
  launch_k(leaf_potrf_kernel, dim3(1), dim3(256), 0, s, T, ldt, nbk, col0, st,
           wait_polls > 0 ? wait_polls : LEAF_WAIT_POLLS);
}

void launch_trsm_rows(double* X, long long xrs, long long xcs, int rows, const double* L,
                      long long ldl, int nbk, int mode, int batch, long long sX, long long sL,
                      cudaStream_t s) {
  if (rows <= 0 || nbk <= 0 || batch <= 0) return;
  dim3 grid((rows + 15) / 16, batch);
  if (mode == 0)
    launch_k(trsm_rows_kernel<0>, grid, dim3(128), 0, s, X, xrs, xcs, rows, L, ldl, nbk, sX, sL);
  else
    launch_k(trsm_rows_kernel<1>, grid, dim3(128), 0, s, X, xrs, xcs, rows, L, ldl, nbk, sX, sL);
}

}  // namespace rgf

// ---------------------------------------------------------------------------
// FP64 peak probe: independent DMMA m8n8k4 chains on every SM, used as the
// denominator of the FP64 roofline (the tensor-pipe FP64 rate of this GPU).
// ---------------------------------------------------------------------------
namespace rgf {
namespace {
__global__ void __launch_bounds__(256) dmma_peak_kernel(double* out, int iters) {
  double a = 1.0 + threadIdx.x * 1e-9, b = 0.5;
  double c[4][2] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) dmma_8x8x4(c[j], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1];
  out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

int measure_fp64_peak(double* tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 4;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 4;
  const int blocks = sms * 8, threads = 256, iters = 1024;
  double* buf = nullptr;
  if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dmma_peak_kernel<<<blocks, threads>>>(buf, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return 4;
  const double flops = 2.0 * 8 * 8 * 4 * 4.0 * iters * (double)blocks * threads / 32.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return 0;
}
}  // namespace rgf
