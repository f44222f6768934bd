// FP64 kernels of the RGF recursion for sm_103a.
//
// On GB300 the FP64 rate is the same for DMMA (mma.sync .f64) and DFMA
// (about 1 TFLOP/s per GPU), so the FP64 GEMM below is bound by the FP64
// pipe, not by memory: 64x64 output tiles, 4 warps of 32x32 built from
// m8n8k4 DMMA fragments, operands staged through shared memory with a
// register prefetch of the next K slice.
#include <cmath>
#include <cstdint>

#include "rgf_internal.h"

namespace rgf {

namespace {

constexpr int GBM = 64, GBN = 64, GBK = 16, GPAD = 68;

__device__ __forceinline__ void dmma_8x8x4(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

struct GemmTileRange {
  int klo, khi;
};

__device__ __forceinline__ GemmTileRange k_range(const GemmDesc& g, int m0, int n0) {
  int klo = 0, khi = g.k;
  if (g.triA == TRI_LOWER) khi = min(khi, m0 + GBM);
  if (g.triA == TRI_UPPER) klo = max(klo, m0);
  if (g.triB == TRI_LOWER) klo = max(klo, n0);
  if (g.triB == TRI_UPPER) khi = min(khi, n0 + GBN);
  klo = (klo / GBK) * GBK;
  return {klo, khi};
}

__global__ void __launch_bounds__(128) gemm_fp64_kernel(GemmDesc g) {
  const int m0 = blockIdx.x * GBM;
  const int n0 = blockIdx.y * GBN;
  if (g.outLower && m0 + GBM <= n0) return;  // tile entirely above the diagonal
  const long long bz = blockIdx.z;
  const double* __restrict__ A = g.A + bz * g.sA;
  const double* __restrict__ B = g.B + bz * g.sB;
  const double* C = g.C ? g.C + bz * g.sC : nullptr;
  double* D = g.D + bz * g.sD;

  __shared__ double As[GBK][GPAD];
  __shared__ double Bs[GBK][GPAD];

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  const GemmTileRange kr = k_range(g, m0, n0);

  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  double ra[8], rb[8];
  auto load = [&](int kt) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int rr, kk;
      if (!g.transA) { rr = tid & 63; kk = (tid >> 6) + 2 * j; }
      else           { kk = tid & 15; rr = (tid >> 4) + 8 * j; }
      const int r = m0 + rr, kg = kt + kk;
      bool ok = r < g.m && kg < kr.khi;
      if (g.triA == TRI_LOWER) ok = ok && kg <= r;
      if (g.triA == TRI_UPPER) ok = ok && kg >= r;
      double v = 0.0;
      if (ok) v = g.transA ? A[(long long)kg + (long long)r * g.lda] : A[(long long)r + (long long)kg * g.lda];
      ra[j] = v;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int cc, kk;
      if (!g.transB) { kk = tid & 15; cc = (tid >> 4) + 8 * j; }
      else           { cc = tid & 63; kk = (tid >> 6) + 2 * j; }
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
    for (int j = 0; j < 8; ++j) {
      if (!g.transA) As[(tid >> 6) + 2 * j][tid & 63] = ra[j];
      else           As[tid & 15][(tid >> 4) + 8 * j] = ra[j];
      if (!g.transB) Bs[tid & 15][(tid >> 4) + 8 * j] = rb[j];
      else           Bs[(tid >> 6) + 2 * j][tid & 63] = rb[j];
    }
  };

  if (kr.klo < kr.khi) {
    load(kr.klo);
    for (int kt = kr.klo; kt < kr.khi; kt += GBK) {
      store();
      __syncthreads();
      if (kt + GBK < kr.khi) load(kt + GBK);
#pragma unroll
      for (int ks = 0; ks < GBK; ks += 4) {
        double af[4], bf[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) af[i] = As[ks + (lane & 3)][wm + i * 8 + (lane >> 2)];
#pragma unroll
        for (int j = 0; j < 4; ++j) bf[j] = Bs[ks + (lane & 3)][wn + j * 8 + (lane >> 2)];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) dmma_8x8x4(acc[i][j], af[i], bf[j]);
      }
      __syncthreads();
    }
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + wm + i * 8 + (lane >> 2);
    if (r >= g.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int c = n0 + wn + j * 8 + (lane & 3) * 2 + e;
        if (c >= g.n) continue;
        if (g.outLower && r < c) continue;
        double v = g.alpha * acc[i][j][e];
        if (g.beta != 0.0) v += g.beta * C[(long long)r + (long long)c * g.ldc];
        D[(long long)r + (long long)c * g.ldd] = v;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Leaf Cholesky of one <= 64 x 64 diagonal tile, right-looking in shared memory.
// GB300's FP64 pipe retires about two lanes per cycle per SM, so every FP64
// warp instruction is expensive: the pivot's reciprocal square root is formed
// once per column by one warp (an FP32 seed refined by two Newton steps), the
// trailing update maps warps to columns and lanes to rows (no index
// arithmetic per element), and the tile's 64 logs run in parallel.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rsqrt_newton(double d) {
  // d > 0 and normal: d = m * 4^k with m in [1, 4)
  const long long b = __double_as_longlong(d);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e == -1023) return 1.0 / sqrt(d);  // subnormal pivot
  const int k = e >> 1;
  const double m = __longlong_as_double(b - ((long long)(2 * k) << 52));
  double y = (double)rsqrtf((float)m);
  const double hm = 0.5 * m;
  y = y * fma(-hm, y * y, 1.5);
  y = y * fma(-hm, y * y, 1.5);
  return y * __longlong_as_double((long long)(1023 - k) << 52);
}

__global__ void __launch_bounds__(256) leaf_potrf_kernel(double* T, long long ldt, int nbk,
                                                         int col0, double* logpart,
                                                         DevStatus* st) {
  __shared__ double S[64][65];
  __shared__ double piv[2];
  __shared__ double lg[64];
  __shared__ int fail;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
  for (int c = warp; c < nbk; c += nw)
    for (int r = lane; r < nbk; r += 32)
      S[r][c] = (r >= c) ? T[(long long)r + (long long)c * ldt] : 0.0;
  if (tid == 0) fail = -1;
  __syncthreads();
  for (int j = 0; j < nbk; ++j) {
    if (warp == 0) {
      const double d = S[j][j];
      const bool ok = d > 0.0;
      const double y = rsqrt_newton(ok ? d : 1.0);
      if (lane == 0) {
        if (!ok && fail < 0) fail = j;
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
        piv[0] = ok ? d * y : nan;  // L_jj
        piv[1] = ok ? y : nan;      // 1 / L_jj
      }
    }
    __syncthreads();
    const double rinv = piv[1];
    for (int r = j + 1 + tid; r < nbk; r += blockDim.x) S[r][j] *= rinv;
    if (tid == 0) S[j][j] = piv[0];
    __syncthreads();
    for (int c = j + 1 + warp; c < nbk; c += nw) {
      const double ljc = S[c][j];
      for (int r = c + lane; r < nbk; r += 32) S[r][c] = fma(-S[r][j], ljc, S[r][c]);
    }
    __syncthreads();
  }
  for (int c = warp; c < nbk; c += nw)
    for (int r = c + lane; r < nbk; r += 32) T[(long long)r + (long long)c * ldt] = S[r][c];
  if (tid < nbk) lg[tid] = log(S[tid][tid]);
  __syncthreads();
  if (warp == 0) {
    double v = (lane < nbk ? lg[lane] : 0.0) + (lane + 32 < nbk ? lg[lane + 32] : 0.0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
      *logpart = v;
      if (fail >= 0) atomicMin(&st->not_spd_col, col0 + fail);
    }
  }
}

// ---------------------------------------------------------------------------
// Row-parallel triangular solve with a <= 64 x 64 lower tile: each thread
// owns one row of X in registers; the tile is broadcast from shared memory.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(32) trsm_rows_kernel(double* X, long long xrs, long long xcs,
                                                        int rows, const double* L, long long ldl,
                                                        int nbk, long long sX, long long sL) {
  __shared__ double Ls[64][65];
  __shared__ double rinv[64];
  X += (long long)blockIdx.y * sX;
  L += (long long)blockIdx.y * sL;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += blockDim.x) {
    const int c = idx >> 6, r = idx & 63;
    double v = 0.0;
    if (r < nbk && c < nbk && r >= c) v = L[(long long)r + (long long)c * ldl];
    Ls[r][c] = v;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < 64; j += blockDim.x) rinv[j] = (j < nbk) ? 1.0 / Ls[j][j] : 0.0;
  __syncthreads();
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double x[64];
#pragma unroll
  for (int j = 0; j < 64; ++j) x[j] = (j < nbk) ? X[r * xrs + (long long)j * xcs] : 0.0;
  if (MODE == 0) {
#pragma unroll
    for (int j = 0; j < 64; ++j) {
      if (j < nbk) {
        double s = x[j];
#pragma unroll
        for (int l = 0; l < j; ++l) s = fma(-x[l], Ls[j][l], s);
        x[j] = s * rinv[j];
      }
    }
  } else {
#pragma unroll
    for (int j = 63; j >= 0; --j) {
      if (j < nbk) {
        double s = x[j];
#pragma unroll
        for (int l = j + 1; l < 64; ++l) s = fma(-x[l], Ls[l][j], s);  // x[l] = 0 beyond nbk
        x[j] = s * rinv[j];
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 64; ++j)
    if (j < nbk) X[r * xrs + (long long)j * xcs] = x[j];
}

}  // namespace

double gemm_flops(const GemmDesc& g) {
  double m = g.m, n = g.n, k = g.k;
  double f = 2.0 * m * n * k;
  if (g.triA != TRI_NONE) f = m * (m + 1.0) * n;
  if (g.triB != TRI_NONE) f = m * n * (n + 1.0);
  if (g.outLower && g.m == g.n && g.n > 0) f = f * (n + 1.0) / (2.0 * n);
  return f * g.batch;
}

void launch_gemm_fp64(const GemmDesc& g, cudaStream_t s) {
  if (g.m <= 0 || g.n <= 0 || g.batch <= 0) return;
  dim3 grid((g.m + GBM - 1) / GBM, (g.n + GBN - 1) / GBN, g.batch);
  gemm_fp64_kernel<<<grid, 128, 0, s>>>(g);
}

void launch_leaf_potrf(double* T, long long ldt, int nbk, int col0, double* logpart,
                       DevStatus* st, cudaStream_t s) {
  if (nbk <= 0) return;
  leaf_potrf_kernel<<<1, 256, 0, s>>>(T, ldt, nbk, col0, logpart, st);
}

void launch_trsm_rows(double* X, long long xrs, long long xcs, int rows, const double* L,
                      long long ldl, int nbk, int mode, int batch, long long sX, long long sL,
                      cudaStream_t s) {
  if (rows <= 0 || nbk <= 0 || batch <= 0) return;
  dim3 grid((rows + 31) / 32, batch);
  if (mode == 0)
    trsm_rows_kernel<0><<<grid, 32, 0, s>>>(X, xrs, xcs, rows, L, ldl, nbk, sX, sL);
  else
    trsm_rows_kernel<1><<<grid, 32, 0, s>>>(X, xrs, xcs, rows, L, ldl, nbk, sX, sL);
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
