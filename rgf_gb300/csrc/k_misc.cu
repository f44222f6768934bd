// Memory-bound kernels of the RGF recursion: CSC ingest into the block
// layout, reductions, diagonal extraction, residual SpMV and small helpers.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "rgf_internal.h"

namespace rgf {

// Block-column layout (the reference's MF, RGF.H:95, 114-138):
// block column i < nt-1 is (2ns+nd) x ns = [L_ii; L_{i+1,i}; C_i],
// block column nt-1 is (ns+nd) x ns = [L_ii; C_i], the corner is nd x nd.
__host__ __device__ inline long long col_offset_d(long long ns, long long nt, long long nd,
                                                  long long i) {
  if (i < nt) return i * ns * (2 * ns + nd);
  return (nt - 1) * ns * (2 * ns + nd) + ns * (ns + nd);
}
__host__ __device__ inline long long lda_d(long long ns, long long nt, long long nd, long long i) {
  if (i < nt - 1) return 2 * ns + nd;
  if (i < nt) return ns + nd;
  return nd;
}
__host__ __device__ inline long long dense_row_d(long long ns, long long nt, long long i) {
  if (i < nt - 1) return 2 * ns;
  if (i == nt - 1) return ns;
  return 0;
}

long long mf_col_offset(const BtaShape& sh, long long i) { return col_offset_d(sh.ns, sh.nt, sh.nd, i); }
long long mf_lda(const BtaShape& sh, long long i) { return lda_d(sh.ns, sh.nt, sh.nd, i); }
long long mf_dense_row(const BtaShape& sh, long long i) { return dense_row_d(sh.ns, sh.nt, i); }

namespace {

// One warp per CSC column: the column's block column and panel offset are
// computed once, then every entry maps to a row of that panel.  Follows the
// mapping of the reference's getPos (CWC_utility.cu:998-1029) without its
// per-entry linear column search (CWC_utility.cu:1093-1095).
__global__ void ingest_kernel(BtaShape sh, long long c_lo, long long c_hi,
                              const size_t* __restrict__ ia, const size_t* __restrict__ ja,
                              const double* __restrict__ a, double* __restrict__ MF,
                              DevStatus* st) {
  pdl_wait();
  pdl_trigger();
  const long long c = c_lo + (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= c_hi) return;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd, n = sh.n;
  const long long ib = c < ns * nt ? c / ns : nt;
  const long long jc = ib < nt ? c - ib * ns : c - nt * ns;
  const long long off = col_offset_d(ns, nt, nd, ib);
  const long long lda = lda_d(ns, nt, nd, ib);
  const long long ro = dense_row_d(ns, nt, ib);
  const size_t e0 = ia[c], e1 = ia[c + 1];
  bool bad = false;
  for (size_t e = e0 + lane; e < e1; e += 32) {
    const long long r = (long long)ja[e];
    bool ok = r >= c && r < n;
    long long row = 0;
    if (ok) {
      const long long rb = r < ns * nt ? r / ns : nt;
      if (rb == ib) row = (ib < nt) ? r - ib * ns : r - nt * ns;
      else if (rb == ib + 1 && rb < nt) row = r - ib * ns;
      else if (rb == nt) row = ro + (r - nt * ns);
      else ok = false;
    }
    if (ok) MF[off + jc * lda + row] = a[e];
    else bad = true;
  }
  if (bad) atomicOr(&st->bad_input, 1);
}

// log of every diagonal entry of the factor MF; each block of 256 columns sums
// its logs in a fixed tree order into parts[block]
__global__ void diag_log_kernel(BtaShape sh, const double* MF, double* parts) {
  pdl_wait();
  pdl_trigger();
  __shared__ double v[256];
  const long long k = (long long)blockIdx.x * 256 + threadIdx.x;
  double x = 0.0;
  if (k < sh.n) {
    const long long ns = sh.ns, nt = sh.nt, nd = sh.nd;
    long long pos;
    if (k < ns * nt) {
      const long long i = k / ns, j = k - i * ns;
      pos = col_offset_d(ns, nt, nd, i) + j * (lda_d(ns, nt, nd, i) + 1);
    } else {
      const long long j = k - ns * nt;
      pos = col_offset_d(ns, nt, nd, nt) + j * (nd + 1);
    }
    x = log(MF[pos]);
  }
  v[threadIdx.x] = x;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) v[threadIdx.x] += v[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = v[0];
}

__global__ void logdet_reduce_kernel(const double* parts, int nparts, double* out) {
  pdl_wait();
  pdl_trigger();
  const int lane = threadIdx.x;
  double s = 0.0;
  for (int i = lane; i < nparts; i += 32) s += parts[i];
  __shared__ double ws[32];
  ws[lane] = s;
  __syncwarp();
  if (lane == 0) {
    double t = 0.0;
    for (int i = 0; i < 32; ++i) t += ws[i];
    *out = 2.0 * t;
  }
}

__global__ void extract_diag_kernel(BtaShape sh, const double* MS, double* diag) {
  pdl_wait();
  pdl_trigger();
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sh.n) return;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd;
  long long pos;
  if (k < ns * nt) {
    const long long i = k / ns, j = k - i * ns;
    pos = col_offset_d(ns, nt, nd, i) + j * (lda_d(ns, nt, nd, i) + 1);
  } else {
    const long long j = k - ns * nt;
    pos = col_offset_d(ns, nt, nd, nt) + j * (nd + 1);
  }
  diag[k] = MS[pos];
}

__global__ void set_identity_kernel(double* X, long long ld, int m, long long stride) {
  pdl_wait();
  pdl_trigger();
  X += (long long)blockIdx.z * stride;
  const int r = blockIdx.x * 32 + threadIdx.x, c = blockIdx.y * 8 + threadIdx.y;
  if (r < m && c < m) X[r + (long long)c * ld] = (r == c) ? 1.0 : 0.0;
}

__global__ void copy_kernel(const double* X, long long ldx, double* Y, long long ldy, int m,
                            int n, long long sX, long long sY) {
  pdl_wait();
  pdl_trigger();
  X += (long long)blockIdx.z * sX;
  Y += (long long)blockIdx.z * sY;
  const int r = blockIdx.x * 32 + threadIdx.x, c = blockIdx.y * 8 + threadIdx.y;
  if (r < m && c < n) Y[r + (long long)c * ldy] = X[r + (long long)c * ldx];
}

// X(r, c) = X(c, r) for r < c: the strictly upper triangle of the n x n
// matrix X (column-major, ld) from its lower one.  The CTA of source tile
// (bi, bj), bi >= bj, reads that 32 x 32 lower tile along its columns into
// shared memory and writes it transposed along the columns of tile (bj, bi);
// no CTA reads a tile another one writes.
__global__ void mirror_lower_kernel(double* X, long long ld, int n) {
  __shared__ double t[32][33];  // t[column offset][row offset] of the source tile
  pdl_wait();
  pdl_trigger();
  const int bi = blockIdx.x, bj = blockIdx.y;
  if (bi < bj) return;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int k = ty; k < 32; k += 8) {
    const int r = bi * 32 + tx, c = bj * 32 + k;
    if (r < n && c < n) t[k][tx] = X[r + (long long)c * ld];
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int r = bj * 32 + tx, c = bi * 32 + k;  // X(r, c) = X(c, r) = t[tx][k]
    if (r < c && c < n) X[r + (long long)c * ld] = t[tx][k];
  }
}

// y = A x with A symmetric, stored as its lower CSC: column c contributes
// a_rc x_c to y_r (scatter) and, off the diagonal, a_rc x_r to y_c (gather).
// Entries outside the lower triangle (r < c) or past the last row (r >= n)
// are skipped, so every write stays inside y[0, n); when `bad` is given such
// an entry also sets *bad.
__global__ void sym_spmv_kernel(long long n, const size_t* __restrict__ ia,
                                const size_t* __restrict__ ja, const double* __restrict__ a,
                                const double* __restrict__ x, double* y, int* bad) {
  pdl_wait();
  pdl_trigger();
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= n) return;
  const double xc = x[c];
  double g = 0.0;
  bool skipped = false;
  for (size_t e = ia[c] + lane; e < ia[c + 1]; e += 32) {
    const size_t ru = ja[e];
    if (ru < (size_t)c || ru >= (size_t)n) {
      skipped = true;
      continue;
    }
    const long long r = (long long)ru;
    const double v = a[e];
    atomicAdd(&y[r], v * xc);
    if (r != c) g += v * x[r];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
  if (lane == 0 && g != 0.0) atomicAdd(&y[c], g);
  if (skipped && bad) atomicExch(bad, 1);
}

// Y[:, q] = A X[:, q] for q < nrhs (<= SPMV_MAX_RHS, columns n apart): the
// product of sym_spmv_kernel for several right-hand sides in one pass over
// the CSC (each entry is read once for all of them).  The CSC must be valid
// (the handle's, which ingest checked).
__global__ void sym_spmv_multi_kernel(long long n, const size_t* __restrict__ ia,
                                      const size_t* __restrict__ ja,
                                      const double* __restrict__ a,
                                      const double* __restrict__ X, double* Y, int nrhs) {
  pdl_wait();
  pdl_trigger();
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= n) return;
  double xc[SPMV_MAX_RHS], g[SPMV_MAX_RHS];
#pragma unroll
  for (int q = 0; q < SPMV_MAX_RHS; ++q) {
    xc[q] = q < nrhs ? X[q * n + c] : 0.0;
    g[q] = 0.0;
  }
  for (size_t e = ia[c] + lane; e < ia[c + 1]; e += 32) {
    const long long r = (long long)ja[e];
    const double v = a[e];
#pragma unroll
    for (int q = 0; q < SPMV_MAX_RHS; ++q) {
      if (q < nrhs) {
        atomicAdd(&Y[q * n + r], v * xc[q]);
        if (r != c) g[q] += v * X[q * n + r];
      }
    }
  }
#pragma unroll
  for (int q = 0; q < SPMV_MAX_RHS; ++q) {
    double t = g[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0 && q < nrhs && t != 0.0) atomicAdd(&Y[q * n + c], t);
  }
}

// out[0] = ||b - y||_2, out[1] = ||b||_2 (one CTA, 1024 threads).  As in
// dnrm2, the sums of squares are scaled so that neither overflows nor
// underflows: a first pass finds max |b - y| and max |b| (order-independent),
// a second sums the squares of the entries scaled by the power of two just
// above each maximum (exact scaling), in a fixed tree order.  If *bad is set
// (an index was out of range in the product) both outputs are NaN.
__device__ __forceinline__ double pow2_below_inv(double mx) {
  // 2^-e with 2^(e-1) <= mx < 2^e (mx > 0 and finite), so mx * 2^-e is in [0.5, 1)
  int e = 0;
  frexp(mx, &e);
  return ldexp(1.0, -e);
}

__global__ void residual_norm_kernel(long long n, const double* b, const double* y, double* out,
                                     const int* bad, const double* rres = nullptr) {
  pdl_wait();
  pdl_trigger();
  __shared__ double s1[1024], s2[1024];
  const int t = threadIdx.x;
  double m1 = 0.0, m2 = 0.0;
  // r_i = b_i - y_i, or rres[i] when the residual is given
  auto res = [&](long long i) { return rres ? rres[i] : b[i] - y[i]; };
  for (long long i = t; i < n; i += blockDim.x) {
    m1 = fmax(m1, fabs(res(i)));
    m2 = fmax(m2, fabs(b[i]));
  }
  s1[t] = m1;
  s2[t] = m2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      s1[t] = fmax(s1[t], s1[t + w]);
      s2[t] = fmax(s2[t], s2[t + w]);
    }
    __syncthreads();
  }
  const double mr = s1[0], mb = s2[0];
  __syncthreads();
  const bool fr = mr > 0.0 && isfinite(mr), fb = mb > 0.0 && isfinite(mb);
  const double sr = fr ? pow2_below_inv(mr) : 1.0, sb = fb ? pow2_below_inv(mb) : 1.0;
  double r2 = 0.0, b2 = 0.0;
  for (long long i = t; i < n; i += blockDim.x) {
    const double r = res(i) * sr, bb = b[i] * sb;
    r2 += r * r;
    b2 += bb * bb;
  }
  s1[t] = r2;
  s2[t] = b2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      s1[t] += s1[t + w];
      s2[t] += s2[t + w];
    }
    __syncthreads();
  }
  if (t == 0) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    const bool invalid = bad && *bad;
    out[0] = invalid ? nan : (fr ? sqrt(s1[0]) / sr : mr);
    out[1] = invalid ? nan : (fb ? sqrt(s2[0]) / sb : mb);
  }
}

// partial[i][q][dd] = sum_j C_i(dd, j) * rhs_i(j, q): one CTA per block
// column i, one warp per (dd, q) pair, fixed-order warp reduction.
__global__ void arrow_gemv_kernel(BtaShape sh, const double* MF, const double* rhs, long long ldr,
                                  int nrhs, double* partial) {
  pdl_wait();
  pdl_trigger();
  const long long i = blockIdx.x;
  const long long ns = sh.ns, nt = sh.nt, nd = sh.nd;
  const double* Cb = MF + col_offset_d(ns, nt, nd, i) + dense_row_d(ns, nt, i);
  const long long lda = lda_d(ns, nt, nd, i);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int p = warp; p < nd * nrhs; p += nw) {
    const int dd = p % nd, q = p / nd;
    const double* R = rhs + i * ns + (long long)q * ldr;
    double s = 0.0;
    for (long long j = lane; j < ns; j += 32) s += Cb[dd + j * lda] * R[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) partial[(i * nrhs + q) * nd + dd] = s;
  }
}

__global__ void arrow_reduce_kernel(BtaShape sh, const double* partial, int nrhs, double* rhs,
                                    long long ldr) {
  pdl_wait();
  pdl_trigger();
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const long long nd = sh.nd;
  if (p >= nd * nrhs) return;
  const int dd = p % nd, q = p / nd;
  double s = 0.0;
  for (long long i = 0; i < sh.nt; ++i) s += partial[(i * nrhs + q) * nd + dd];
  rhs[sh.nt * sh.ns + dd + (long long)q * ldr] -= s;
}

}  // namespace

void launch_ingest(const BtaShape& sh, const size_t* ia, const size_t* ja, const double* a,
                   double* MF, DevStatus* st, cudaStream_t s, long long c_lo, long long c_hi) {
  if (c_hi < 0) c_hi = sh.n;
  if (c_hi <= c_lo) return;
  const long long threads = (c_hi - c_lo) * 32;
  const int bs = 256;
  launch_k(ingest_kernel, dim3((unsigned)((threads + bs - 1) / bs)), dim3(bs), 0, s, sh, c_lo,
           c_hi, ia, ja, a, MF, st);
}

int logdet_parts(const BtaShape& sh) { return (int)((sh.n + 255) / 256); }

void launch_logdet(const BtaShape& sh, const double* MF, double* parts, double* out,
                   cudaStream_t s) {
  const int np = logdet_parts(sh);
  launch_k(diag_log_kernel, dim3(np), dim3(256), 0, s, sh, MF, parts);
  launch_k(logdet_reduce_kernel, dim3(1), dim3(32), 0, s, parts, np, out);
}

void launch_extract_diag(const BtaShape& sh, const double* MS, double* diag, cudaStream_t s) {
  launch_k(extract_diag_kernel, dim3((unsigned)((sh.n + 255) / 256)), dim3(256), 0, s, sh, MS,
           diag);
}

void launch_set_identity(double* X, long long ld, int m, int batch, long long stride,
                         cudaStream_t s) {
  if (m <= 0 || batch <= 0) return;
  dim3 grid((m + 31) / 32, (m + 7) / 8, batch);
  launch_k(set_identity_kernel, grid, dim3(32, 8), 0, s, X, ld, m, stride);
}

void launch_mirror_lower(double* X, long long ld, int n, cudaStream_t s) {
  if (n <= 1) return;
  const unsigned nb = (unsigned)((n + 31) / 32);
  launch_k(mirror_lower_kernel, dim3(nb, nb), dim3(32, 8), 0, s, X, ld, n);
}

void launch_copy(const double* X, long long ldx, double* Y, long long ldy, int m, int n,
                 int batch, long long sX, long long sY, cudaStream_t s) {
  if (m <= 0 || n <= 0 || batch <= 0) return;
  dim3 grid((m + 31) / 32, (n + 7) / 8, batch);
  launch_k(copy_kernel, grid, dim3(32, 8), 0, s, X, ldx, Y, ldy, m, n, sX, sY);
}

// r = b - y; x += d (element-wise over len entries)
__global__ void sub_kernel(long long len, const double* b, const double* y, double* r) {
  pdl_wait();
  pdl_trigger();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) r[i] = b[i] - y[i];
}
__global__ void add_kernel(long long len, double* x, const double* d) {
  pdl_wait();
  pdl_trigger();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < len) x[i] += d[i];
}

void launch_residual_vectors(long long n, int nrhs, const size_t* ia, const size_t* ja,
                             const double* a, const double* X, const double* B, double* Y,
                             double* R, cudaStream_t s) {
  cudaMemsetAsync(Y, 0, sizeof(double) * n * nrhs, s);
  const long long threads = n * 32;
  const unsigned grid = (unsigned)((threads + 255) / 256);
  for (int q0 = 0; q0 < nrhs; q0 += SPMV_MAX_RHS)  // the CSC is read once per 16 RHS
    launch_k(sym_spmv_multi_kernel, dim3(grid), dim3(256), 0, s, n, ia, ja, a, X + q0 * n,
             Y + q0 * n, std::min(SPMV_MAX_RHS, nrhs - q0));
  const long long len = n * nrhs;
  launch_k(sub_kernel, dim3((unsigned)((len + 255) / 256)), dim3(256), 0, s, len, B, Y, R);
}

void launch_rhs_norms(long long n, int nrhs, const double* R, const double* B, double* out,
                      cudaStream_t s) {
  for (int q = 0; q < nrhs; ++q)
    launch_k(residual_norm_kernel, dim3(1), dim3(1024), 0, s, n, B + q * n, B + q * n, out + 2 * q,
             (const int*)nullptr, (const double*)(R + q * n));
}

void launch_add(long long len, double* x, const double* d, cudaStream_t s) {
  launch_k(add_kernel, dim3((unsigned)((len + 255) / 256)), dim3(256), 0, s, len, x, d);
}

cudaError_t launch_residual(long long n, const size_t* ia, const size_t* ja, const double* a,
                            const double* x, const double* b, double* scratch, double* out,
                            int* bad, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(double) * n, s);
  if (e == cudaSuccess && bad) e = cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  const long long threads = n * 32;
  launch_k(sym_spmv_kernel, dim3((unsigned)((threads + 255) / 256)), dim3(256), 0, s, n, ia, ja,
           a, x, scratch, bad);
  launch_k(residual_norm_kernel, dim3(1), dim3(1024), 0, s, n, b, (const double*)scratch, out,
           (const int*)bad, (const double*)nullptr);
  return cudaGetLastError();
}

void launch_arrow_gemv(const BtaShape& sh, const double* MF, const double* rhs, long long ldr,
                       int nrhs, double* partial, cudaStream_t s) {
  if (sh.nd <= 0) return;
  launch_k(arrow_gemv_kernel, dim3((unsigned)sh.nt), dim3(256), 0, s, sh, MF, rhs, ldr, nrhs,
           partial);
}

void launch_arrow_reduce(const BtaShape& sh, const double* partial, int nrhs, double* rhs,
                         long long ldr, cudaStream_t s) {
  if (sh.nd <= 0) return;
  const int p = (int)(sh.nd * nrhs);
  launch_k(arrow_reduce_kernel, dim3((p + 127) / 128), dim3(128), 0, s, sh, partial, nrhs, rhs, ldr);
}

}  // namespace rgf
