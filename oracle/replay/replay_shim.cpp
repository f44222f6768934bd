// Host stand-ins for the library layer under the reference's RGF.H, so the
// unmodified reference sources (RGF.H, Blas.H, Utilities.C, main.C) run on the
// CPU as a replay oracle.  TEST INFRASTRUCTURE ONLY: it is built here from the
// reference sources into oracle/_ref/ and used to generate golden vectors.
//
// What it provides, written from the interfaces' documented semantics:
// * the MAGMA v2 routines RGF<double> calls (dgemm, dtrsm, dpotrf, dtrtri,
//   dlacpy) as plain host loops, "device" pointers being host pointers;
// * the Fortran BLAS symbols the reference's host stage calls (dgemm_, dtrsm_,
//   dnrm2_);
// * host versions of the nine CWC_utility.H entry points RGF.H uses:
//   allocation, copies, fill, tril, identity, indexed copy and the supernode
//   scatter of the block-column layout.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime_api.h>

#include "magma_v2.h"

namespace {

struct TriView {
  const double* a;
  int lda;
  bool trans;
  double operator()(int i, int j) const { return trans ? a[j + (long)i * lda] : a[i + (long)j * lda]; }
};

void gemm_host(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
               const double* B, int ldb, double beta, double* C, int ldc) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int l = 0; l < k; ++l) {
        const double x = ta ? A[l + (long)i * lda] : A[i + (long)l * lda];
        const double y = tb ? B[j + (long)l * ldb] : B[l + (long)j * ldb];
        s += x * y;
      }
      double& c = C[i + (long)j * ldc];
      c = (beta == 0.0) ? alpha * s : alpha * s + beta * c;
    }
}

// B := alpha * op(A)^{-1} B (left) or alpha * B op(A)^{-1} (right), A triangular
void trsm_host(bool left, bool lower, bool trans, bool unit, int m, int n, double alpha,
               const double* A, int lda, double* B, int ldb) {
  const TriView T{A, lda, trans};
  const bool tlower = lower != trans;  // op(A) lower?
  auto b = [&](int i, int j) -> double& { return B[i + (long)j * ldb]; };
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) b(i, j) *= alpha;
  if (left) {
    for (int j = 0; j < n; ++j) {
      if (tlower) {
        for (int i = 0; i < m; ++i) {
          double s = b(i, j);
          for (int l = 0; l < i; ++l) s -= T(i, l) * b(l, j);
          b(i, j) = unit ? s : s / T(i, i);
        }
      } else {
        for (int i = m - 1; i >= 0; --i) {
          double s = b(i, j);
          for (int l = i + 1; l < m; ++l) s -= T(i, l) * b(l, j);
          b(i, j) = unit ? s : s / T(i, i);
        }
      }
    }
  } else {  // X op(A) = B, row by row
    for (int i = 0; i < m; ++i) {
      if (tlower) {
        for (int j = n - 1; j >= 0; --j) {
          double s = b(i, j);
          for (int l = j + 1; l < n; ++l) s -= b(i, l) * T(l, j);
          b(i, j) = unit ? s : s / T(j, j);
        }
      } else {
        for (int j = 0; j < n; ++j) {
          double s = b(i, j);
          for (int l = 0; l < j; ++l) s -= b(i, l) * T(l, j);
          b(i, j) = unit ? s : s / T(j, j);
        }
      }
    }
  }
}

// Block-column layout position of the lower entry (r, c): the panel of c's
// block column, and the row of r inside it (own block, next block, or the
// arrowhead rows).
long bta_pos(long r, long c, long ns, long nt, long nd) {
  const long ib = c < ns * nt ? c / ns : nt;
  const long jc = ib < nt ? c - ib * ns : c - nt * ns;
  long off, lda, ro;
  if (ib < nt - 1) { off = ib * ns * (2 * ns + nd); lda = 2 * ns + nd; ro = 2 * ns; }
  else if (ib == nt - 1) { off = ib * ns * (2 * ns + nd); lda = ns + nd; ro = ns; }
  else { off = (nt - 1) * ns * (2 * ns + nd) + ns * (ns + nd); lda = nd; ro = 0; }
  const long row = r >= ns * nt ? ro + (r - ns * nt) : r - ib * ns;
  return off + jc * lda + row;
}

}  // namespace

// ---- MAGMA v2 subset ----
magma_trans_t magma_trans_const(char c) {
  return (c == 'T' || c == 't') ? MagmaTrans : (c == 'C' || c == 'c') ? MagmaConjTrans : MagmaNoTrans;
}
magma_uplo_t magma_uplo_const(char c) {
  return (c == 'L' || c == 'l') ? MagmaLower : (c == 'U' || c == 'u') ? MagmaUpper : MagmaFull;
}
magma_diag_t magma_diag_const(char c) { return (c == 'U' || c == 'u') ? MagmaUnit : MagmaNonUnit; }
magma_side_t magma_side_const(char c) { return (c == 'R' || c == 'r') ? MagmaRight : MagmaLeft; }
magma_int_t magma_init() { return 0; }
magma_int_t magma_finalize() { return 0; }
void magma_getdevice(magma_device_t* dev) { *dev = 0; }
void magma_queue_create_from_cuda(magma_device_t, void*, void*, void*, magma_queue_t* q) { *q = nullptr; }
void magma_queue_destroy(magma_queue_t) {}
cudaStream_t magma_queue_get_cuda_stream(magma_queue_t) { return nullptr; }
void* magma_queue_get_cublas_handle(magma_queue_t) { return nullptr; }

void magma_dgemm(magma_trans_t ta, magma_trans_t tb, magma_int_t m, magma_int_t n, magma_int_t k,
                 double alpha, const double* A, magma_int_t lda, const double* B, magma_int_t ldb,
                 double beta, double* C, magma_int_t ldc, magma_queue_t) {
  gemm_host(ta != MagmaNoTrans, tb != MagmaNoTrans, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

void magma_dtrsm(magma_side_t side, magma_uplo_t uplo, magma_trans_t trans, magma_diag_t diag,
                 magma_int_t m, magma_int_t n, double alpha, const double* A, magma_int_t lda,
                 double* B, magma_int_t ldb, magma_queue_t) {
  trsm_host(side == MagmaLeft, uplo == MagmaLower, trans != MagmaNoTrans, diag == MagmaUnit, m, n,
            alpha, A, lda, B, ldb);
}

magma_int_t magma_dpotrf_gpu(magma_uplo_t uplo, magma_int_t n, double* A, magma_int_t lda,
                             magma_int_t* info) {
  *info = 0;
  if (uplo != MagmaLower) { *info = -1; return *info; }
  auto a = [&](int i, int j) -> double& { return A[i + (long)j * lda]; };
  for (int j = 0; j < n; ++j) {
    double d = a(j, j);
    for (int l = 0; l < j; ++l) d -= a(j, l) * a(j, l);
    if (!(d > 0.0)) { *info = j + 1; return *info; }
    d = std::sqrt(d);
    a(j, j) = d;
    for (int i = j + 1; i < n; ++i) {
      double s = a(i, j);
      for (int l = 0; l < j; ++l) s -= a(i, l) * a(j, l);
      a(i, j) = s / d;
    }
  }
  return 0;
}

magma_int_t magma_dtrtri_gpu(magma_uplo_t uplo, magma_diag_t diag, magma_int_t n, double* A,
                             magma_int_t lda, magma_int_t* info) {
  *info = 0;
  if (uplo != MagmaLower) { *info = -1; return *info; }
  std::vector<double> X((size_t)n * n, 0.0);
  auto a = [&](int i, int j) { return A[i + (long)j * lda]; };
  for (int j = 0; j < n; ++j) {
    const double djj = diag == MagmaUnit ? 1.0 : a(j, j);
    if (djj == 0.0) { *info = j + 1; return *info; }
    X[j + (size_t)j * n] = 1.0 / djj;
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int l = j; l < i; ++l) s += a(i, l) * X[l + (size_t)j * n];
      X[i + (size_t)j * n] = -s / (diag == MagmaUnit ? 1.0 : a(i, i));
    }
  }
  for (int j = 0; j < n; ++j)
    for (int i = j; i < n; ++i) A[i + (long)j * lda] = X[i + (size_t)j * n];
  return 0;
}

void magmablas_dlacpy(magma_uplo_t uplo, magma_int_t m, magma_int_t n, const double* A,
                      magma_int_t lda, double* B, magma_int_t ldb, magma_queue_t) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) {
      if (uplo == MagmaLower && i < j) continue;
      if (uplo == MagmaUpper && i > j) continue;
      B[i + (long)j * ldb] = A[i + (long)j * lda];
    }
}

// ---- Fortran BLAS symbols of the host stage ----
extern "C" {
void dgemm_(char* ta, char* tb, int* m, int* n, int* k, double* alpha, double* a, int* lda,
            double* b, int* ldb, double* beta, double* c, int* ldc) {
  gemm_host(*ta != 'N' && *ta != 'n', *tb != 'N' && *tb != 'n', *m, *n, *k, *alpha, a, *lda, b,
            *ldb, *beta, c, *ldc);
}
void dtrsm_(char* side, char* uplo, char* transa, char* diag, int* m, int* n, double* alpha,
            double* a, int* lda, double* b, int* ldb) {
  trsm_host(*side == 'L' || *side == 'l', *uplo == 'L' || *uplo == 'l',
            !(*transa == 'N' || *transa == 'n'), *diag == 'U' || *diag == 'u', *m, *n, *alpha, a,
            *lda, b, *ldb);
}
double dnrm2_(int* n, double* x, int* incx) {
  double s = 0.0;
  for (int i = 0; i < *n; ++i) s += x[(long)i * *incx] * x[(long)i * *incx];
  return std::sqrt(s);
}

// ---- CWC_utility.H entry points used by RGF.H ----
size_t allocate_data_on_device(void** data, size_t size) {
  *data = std::calloc(size ? size : 1, 1);
  return size;
}
size_t deallocate_data_on_dev(void* data, size_t size) {
  std::free(data);
  return size;
}
void memcpy_to_device(void* host, void* dev, size_t size) { std::memcpy(dev, host, size); }
void memcpy_to_host(void* host, void* dev, size_t size) { std::memcpy(host, dev, size); }
void d_fill_on_dev(double* x, const double value, size_t n) {
  for (size_t i = 0; i < n; ++i) x[i] = value;
}
void d_tril_on_dev(double* A, int lda, int N) {
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < j; ++i) A[i + (long)j * lda] = 0.0;
}
void d_init_eye_on_dev(double* var, int N, cudaStream_t) {
  for (long i = 0; i < (long)N * N; ++i) var[i] = 0.0;
  for (int i = 0; i < N; ++i) var[i + (long)i * N] = 1.0;
}
void d_indexed_copy_offset_on_dev(double* src, double* dst, size_t* index, size_t N,
                                  size_t offset) {
  for (size_t i = 0; i < N; ++i) dst[i] = src[index[i] - offset];
}
// ia: the supernode's cols+1 column pointers (absolute); ja/a: its entries.
void d_init_supernode_on_dev(double* M, size_t* ia, size_t* ja, double* a, size_t supernode,
                             size_t supernode_nnz, size_t supernode_offset, size_t ns, size_t nt,
                             size_t nd) {
  const long fc = (long)(supernode * ns);
  const long lc = supernode < nt ? (long)((supernode + 1) * ns) : (long)(ns * nt + nd);
  const long base = bta_pos(fc, fc, ns, nt, nd);
  for (long cc = 0; cc < lc - fc; ++cc)
    for (size_t e = ia[cc] - supernode_offset; e < ia[cc + 1] - supernode_offset; ++e) {
      if (e >= supernode_nnz) break;
      M[bta_pos((long)ja[e], fc + cc, ns, nt, nd) - base] = a[e];
    }
}
}  // extern "C"
