// Replay driver: runs the reference's RGF<double> (RGF.H, unmodified, on the
// host stand-ins of replay_shim.cpp) on one matrix and writes every result at
// full precision.  TEST INFRASTRUCTURE ONLY (golden-vector generation).
//
// usage: rgf_replay ns nt nd matrix.dat rhs.txt nrhs out_prefix
// writes: out_prefix.mf  (factor MF after factorize, mf_size doubles)
//         out_prefix.x   (solve result, n*nrhs doubles, column-major)
//         out_prefix.diag (RGFdiag, n doubles)
//         out_prefix.txt (logdet residual residual_normalized, %.17g)
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <vector>
#include <cmath>
#include <sys/time.h>
#include <sys/stat.h>
#include <cuda_runtime.h>
#include "cublas_v2.h"
#include "Types.H"
#include "Utilities.H"
#include "CWC_utility.H"
// MF is a private member; expose it to dump the factor.
#define private public
#include "RGF.H"
#undef private

static void dump(const char* prefix, const char* ext, const double* p, size_t n) {
  char path[4096];
  std::snprintf(path, sizeof(path), "%s.%s", prefix, ext);
  FILE* f = std::fopen(path, "wb");
  if (!f || std::fwrite(p, sizeof(double), n, f) != n) {
    std::fprintf(stderr, "write failed: %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 8) {
    std::fprintf(stderr, "usage: %s ns nt nd matrix.dat rhs.txt nrhs out_prefix\n", argv[0]);
    return 1;
  }
  const size_t ns = std::strtoul(argv[1], nullptr, 10), nt = std::strtoul(argv[2], nullptr, 10),
               nd = std::strtoul(argv[3], nullptr, 10);
  const size_t nrhs = std::strtoul(argv[6], nullptr, 10);
  FILE* F = std::fopen(argv[4], "r");
  if (!F) return 1;
  size_t n, n2, nnz;
  if (std::fscanf(F, "%zu %zu %zu", &n, &n2, &nnz) != 3) return 1;
  std::vector<size_t> ia(n + 1);
  for (auto& v : ia) if (std::fscanf(F, "%zu", &v) != 1) return 1;
  nnz = ia[n];
  std::vector<size_t> ja(nnz);
  std::vector<double> a(nnz);
  for (auto& v : ja) if (std::fscanf(F, "%zu", &v) != 1) return 1;
  for (auto& v : a) if (std::fscanf(F, "%lf", &v) != 1) return 1;
  std::fclose(F);
  std::vector<double> b(n * nrhs), x(n * nrhs), diag(n);
  F = std::fopen(argv[5], "r");
  if (!F) return 1;
  for (auto& v : b) if (std::fscanf(F, "%lf", &v) != 1) return 1;
  std::fclose(F);

  RGF<double> solver(ia.data(), ja.data(), a.data(), ns, nt, nd);
  solver.factorize();
  dump(argv[7], "mf", solver.MF, solver.matrix_n_nonzeros);
  solver.solve(x.data(), b.data(), nrhs);
  const double logdet = solver.logDet();
  solver.RGFdiag(diag.data());
  const double res = solver.residualNorm(x.data(), b.data());
  const double resn = solver.residualNormNormalized(x.data(), b.data());
  dump(argv[7], "x", x.data(), x.size());
  dump(argv[7], "diag", diag.data(), diag.size());
  char path[4096];
  std::snprintf(path, sizeof(path), "%s.txt", argv[7]);
  FILE* T = std::fopen(path, "w");
  std::fprintf(T, "%.17g %.17g %.17g\n", logdet, res, resn);
  std::fclose(T);
  return 0;
}
