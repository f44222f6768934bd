// rgf_main: command-line driver with the reference driver's interface
// (main.C:18-134): argv = ns nt nd matrix.dat rhs.txt; reads the .dat matrix
// (n, n, nnz, ia[n+1], ja[nnz], a[nnz]) and one right-hand side, runs
// factorize, solve, logDet and RGFdiag through the drop-in RGF<double>, and
// prints the same report: logdet, the four stage times, the two residual
// norms and the solution vector.
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <exception>
#include <vector>

#include "RGF.H"

static bool read_matrix(const char* path, size_t& n, std::vector<size_t>& ia,
                        std::vector<size_t>& ja, std::vector<double>& a) {
  FILE* f = std::fopen(path, "r");
  if (!f) return false;
  size_t n2 = 0, nnz = 0;
  bool ok = std::fscanf(f, "%zu %zu %zu", &n, &n2, &nnz) == 3;
  if (ok) {
    ia.resize(n + 1);
    for (size_t i = 0; ok && i <= n; ++i) ok = std::fscanf(f, "%zu", &ia[i]) == 1;
  }
  if (ok) {
    nnz = ia[n];
    ja.resize(nnz);
    a.resize(nnz);
    for (size_t i = 0; ok && i < nnz; ++i) ok = std::fscanf(f, "%zu", &ja[i]) == 1;
    for (size_t i = 0; ok && i < nnz; ++i) ok = std::fscanf(f, "%lf", &a[i]) == 1;
  }
  std::fclose(f);
  return ok;
}

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s ns nt nd matrix.dat rhs.txt\n", argv[0]);
    return 1;
  }
  std::time_t now = std::time(nullptr);
  std::printf("The current date/time is: %s\n", std::asctime(std::localtime(&now)));
  const size_t ns = std::strtoul(argv[1], nullptr, 10);
  const size_t nt = std::strtoul(argv[2], nullptr, 10);
  const size_t nd = std::strtoul(argv[3], nullptr, 10);
  const size_t size = ns * nt + nd;
  size_t n = 0;
  std::vector<size_t> ia, ja;
  std::vector<double> a;
  if (!read_matrix(argv[4], n, ia, ja, a) || n != size) {
    std::fprintf(stderr, "cannot read a %zu x %zu matrix from %s\n", size, size, argv[4]);
    return 1;
  }
  const size_t nrhs = 1;
  std::vector<double> b(nrhs * size), x(nrhs * size), diag(size);
  FILE* f = std::fopen(argv[5], "r");
  if (!f) {
    std::fprintf(stderr, "cannot open %s\n", argv[5]);
    return 1;
  }
  for (size_t i = 0; i < b.size(); ++i)
    if (std::fscanf(f, "%lf", &b[i]) != 1) {
      std::fprintf(stderr, "short right-hand side in %s\n", argv[5]);
      return 1;
    }
  std::fclose(f);
  try {
    RGF<double> solver(ia.data(), ja.data(), a.data(), ns, nt, nd);
    double t0 = get_time(0.0);
    solver.factorize();
    t0 = get_time(t0);
    double t1 = get_time(0.0);
    solver.solve(x.data(), b.data(), nrhs);
    t1 = get_time(t1);
    double t2 = get_time(0.0);
    const double logdet = solver.logDet();
    t2 = get_time(t2);
    double t3 = get_time(0.0);
    solver.RGFdiag(diag.data());
    t3 = get_time(t3);
    std::printf("logdet: %f\n\n", logdet);
    std::printf("factorize time: %lg\n", t0);
    std::printf("solve time: %lg\n", t1);
    std::printf("logdet time: %lg\n", t2);
    std::printf("RGF time: %lg\n\n", t3);
    std::printf("Residual norm: %e\n", solver.residualNorm(x.data(), b.data()));
    std::printf("Residual norm normalized: %e\n\n", solver.residualNormNormalized(x.data(), b.data()));
    for (size_t i = 0; i < x.size(); ++i) std::printf("%32.24e\n", x[i]);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 2;
  }
  return 0;
}
