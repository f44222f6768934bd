/*
 * RGF.H -- drop-in C++ class for the reference's RGF<double> (RGF.H:11-80),
 * implemented over the C ABI of librgf_gb300 (rgf.h).
 *
 * Same class name, constructor and method signatures as the reference, so a
 * program written against the reference (its driver main.C included)
 * compiles unchanged with -I<this dir> and links with -lrgf_gb300.
 * Differences, all behaviour-compatible:
 *   - the CSC arrays are copied to the GPU at construction (the pointers are
 *     still kept, as in the reference, but no longer read after it);
 *   - the factor stays resident on the GPU; RGFdiag does not invalidate it;
 *   - errors throw std::runtime_error instead of being ignored;
 *   - RGFdiag returns the exact diag(A^{-1}).  Set RGF_GB300_SELINV=compat to
 *     get the reference's recursion instead, RGF_GB300_PRECISION=split for
 *     the split-precision path.
 * T = double, and T = std::complex<double> for Hermitian positive-definite
 * matrices (the reference's RGF<CPX>, RGF.H:756-774; logDet then returns
 * log det A as a complex number with zero imaginary part).
 */
#ifndef RGF_GB300_DROPIN_RGF_H
#define RGF_GB300_DROPIN_RGF_H

#include <sys/time.h>

#include <complex>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

#include "rgf.h"

/* Wall-clock helper of the reference's Utilities.C (main.C times with it). */
inline double get_time(double t0) {
  timeval tim;
  gettimeofday(&tim, NULL);
  return (double)(tim.tv_sec + (tim.tv_usec / 1000000.0)) - t0;
}

template <class T>
class RGF;

namespace rgf_gb300_detail {
inline void check(int status, const char* what) {
  if (status != RGF_OK) throw std::runtime_error(std::string(what) + ": " + rgf_status_string(status));
}
inline void env_opts(rgf_opts* o) {
  rgf_default_opts(o);
  const char* sel = std::getenv("RGF_GB300_SELINV");
  if (sel && std::strcmp(sel, "compat") == 0) o->selinv_mode = RGF_SELINV_COMPAT;
  const char* prec = std::getenv("RGF_GB300_PRECISION");
  if (prec && std::strcmp(prec, "split") == 0) o->precision = RGF_PREC_SPLIT;
  // the reference keeps the caller's arrays (RGF.H:87-89), so the upload may
  // overlap the first factorization; RGF_GB300_ASYNC_UPLOAD=0 copies at once
  const char* up = std::getenv("RGF_GB300_ASYNC_UPLOAD");
  o->async_upload = (up && up[0] == '0') ? 0 : 1;
}
}  // namespace rgf_gb300_detail

template <>
class RGF<double> {
 public:
  RGF(size_t* ia, size_t* ja, double* a, size_t ns, size_t nt, size_t nd)
      : ia_(ia), ja_(ja), a_(a), n_(ns * nt + nd), h_(NULL) {
    rgf_opts o;
    rgf_gb300_detail::env_opts(&o);
    check(rgf_create(ia, ja, a, ns, nt, nd, &o, &h_), "RGF::RGF");
  }

  RGF(size_t* ia, size_t* ja, double* a, size_t ns, size_t nt, size_t nd, const rgf_opts& o)
      : ia_(ia), ja_(ja), a_(a), n_(ns * nt + nd), h_(NULL) {
    check(rgf_create(ia, ja, a, ns, nt, nd, &o, &h_), "RGF::RGF");
  }

  ~RGF() {
    if (h_) rgf_destroy(h_);
  }

  void factorize() { check(rgf_factorize(h_), "RGF::factorize"); }

  void solve(double* b, size_t nrhs) { solve(b, b, nrhs); }

  void solve(double* x, double* b, size_t nrhs) {
    check(rgf_solve(h_, x, b, nrhs), "RGF::solve");
  }

  void RGFdiag(double* diag) { check(rgf_diag(h_, diag), "RGF::RGFdiag"); }

  double logDet() {
    double v = 0.0;
    check(rgf_logdet(h_, &v), "RGF::logDet");
    return v;
  }

  double residualNorm(double* x, double* b) {
    double v = 0.0;
    check(rgf_residual_norm(h_, x, b, &v), "RGF::residualNorm");
    return v;
  }

  double residualNormNormalized(double* x, double* b) {
    double v = 0.0;
    check(rgf_residual_norm_normalized(h_, x, b, &v), "RGF::residualNormNormalized");
    return v;
  }

  rgf_handle* handle() { return h_; }

 private:
  RGF(const RGF&);
  RGF& operator=(const RGF&);

  static void check(int status, const char* what) { rgf_gb300_detail::check(status, what); }

  size_t* ia_;
  size_t* ja_;
  double* a_;
  size_t n_;
  rgf_handle* h_;
};

/* Hermitian positive-definite matrices: the lower CSC holds complex values;
 * every array is std::complex<double> (interleaved re, im, as the C ABI takes). */
template <>
class RGF<std::complex<double> > {
 public:
  typedef std::complex<double> CPX;

  RGF(size_t* ia, size_t* ja, CPX* a, size_t ns, size_t nt, size_t nd) : h_(NULL) {
    rgf_opts o;
    rgf_gb300_detail::env_opts(&o);
    rgf_gb300_detail::check(rgf_create_hermitian(ia, ja, reinterpret_cast<double*>(a), ns, nt,
                                                 nd, &o, &h_),
                            "RGF<CPX>::RGF");
  }

  ~RGF() {
    if (h_) rgf_destroy(h_);
  }

  void factorize() { rgf_gb300_detail::check(rgf_factorize(h_), "RGF<CPX>::factorize"); }

  void solve(CPX* b, size_t nrhs) { solve(b, b, nrhs); }

  void solve(CPX* x, CPX* b, size_t nrhs) {
    rgf_gb300_detail::check(rgf_solve(h_, reinterpret_cast<double*>(x),
                                      reinterpret_cast<double*>(b), nrhs),
                            "RGF<CPX>::solve");
  }

  void RGFdiag(CPX* diag) {
    rgf_gb300_detail::check(rgf_diag(h_, reinterpret_cast<double*>(diag)), "RGF<CPX>::RGFdiag");
  }

  CPX logDet() {
    double v = 0.0;
    rgf_gb300_detail::check(rgf_logdet(h_, &v), "RGF<CPX>::logDet");
    return CPX(v, 0.0);
  }

  double residualNorm(CPX* x, CPX* b) {
    double v = 0.0;
    rgf_gb300_detail::check(rgf_residual_norm(h_, reinterpret_cast<double*>(x),
                                              reinterpret_cast<double*>(b), &v),
                            "RGF<CPX>::residualNorm");
    return v;
  }

  double residualNormNormalized(CPX* x, CPX* b) {
    double v = 0.0;
    rgf_gb300_detail::check(rgf_residual_norm_normalized(h_, reinterpret_cast<double*>(x),
                                                         reinterpret_cast<double*>(b), &v),
                            "RGF<CPX>::residualNormNormalized");
    return v;
  }

  rgf_handle* handle() { return h_; }

 private:
  RGF(const RGF&);
  RGF& operator=(const RGF&);
  rgf_handle* h_;
};

#endif /* RGF_GB300_DROPIN_RGF_H */
