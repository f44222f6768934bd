// Complex Hermitian positive-definite BTA matrices through their real
// symmetric embedding.
//
// A = X + iY (X symmetric, Y antisymmetric) of size n = ns*nt + nd is
// positive definite iff M = [[X, -Y], [Y, X]] is, and M keeps the
// block-tridiagonal-arrowhead structure when its unknowns are ordered per
// block: block i holds Re of A's block i (ns) then Im of it (ns), the arrowhead
// holds Re (nd) then Im (nd).  So M is a real BTA matrix with (2ns, nt, 2nd):
//   logdet A = logdet M / 2        (det M = |det A|^2 = det(A)^2)
//   A x = b  <=>  M [Re x; Im x] = [Re b; Im b]
//   diag(A^{-1})_k = (M^{-1})_{R(k),R(k)}   (real for Hermitian A)
// The reference instantiates RGF<CPX> (RGF.H:756-774) but its recursion uses
// plain transposes with a Hermitian POTRF, which is a consistent factorization
// only for real data; this path implements the Hermitian definition.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/rgf.h"
#include "rgf_internal.h"

namespace rgf {

namespace {

struct Map {
  size_t ns, nt, nd;
  // real index of Re / Im of complex unknown k
  size_t re(size_t k) const {
    if (k < ns * nt) return 2 * ns * (k / ns) + (k % ns);
    return 2 * ns * nt + (k - ns * nt);
  }
  size_t im(size_t k) const {
    if (k < ns * nt) return 2 * ns * (k / ns) + ns + (k % ns);
    return 2 * ns * nt + nd + (k - ns * nt);
  }
};

}  // namespace

size_t hermitian_real_index(size_t ns, size_t nt, size_t nd, size_t k, int imag) {
  const Map m{ns, nt, nd};
  return imag ? m.im(k) : m.re(k);
}

int hermitian_embed(const size_t* ia, const size_t* ja, const double* a, size_t ns, size_t nt,
                    size_t nd, std::vector<size_t>& ia2, std::vector<size_t>& ja2,
                    std::vector<double>& a2) {
  const size_t n = ns * nt + nd, n2 = 2 * n;
  const Map m{ns, nt, nd};
  // every stored entry (r, c), r >= c, of A gives four entries of M (two on
  // A's diagonal, whose imaginary part is ignored); keep the lower one of each
  // symmetric pair
  struct E {
    size_t col, row;
    double v;
  };
  std::vector<E> es;
  es.reserve(4 * ia[n]);
  auto put = [&](size_t p, size_t q, double v) {
    if (p >= q) es.push_back({q, p, v});
    else es.push_back({p, q, v});
  };
  for (size_t c = 0; c < n; ++c) {
    for (size_t e = ia[c]; e < ia[c + 1]; ++e) {
      const size_t r = ja[e];
      if (r < c || r >= n) return RGF_EINVAL;
      const double x = a[2 * e], y = a[2 * e + 1];
      put(m.re(r), m.re(c), x);
      put(m.im(r), m.im(c), x);
      if (r != c) {  // the diagonal of a Hermitian matrix is real
        put(m.im(r), m.re(c), y);
        put(m.re(r), m.im(c), -y);
      }
    }
  }
  std::sort(es.begin(), es.end(), [](const E& u, const E& w) {
    return u.col != w.col ? u.col < w.col : u.row < w.row;
  });
  ia2.assign(n2 + 1, 0);
  ja2.resize(es.size());
  a2.resize(es.size());
  for (size_t i = 0; i < es.size(); ++i) {
    if (i > 0 && es[i].col == es[i - 1].col && es[i].row == es[i - 1].row) return RGF_EINVAL;
    ja2[i] = es[i].row;
    a2[i] = es[i].v;
    ia2[es[i].col + 1]++;
  }
  for (size_t c = 0; c < n2; ++c) ia2[c + 1] += ia2[c];
  return RGF_OK;
}

}  // namespace rgf

extern "C" int rgf_hermitian_embed(const size_t* ia, const size_t* ja, const double* a,
                                   size_t ns, size_t nt, size_t nd, size_t* ia2, size_t* ja2,
                                   double* a2, size_t* nnz2) {
  if (!ia || !ja || !a || !nnz2 || ns < 1 || nt < 1) return RGF_EINVAL;
  std::vector<size_t> i2, j2;
  std::vector<double> v2;
  const int st = rgf::hermitian_embed(ia, ja, a, ns, nt, nd, i2, j2, v2);
  if (st) return st;
  *nnz2 = j2.size();
  if (ia2) std::memcpy(ia2, i2.data(), sizeof(size_t) * i2.size());
  if (ja2) std::memcpy(ja2, j2.data(), sizeof(size_t) * j2.size());
  if (a2) std::memcpy(a2, v2.data(), sizeof(double) * v2.size());
  return RGF_OK;
}
