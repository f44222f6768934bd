"""Complex Hermitian instances go through a real symmetric embedding (host
code, no GPU): M = [[X, -Y], [Y, X]] for A = X + iY, unknowns ordered per block
(Re then Im of each diagonal block, then of the arrowhead) so that M is a BTA
matrix with (2ns, nt, 2nd).  Checked against the same matrix built densely
with numpy, and the identities the solver relies on:
logdet M = 2 logdet A, M^{-1} embeds A^{-1}, M [Re x; Im x] = [Re b; Im b]."""
import numpy as np
import pytest

from oracle import rgf_oracle as O
from rgf_gb300 import gen


def _dense_hermitian(ia, ja, a, n):
    A = np.zeros((n, n), dtype=np.complex128)
    for c in range(n):
        for e in range(int(ia[c]), int(ia[c + 1])):
            A[int(ja[e]), c] = a[e]
    return A + np.tril(A, -1).conj().T


def _real_index(ns, nt, nd, k, imag):
    if k < ns * nt:
        return 2 * ns * (k // ns) + (ns if imag else 0) + k % ns
    return 2 * ns * nt + (nd if imag else 0) + (k - ns * nt)


@pytest.mark.parametrize("ns,nt,nd", [(3, 3, 2), (5, 4, 0), (4, 1, 3), (6, 2, 7)])
def test_embedding_matches_dense_construction(ns, nt, nd):
    import rgf_gb300
    n = ns * nt + nd
    ia, ja, a = gen.generate_bta_hermitian(ns, nt, nd, seed=ns + nt + nd)
    A = _dense_hermitian(ia, ja, a, n)
    ia2, ja2, a2 = rgf_gb300.hermitian_embed(ia, ja, a, ns, nt, nd)
    # lower CSC, sorted rows, within the (2ns, nt, 2nd) block pattern
    O.check_pattern(O.Layout(2 * ns, nt, 2 * nd), ia2, ja2)
    M = O.to_dense(ia2, ja2, a2)
    P = np.zeros((2 * n, n), dtype=np.complex128)  # real unknown -> complex
    for k in range(n):
        P[_real_index(ns, nt, nd, k, 0), k] = 1.0
        P[_real_index(ns, nt, nd, k, 1), k] = 1j
    Mref = np.zeros((2 * n, 2 * n))
    re = [_real_index(ns, nt, nd, k, 0) for k in range(n)]
    im = [_real_index(ns, nt, nd, k, 1) for k in range(n)]
    Mref[np.ix_(re, re)] = A.real
    Mref[np.ix_(im, im)] = A.real
    Mref[np.ix_(im, re)] = A.imag
    Mref[np.ix_(re, im)] = -A.imag
    assert np.array_equal(M, Mref)
    s_a, ld_a = np.linalg.slogdet(A)
    s_m, ld_m = np.linalg.slogdet(M)
    assert s_m > 0 and abs(ld_m - 2 * ld_a) <= 1e-12 * abs(ld_m)
    Mi = np.linalg.inv(M)
    Ai = np.linalg.inv(A)
    assert np.allclose(Mi[re, re], np.diag(Ai).real, rtol=1e-12)
    assert np.max(np.abs(np.diag(Ai).imag)) <= 1e-14 * np.max(np.abs(np.diag(Ai)))


def test_embedding_rejects_upper_entries():
    import rgf_gb300
    ia = np.array([0, 2, 3], dtype=np.uint64)
    ja = np.array([0, 1, 0], dtype=np.uint64)   # column 1 holds row 0: upper
    a = np.ones(3, dtype=np.complex128)
    with pytest.raises(rgf_gb300.RGFError):
        rgf_gb300.hermitian_embed(ia, ja, a, 1, 2, 0)


def test_complex_dropin_class_compiles_and_links(tmp_path):
    """include/RGF.H's RGF<std::complex<double>> builds against the library
    (the reference's RGF<CPX> surface: complex arrays, complex logDet)."""
    import shutil
    import subprocess
    import os
    import rgf_gb300
    if not shutil.which("g++"):
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "t.cpp"
    src.write_text(
        '#include "RGF.H"\n'
        "typedef std::complex<double> CPX;\n"
        "int main(int argc, char**) {\n"
        "  size_t ia[3] = {0, 1, 2}, ja[2] = {0, 1};\n"
        "  CPX a[2] = {CPX(2.0, 0.0), CPX(3.0, 0.0)}, b[2] = {1.0, 1.0}, x[2], d[2];\n"
        "  if (argc > 1) {\n"
        "    RGF<CPX> r(ia, ja, a, 1, 2, 0);\n"
        "    CPX l = r.logDet(); r.solve(x, b, 1); r.RGFdiag(d);\n"
        "    return (int)(l.real() + r.residualNormNormalized(x, b));\n"
        "  }\n"
        "  return 0;\n"
        "}\n")
    lib = os.path.dirname(rgf_gb300.library_path())
    r = subprocess.run(["g++", "-std=c++11", "-O1", str(src), "-I", os.path.join(root, "include"),
                        "-L", lib, "-lrgf_gb300", "-Wl,-rpath," + lib, "-o",
                        str(tmp_path / "t")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
