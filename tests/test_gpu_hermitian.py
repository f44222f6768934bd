"""Complex Hermitian instances (RGF<complex<double>>) on the GPU against dense
numpy: logDet = log det A, solve, RGFdiag = diag(A^{-1}) (real), the residual
norm; in FP64 (the FP64 tolerances) and split precision (logDet 1e-9, RGFdiag
1e-8, refined solves 1e-13)."""
import numpy as np
import pytest

from rgf_gb300 import gen

pytestmark = pytest.mark.gpu


def _dense(ia, ja, a, n):
    A = np.zeros((n, n), dtype=np.complex128)
    for c in range(n):
        for e in range(int(ia[c]), int(ia[c + 1])):
            A[int(ja[e]), c] = a[e]
    return A + np.tril(A, -1).conj().T


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("ns,nt,nd", [(5, 3, 2), (40, 4, 3), (64, 3, 0), (33, 2, 7), (70, 1, 4)])
def test_hermitian_matches_dense(rgf, precision, ns, nt, nd):
    n = ns * nt + nd
    ia, ja, a = gen.generate_bta_hermitian(ns, nt, nd, seed=7 * ns + nt)
    A = _dense(ia, ja, a, n)
    rng = np.random.default_rng(n)
    b = rng.standard_normal((n, 3)) + 1j * rng.standard_normal((n, 3))
    s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
    ld = s.logDet()
    x = s.solve(np.empty_like(b, order="F"), b, 3)
    d = s.RGFdiag()
    ld_ref = np.linalg.slogdet(A)[1]
    x_ref = np.linalg.solve(A, b)
    d_ref = np.diag(np.linalg.inv(A))
    ltol, dtol = (1e-12, 1e-10) if precision == "fp64" else (1e-9, 1e-8)
    assert abs(ld - ld_ref) <= ltol * abs(ld_ref)
    assert np.max(np.abs(d - d_ref) / np.abs(d_ref)) <= dtol
    assert np.all(d.imag == 0.0)
    assert np.max(np.abs(x - x_ref)) <= 1e-12 * np.max(np.abs(x_ref))
    for q in range(3):
        r = np.linalg.norm(b[:, q] - A @ x[:, q]) / np.linalg.norm(b[:, q])
        assert r <= 1e-13
    res = s.residualNormNormalized(np.ascontiguousarray(x[:, 0]), np.ascontiguousarray(b[:, 0]))
    assert res <= 1e-13
    s.close()
