"""Split-precision (Ozaki, bf16 slices on tcgen05) GEMM and solver parity.

The split GEMM is checked against the FP64 DMMA kernel and numpy on the same
device operands: every entry within 2e-11 of (|A||B|)_{rc}, the bound of a
40-bit (5 slices x 8 bits) split.  The solver in split precision is checked
against the FP64 oracle at the split tolerances: logDet relative error
<= 1e-9, RGFdiag max relative error <= 1e-8; its solves are refined in FP64 to
a normalized residual <= 1e-13.
"""
import numpy as np
import pytest

from oracle import rgf_oracle as O
from rgf_gb300 import gen

pytestmark = pytest.mark.gpu

GEMM_TOL = 2e-11
LOGDET_TOL = 1e-9
DIAG_TOL = 1e-8


def _gemm_case(rgf, ta, tb, m, n, k, alpha, beta, seed, slices=0):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((k, m) if ta == "T" else (m, k))
    B = rng.standard_normal((n, k) if tb == "T" else (k, n))
    C0 = rng.standard_normal((m, n))
    dev = torch.device("cuda", 0)
    # column-major device copies: a C-contiguous transpose
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)
    lda, ldb = A.shape[0], B.shape[0]
    out = {}
    for prec in ("fp64", "split"):
        dC = torch.from_numpy(np.ascontiguousarray(C0.T)).to(dev)
        torch.cuda.synchronize()
        rgf.dgemm_device(prec, ta, tb, m, n, k, alpha, dA.data_ptr(), lda, dB.data_ptr(), ldb,
                         beta, dC.data_ptr(), m, slices=slices)
        out[prec] = dC.cpu().numpy().T
    opA = A.T if ta == "T" else A
    opB = B.T if tb == "T" else B
    ref = alpha * (opA @ opB) + beta * C0
    bound = abs(alpha) * (np.abs(opA) @ np.abs(opB))
    return out, ref, bound


@pytest.mark.parametrize("ta,tb,m,n,k", [
    ("N", "T", 128, 128, 256),
    ("N", "N", 300, 200, 1000),
    ("T", "N", 257, 129, 700),
    ("T", "T", 130, 520, 1536),
    ("N", "T", 1000, 1000, 2000),
])
def test_split_gemm_matches_fp64(rgf, ta, tb, m, n, k):
    out, ref, bound = _gemm_case(rgf, ta, tb, m, n, k, -1.0, 1.0, seed=m + n + k)
    assert np.max(np.abs(out["fp64"] - ref) / bound) <= 1e-14
    err = np.max(np.abs(out["split"] - ref) / bound)
    assert err <= GEMM_TOL, err


def test_split_gemm_scaled_rows_and_beta_zero(rgf):
    """Rows and columns of very different magnitude (per-row/column scaling)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    m, n, k = 256, 192, 512
    A = rng.standard_normal((m, k)) * np.logspace(-30, 30, m)[:, None]
    B = rng.standard_normal((k, n)) * np.logspace(20, -20, n)[None, :]
    dev = torch.device("cuda", 0)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).to(dev)
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).to(dev)
    dC = torch.full((n, m), float("nan"), dtype=torch.float64, device=dev)
    rgf.dgemm_device("split", "N", "N", m, n, k, 2.0, dA.data_ptr(), m, dB.data_ptr(), k, 0.0,
                     dC.data_ptr(), m)
    got = dC.cpu().numpy().T
    ref = 2.0 * A @ B
    bound = 2.0 * np.abs(A) @ np.abs(B)
    assert np.all(np.isfinite(got))
    assert np.max(np.abs(got - ref) / bound) <= GEMM_TOL


@pytest.mark.parametrize("slices", [7, 8])
def test_split_gemm_seven_slices_is_fp64_accurate(rgf, slices):
    """7 slices (56-bit operands) reach the accuracy of an FP64 GEMM."""
    out, ref, bound = _gemm_case(rgf, "N", "T", 640, 384, 1500, 1.0, 0.0, seed=3, slices=slices)
    assert np.max(np.abs(out["split"] - ref) / bound) <= 1e-15
    assert np.max(np.abs(out["split"] - ref) / bound) <= 4 * np.max(np.abs(out["fp64"] - ref) / bound) + 1e-16


@pytest.mark.parametrize("ns,nt,nd,fp64_diag", [
    (300, 3, 2, 1), (300, 3, 0, 0), (520, 4, 4, 1), (520, 4, 4, 0), (200, 5, 3, "native"),
])
def test_split_solver_parity(rgf, ns, nt, nd, fp64_diag):
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=4)
    n = ns * nt + nd
    b = gen.random_rhs(n, 2, 4)
    s = rgf.RGF(ia, ja, a, ns, nt, nd, precision="split", fp64_diag=fp64_diag)
    ld = s.logDet()
    d = s.RGFdiag()
    x = s.solve(np.empty_like(b), b, 2)
    ref = O.run_all(ns, nt, nd, ia, ja, a, b=b, exact=True)
    assert abs(ld - ref["logdet"]) <= LOGDET_TOL * abs(ref["logdet"])
    assert np.max(np.abs(d - ref["diag"]) / np.abs(ref["diag"])) <= DIAG_TOL
    assert np.max(np.abs(x - ref["x"])) <= 1e-12 * np.max(np.abs(ref["x"]))
    for q in range(2):
        assert O.residual_norm_normalized(ia, ja, a, x[:, q], b[:, q]) <= 1e-13


def test_split_solver_ns1000_nt50_nd4_spde_vs_oracle(rgf):
    """The ns=1000, nt=50, nd=4 workload (5-point SPDE operator on a 40 x 25
    grid plus the dense random term, seed 2) in split precision against the
    oracle's FP64 block recursion: logDet, RGFdiag and an 8-RHS refined solve."""
    ns, nt, nd = 1000, 50, 4
    ia, ja, a = gen.generate_bta(ns, nt, nd, 2, spde_grid=(40, 25))
    n = ns * nt + nd
    b = gen.random_rhs(n, 8, 2)
    s = rgf.RGF(ia, ja, a, ns, nt, nd, precision="split")
    ld = s.logDet()
    d = s.RGFdiag()
    x = s.solve(np.empty_like(b), b, 8)
    ref = O.run_all(ns, nt, nd, ia, ja, a, b=b, exact=True)
    assert abs(ld - ref["logdet"]) <= LOGDET_TOL * abs(ref["logdet"])
    assert np.max(np.abs(d - ref["diag"]) / np.abs(ref["diag"])) <= DIAG_TOL
    for q in range(8):
        assert s.residualNormNormalized(np.ascontiguousarray(x[:, q]),
                                        np.ascontiguousarray(b[:, q])) <= 1e-13
    assert np.max(np.abs(x - ref["x"])) <= 1e-10 * np.max(np.abs(ref["x"]))
    s.close()
