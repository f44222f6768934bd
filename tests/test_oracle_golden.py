"""The CPU oracle pinned against golden vectors from the reference itself.

tests/golden/*.npz were produced by tests/golden/make_golden.py from the CPU
replay of the reference's unmodified RGF.H (oracle/_ref).  Here the numpy
oracle must reproduce them: factor (lower triangles), logDet, solve and the
reference's RGFdiag recursion to rounding, and the exact selected inversion
must match dense LAPACK.
"""
import glob
import os

import numpy as np
import pytest

from oracle import rgf_oracle as O

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "golden_*.npz")))


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[7:-4] for p in GOLDEN])
def test_oracle_matches_reference_replay(path):
    g = load(path)
    ns, nt, nd = int(g["ns"]), int(g["nt"]), int(g["nd"])
    L = O.Layout(ns, nt, nd)
    MF = O.ingest(L, g["ia"], g["ja"], g["a"])
    O.factorize(L, MF)
    for i in range(nt + (1 if nd else 0)):
        o = L.panel(MF, i)
        r = L.panel(g["mf"], i)
        low = np.tril(np.ones(o.shape, dtype=bool))
        assert np.max(np.abs(o[low] - r[low])) <= 1e-13 * np.max(np.abs(r[low]))
    ld = O.logdet(L, MF)
    assert abs(ld - float(g["logdet"])) <= 1e-13 * abs(float(g["logdet"]))
    assert abs(ld - float(g["logdet_dense"])) <= 1e-12 * abs(float(g["logdet_dense"]))
    x = O.solve(L, MF, g["b"])
    assert np.max(np.abs(x - g["x"])) <= 1e-12 * np.max(np.abs(g["x"]))
    dc = O.selinv_compat(L, MF)
    np.testing.assert_allclose(dc, g["diag"], rtol=1e-12, atol=0)
    de = O.selinv_exact(L, MF)
    np.testing.assert_allclose(de, g["diag_dense"], rtol=1e-12, atol=0)
    assert abs(O.residual_norm(g["ia"], g["ja"], g["a"], g["x"][:, 0], g["b"][:, 0])
               - float(g["res"])) <= 1e-14 + 1e-6 * float(g["res"])


def test_reference_rgfdiag_is_truncated_when_nd_positive():
    """The reference's recursion drops the arrowhead cross terms (nd > 0)."""
    g = load(os.path.join(os.path.dirname(__file__), "golden", "golden_A11.npz"))
    rel = np.max(np.abs(g["diag"] - g["diag_dense"]) / np.abs(g["diag_dense"]))
    assert 1e-6 < rel < 1e-3
    g = load(os.path.join(os.path.dirname(__file__), "golden", "golden_A9.npz"))
    np.testing.assert_allclose(g["diag"], g["diag_dense"], rtol=1e-13)


def test_diag_pos_matches_layout():
    L = O.Layout(3, 3, 2)
    # RGF.H:114-138 for ns=3, nt=3, nd=2: lda 8 for blocks 0,1; 5 for block 2
    exp = [0, 9, 18, 24, 33, 42, 48, 54, 60, 63, 66]
    assert list(L.diag_pos()) == exp
    assert L.mf_size == 2 * 2 * 9 + 9 + 11 * 2


def test_oracle_rejects_pattern_violation():
    g = load(GOLDEN[0])
    L = O.Layout(int(g["ns"]), int(g["nt"]), int(g["nd"]))
    ja = g["ja"].copy()
    ja[0] = len(g["ia"]) + 5
    with pytest.raises(ValueError):
        O.ingest(L, g["ia"], ja, g["a"])
