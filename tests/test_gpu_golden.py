"""GPU parity against golden vectors produced by the reference itself.

Each tests/golden/golden_*.npz holds a matrix, right-hand sides and the
outputs of the reference's RGF<double> (CPU replay of its unmodified RGF.H).
The GPU path must reproduce: the factor (lower triangles of the block-column
layout), logDet (relative 1e-12), the solve, the reference's RGFdiag
recursion in compat mode (relative 1e-10), and the exact diag(A^{-1}) from
dense LAPACK in exact mode (relative 1e-10).  The normalized residual must be
<= 1e-13 or no worse than 4x the reference's own on that matrix.
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "golden_*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[7:-4] for p in GOLDEN])
def test_gpu_matches_reference_golden(rgf, path):
    from oracle import rgf_oracle as O
    z = np.load(path)
    g = {k: z[k] for k in z.files}
    ns, nt, nd = int(g["ns"]), int(g["nt"]), int(g["nd"])
    nrhs = g["b"].shape[1]
    s = rgf.RGF(g["ia"], g["ja"], g["a"], ns, nt, nd, selinv="compat")
    s.factorize()
    mf = s.export_factor()
    L = O.Layout(ns, nt, nd)
    for i in range(nt + (1 if nd else 0)):
        o = L.panel(mf, i)
        r = L.panel(g["mf"], i)
        low = np.tril(np.ones(o.shape, dtype=bool))
        assert np.max(np.abs(o[low] - r[low])) <= 1e-12 * np.max(np.abs(r[low]))
    ld = s.logDet()
    assert abs(ld - float(g["logdet"])) <= 1e-12 * abs(float(g["logdet"]))
    x = s.solve(np.empty_like(g["b"]), g["b"], nrhs)
    assert np.max(np.abs(x - g["x"])) <= 1e-10 * np.max(np.abs(g["x"]))
    res = s.residualNormNormalized(x, g["b"])
    assert res <= max(1e-13, 4 * float(g["resn"]))
    np.testing.assert_allclose(s.RGFdiag(), g["diag"], rtol=1e-10, atol=0)
    e = rgf.RGF(g["ia"], g["ja"], g["a"], ns, nt, nd, selinv="exact")
    np.testing.assert_allclose(e.RGFdiag(), g["diag_dense"], rtol=1e-10, atol=0)
    assert abs(e.logDet() - float(g["logdet_dense"])) <= 1e-12 * abs(float(g["logdet_dense"]))
