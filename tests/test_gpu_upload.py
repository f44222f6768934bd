"""Asynchronous upload (rgf_opts.async_upload, the Python default, for
page-locked arrays): create queues the CSC copy and the ingest of each block
column and returns; the first factorization waits for each block column just
before using it.  Every result
must be bitwise that of the synchronous upload -- the first (direct) run, the
captured second run and its replay, which ingest from the device CSC -- except
split-precision solves, whose FP64 refinement residual sums with atomics
(1e-13 relative)."""
import numpy as np
import pytest

from rgf_gb300 import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("shape", [(300, 6, 4), (257, 3, 0), (64, 1, 5), (520, 4, 4)])
def test_async_upload_equals_sync(rgf, pinned, precision, shape):
    ns, nt, nd = shape
    n = ns * nt + nd
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=41)
    b = gen.random_rhs(n, 2, 41)
    out = {}
    for mode in (False, True):
        arrays = pinned(ia, ja, a) if mode else (ia, ja, a)
        s = rgf.RGF(*arrays, ns, nt, nd, precision=precision, async_upload=mode)
        ld = s.logDet()
        d = s.RGFdiag()
        x = s.solve(np.empty_like(b, order="F"), b, 2)
        lds = [ld]
        for _ in range(2):  # captured, then replayed
            s.factorize()
            lds.append(s.logDet())
        out[mode] = (lds, d, x)
        s.close()
    (l0, d0, x0), (l1, d1, x1) = out[False], out[True]
    assert len(set(l0 + l1)) == 1, (l0, l1)
    assert np.array_equal(d0, d1)
    if precision == "fp64":
        assert np.array_equal(x0, x1)
    else:
        assert np.max(np.abs(x0 - x1)) <= 1e-13 * np.max(np.abs(x0))


def test_residual_norm_before_factorize(rgf, pinned):
    """A call that reads the device CSC before any factorization waits for
    the upload (the residual of x = 0 is ||b||)."""
    ns, nt, nd = 400, 8, 3
    n = ns * nt + nd
    ia, ja, a = pinned(*gen.generate_bta(ns, nt, nd, seed=43))
    b = gen.random_rhs(n, 1, 43)[:, 0]
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    r = s.residualNorm(np.zeros(n), b)
    assert abs(r - np.linalg.norm(b)) <= 1e-14 * np.linalg.norm(b)
    s.close()


def test_destroy_with_upload_in_flight(rgf, pinned):
    """Destroying a handle right after an asynchronous create waits for its
    copies before freeing; later handles are unaffected."""
    ns, nt, nd = 500, 20, 3
    ia, ja, a = pinned(*gen.generate_bta(ns, nt, nd, seed=44))
    for _ in range(3):
        rgf.RGF(ia, ja, a, ns, nt, nd).close()
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    t = rgf.RGF(ia, ja, a, ns, nt, nd, async_upload=False)
    assert s.logDet() == t.logDet()
    s.close()
    t.close()
