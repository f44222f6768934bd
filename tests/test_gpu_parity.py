"""GPU parity: the sm_103a path through the C ABI against the CPU oracle.

Tolerances (plain FP64): logDet relative error <= 1e-12, RGFdiag max
relative error <= 1e-10, normalized solve residual <= 1e-13, factor entries
within 1e-11 relative to the block's largest entry.
"""
import numpy as np
import pytest

from oracle import rgf_oracle as O
from rgf_gb300 import gen

pytestmark = pytest.mark.gpu

LOGDET_TOL = 1e-12
DIAG_TOL = 1e-10
RES_TOL = 1e-13

SHAPES = [
    (3, 3, 2), (5, 4, 1), (8, 1, 3), (6, 2, 7), (16, 5, 0), (7, 1, 0), (1, 5, 1),
    (64, 3, 2), (65, 3, 2), (100, 4, 6), (130, 3, 0), (200, 6, 4), (129, 2, 70),
]


def _run(rgf, ns, nt, nd, seed, selinv="exact", nrhs=2, spde=None, use_graphs=True):
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed, spde_grid=spde)
    n = ns * nt + nd
    b = gen.random_rhs(n, nrhs, seed)
    s = rgf.RGF(ia, ja, a, ns, nt, nd, selinv=selinv, use_graphs=use_graphs)
    s.factorize()
    out = {"logdet": s.logDet(), "x": s.solve(np.empty_like(b), b, nrhs),
           "diag": s.RGFdiag(), "MF": s.export_factor(), "solver": s,
           "ia": ia, "ja": ja, "a": a, "b": b}
    return out


def _rel(x, y):
    return float(np.max(np.abs(x - y) / np.maximum(np.abs(y), 1e-300)))


@pytest.mark.parametrize("ns,nt,nd", SHAPES)
def test_parity_generated(rgf, ns, nt, nd):
    r = _run(rgf, ns, nt, nd, seed=1)
    ref = O.run_all(ns, nt, nd, r["ia"], r["ja"], r["a"], b=r["b"], exact=True)
    assert abs(r["logdet"] - ref["logdet"]) <= LOGDET_TOL * abs(ref["logdet"])
    assert _rel(r["diag"], ref["diag"]) <= DIAG_TOL
    assert np.max(np.abs(r["x"] - ref["x"])) <= 1e-10 * np.max(np.abs(ref["x"]))
    L = O.Layout(ns, nt, nd)
    for i in range(nt + (1 if nd else 0)):
        g = L.panel(r["MF"], i)
        o = L.panel(ref["MF"], i)
        c = g.shape[1]
        lower = np.tril(np.ones((g.shape[0], c), dtype=bool))
        scale = np.max(np.abs(o[lower]))
        assert np.max(np.abs(g[lower] - o[lower])) <= 1e-11 * scale
        assert np.all(g[~lower] == 0.0)
    res = r["solver"].residualNormNormalized(r["x"], r["b"])
    assert res <= RES_TOL
    ref_res = O.residual_norm_normalized(r["ia"], r["ja"], r["a"], r["x"][:, 0], r["b"][:, 0])
    # both are rounding-level numbers; they must agree to well below the gate
    assert abs(res - ref_res) <= 1e-14


@pytest.mark.parametrize("ns,nt,nd", [(3, 3, 2), (50, 4, 3), (100, 3, 0), (64, 5, 6)])
def test_compat_selinv_matches_reference_recursion(rgf, ns, nt, nd):
    r = _run(rgf, ns, nt, nd, seed=2, selinv="compat")
    L = O.Layout(ns, nt, nd)
    MF = O.ingest(L, r["ia"], r["ja"], r["a"])
    O.factorize(L, MF)
    ref = O.selinv_compat(L, MF)
    assert _rel(r["diag"], ref) <= DIAG_TOL


@pytest.mark.parametrize("ns,nt,nd", [(40, 4, 3), (100, 3, 2)])
def test_exact_selinv_blocks(rgf, ns, nt, nd):
    ia, ja, a = gen.generate_bta(ns, nt, nd, 3)
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    MS = s.export_selinv()
    dense = O.dense_reference(ia, ja, a)["inv"]
    L = O.Layout(ns, nt, nd)
    for i in range(nt):
        Q = L.panel(MS, i)
        np.testing.assert_allclose(Q[:ns], dense[i * ns:(i + 1) * ns, i * ns:(i + 1) * ns],
                                   rtol=0, atol=1e-12 * np.abs(dense).max())
        if i < nt - 1:
            np.testing.assert_allclose(Q[ns:2 * ns], dense[(i + 1) * ns:(i + 2) * ns,
                                                           i * ns:(i + 1) * ns],
                                       rtol=0, atol=1e-12 * np.abs(dense).max())
        if nd:
            ro = L.dense_row_offset(i)
            np.testing.assert_allclose(Q[ro:ro + nd], dense[nt * ns:, i * ns:(i + 1) * ns],
                                       rtol=0, atol=1e-12 * np.abs(dense).max())
    if nd:
        np.testing.assert_allclose(L.panel(MS, nt), dense[nt * ns:, nt * ns:], rtol=1e-12)


def test_config_ns1000_nt50_nd4_spde(rgf):
    """The ns=1000, nt=50, nd=4 SPDE-like workload against the oracle."""
    ns, nt, nd = 1000, 50, 4
    r = _run(rgf, ns, nt, nd, seed=2, nrhs=8, spde=(40, 25))
    ref = O.run_all(ns, nt, nd, r["ia"], r["ja"], r["a"], b=r["b"], exact=True)
    assert abs(r["logdet"] - ref["logdet"]) <= LOGDET_TOL * abs(ref["logdet"])
    assert _rel(r["diag"], ref["diag"]) <= DIAG_TOL
    for q in range(8):
        res = O.residual_norm_normalized(r["ia"], r["ja"], r["a"], r["x"][:, q], r["b"][:, q])
        assert res <= RES_TOL


def test_repeat_is_bitwise_deterministic(rgf):
    ia, ja, a = gen.generate_bta(70, 5, 3, 7)
    s = rgf.RGF(ia, ja, a, 70, 5, 3)
    l1, d1 = s.logDet(), s.RGFdiag()
    s.factorize()
    l2, d2 = s.logDet(), s.RGFdiag()
    t = rgf.RGF(ia, ja, a, 70, 5, 3, use_graphs=False)
    l3, d3 = t.logDet(), t.RGFdiag()
    assert l1 == l2 == l3
    assert np.array_equal(d1, d2) and np.array_equal(d1, d3)


@pytest.mark.parametrize("nrhs", [1, 3, 16])
def test_solve_nrhs(rgf, nrhs):
    ns, nt, nd = 90, 4, 5
    ia, ja, a = gen.generate_bta(ns, nt, nd, 11)
    n = ns * nt + nd
    b = gen.random_rhs(n, nrhs, 11)
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    x = s.solve(np.empty_like(b), b, nrhs)
    A = O.to_dense(ia, ja, a)
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=0, atol=1e-12)
    # in-place form solve(b, nrhs) (RGF.H:550-554)
    bb = b.copy(order="F")
    s.solve(bb, None, nrhs)
    np.testing.assert_array_equal(bb, x)


def test_not_spd_reports_column(rgf):
    ns, nt, nd = 20, 3, 2
    ia, ja, a = gen.generate_bta(ns, nt, nd, 5)
    # make diagonal entry of global column 27 negative
    col = 27
    a = a.copy()
    a[int(ia[col])] = -50.0
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    with pytest.raises(rgf.RGFError) as e:
        s.factorize()
    assert e.value.status == 3
    assert s.info()["not_spd_column"] == col


@pytest.mark.parametrize("async_upload", [False, True])
def test_pattern_violation_rejected(rgf, pinned, async_upload):
    ns, nt, nd = 10, 4, 2
    ia, ja, a = gen.generate_bta(ns, nt, nd, 5)
    ja = ja.copy()
    # column 0 row entry moved into block 2 (outside the tridiagonal pattern)
    ja[int(ia[1]) - 1 - nd] = 2 * ns + 1
    # pageable arrays: validated before the constructor returns (an
    # asynchronous upload asked for them is done at once: nothing to overlap)
    try:
        s = rgf.RGF(ia, ja, a, ns, nt, nd, async_upload=async_upload)
    except rgf.RGFError as e:
        assert e.status == 1
    else:  # only an asynchronous upload may defer the check
        assert async_upload
        with pytest.raises(rgf.RGFError) as e:
            s.factorize()
        assert e.value.status == 1
        s.close()
    if not async_upload:
        return
    # asynchronous upload of page-locked arrays: the first call that
    # factorizes reports it, and so does every later one (the pattern is
    # ingested again)
    ia, ja, a = pinned(ia, ja, a)
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    for _ in range(2):
        with pytest.raises(rgf.RGFError) as e:
            s.factorize()
        assert e.value.status == 1
    s.close()
    s = rgf.RGF(ia, ja, a, ns, nt, nd)  # residualNorm first: it waits for the upload
    with pytest.raises(rgf.RGFError) as e:
        s.residualNorm(np.ones(s.n), np.ones(s.n))
    assert e.value.status == 1
    with pytest.raises(rgf.RGFError) as e:
        s.logDet()
    assert e.value.status == 1
    s.close()
