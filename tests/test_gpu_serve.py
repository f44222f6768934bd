"""Request loop: results in a concurrent mix equal the same work done alone.

Factorizations, solves and RGFdiag requests on several resident factors are
submitted together so that they overlap on the GPU; every result must be
bitwise what a fresh instance computes alone (the kernels are deterministic
and independent of what else runs) -- except split-precision solves, whose
FP64 refinement residual sums with atomics: those agree to 1e-13 relative.  Eviction: a budget that holds one
factor evicts the older one, and a request for it fails cleanly.
"""
import numpy as np
import pytest

from rgf_gb300 import gen

pytestmark = pytest.mark.gpu

SHAPES = [(64, 4, 2), (130, 3, 0), (257, 2, 6), (100, 5, 3), (300, 3, 4), (42, 6, 1)]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_results_in_the_mix_equal_alone(rgf, precision):
    mats = [gen.generate_bta(ns, nt, nd, seed=30 + i) for i, (ns, nt, nd) in enumerate(SHAPES)]
    srv = rgf.RGFServer(hbm_budget_bytes=8 << 30, slots=4, precision=precision)
    tickets = [srv.submit_factor(*m, *sh) for m, sh in zip(mats, SHAPES)]
    res = [srv.wait(t) for t in tickets]
    assert all(r["status"] == 0 for r in res)
    fids = [r["factor_id"] for r in res]
    # a second wave: solves and diags on every factor, plus new factorizations
    rng = np.random.default_rng(3)
    jobs = []
    for i, (ns, nt, nd) in enumerate(SHAPES):
        n = ns * nt + nd
        b = rng.standard_normal((n, 1 + i % 3))
        jobs.append(("solve", i, b, srv.submit_solve(fids[i], b)))
        jobs.append(("diag", i, None, srv.submit_diag(fids[i], n)))
        jobs.append(("factor", i, None, srv.submit_factor(*mats[i], *SHAPES[i])))
    done = {t: srv.wait(t) for (_, _, _, t) in jobs}
    for kind, i, b, t in jobs:
        r = done[t]
        assert r["status"] == 0, (kind, i, r["status"])
        ns, nt, nd = SHAPES[i]
        alone = rgf.RGF(*mats[i], ns, nt, nd, precision=precision)
        if kind == "solve":
            x = alone.solve(np.empty_like(b, order="F"), b, b.shape[1])
            if precision == "fp64":
                assert np.array_equal(r["x"], x)
            else:
                assert np.max(np.abs(r["x"] - x)) <= 1e-13 * np.max(np.abs(x))
        elif kind == "diag":
            assert np.array_equal(r["diag"], alone.RGFdiag())
        else:
            assert r["logdet"] == alone.logDet() == res[i]["logdet"]
        alone.close()
    st = srv.stats()
    assert st["completed"] == st["submitted"] == len(SHAPES) + len(jobs)
    # every handle's device memory came from the pre-reserved arena
    assert st["arena_bytes"] == 8 << 30 and st["arena_fallbacks"] == 0
    srv.close()


def test_eviction_and_release(rgf):
    ns, nt, nd = 200, 3, 2
    m1 = gen.generate_bta(ns, nt, nd, seed=1)
    m2 = gen.generate_bta(ns, nt, nd, seed=2)
    # a budget for one factor only
    srv = rgf.RGFServer(hbm_budget_bytes=30 << 20, slots=2)
    f1 = srv.wait(srv.submit_factor(*m1, ns, nt, nd))
    assert f1["status"] == 0
    f2 = srv.wait(srv.submit_factor(*m2, ns, nt, nd))
    assert f2["status"] == 0
    assert srv.stats()["evicted"] == 1
    gone = srv.wait(srv.submit_diag(f1["factor_id"], ns * nt + nd))
    assert gone["status"] == 1          # RGF_EINVAL: evicted
    ok = srv.wait(srv.submit_diag(f2["factor_id"], ns * nt + nd))
    assert ok["status"] == 0
    rel = srv.wait(srv.submit_release(f2["factor_id"]))
    assert rel["status"] == 0 and srv.stats()["resident_factors"] == 0
    # eviction and release gave the memory back to the arena (no cudaFree)
    assert srv.stats()["arena_in_use"] == 0
    srv.close()


def test_queued_request_keeps_its_factor_resident(rgf):
    """A diag queued on a factor pins it: a factorization that needs its memory
    waits until the diag has run, then evicts it."""
    ns, nt, nd = 200, 3, 2
    m1 = gen.generate_bta(ns, nt, nd, seed=1)
    m2 = gen.generate_bta(ns, nt, nd, seed=2)
    srv = rgf.RGFServer(hbm_budget_bytes=30 << 20, slots=2)
    f1 = srv.wait(srv.submit_factor(*m1, ns, nt, nd))
    assert f1["status"] == 0
    td = [srv.submit_diag(f1["factor_id"], ns * nt + nd) for _ in range(3)]
    tf = srv.submit_factor(*m2, ns, nt, nd)
    diags = [srv.wait(t) for t in td]
    f2 = srv.wait(tf)
    assert all(d["status"] == 0 for d in diags) and f2["status"] == 0
    assert srv.stats()["evicted"] == 1
    alone = rgf.RGF(*m1, ns, nt, nd)
    assert np.array_equal(diags[0]["diag"], alone.RGFdiag())
    alone.close()
    srv.close()
