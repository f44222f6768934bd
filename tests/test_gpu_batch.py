"""Batches of uneven instances: every instance's result in the concurrent
batch graph is bitwise the result of the same instance alone, and matches
the oracle (FP64: logDet 1e-12, RGFdiag 1e-10; split: 1e-9 / 1e-8)."""
import numpy as np
import pytest

from oracle import rgf_oracle as O
from rgf_gb300 import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,ltol,dtol", [("fp64", 1e-12, 1e-10), ("split", 1e-9, 1e-8)])
def test_batch_matches_alone_and_oracle(rgf, precision, ltol, dtol):
    # reused device memory must not leak into results: allocate, fill and free
    # a large buffer first so later allocations start from non-zero memory
    torch = pytest.importorskip("torch")
    junk = torch.full((1 << 27,), 3.0e77, dtype=torch.float64, device="cuda")
    del junk
    torch.cuda.empty_cache()
    inst = gen.generate_batch(10, seed=7, ns_choices=(42, 64, 100, 130, 300), nt_range=(1, 5))
    b = rgf.RGFBatch(inst, precision=precision)
    ld, diags = b.run(concurrent=True)
    ld2, diags2 = b.run(concurrent=True)          # replay of the captured graph
    ld3, diags3 = b.run(concurrent=False)         # per-instance launches
    for i, (ia, ja, a, ns, nt, nd) in enumerate(inst):
        s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
        l1, d1 = s.logDet(), s.RGFdiag()
        assert ld[i] == l1 == ld2[i] == ld3[i]
        assert np.array_equal(diags[i], d1) and np.array_equal(diags2[i], d1)
        assert np.array_equal(diags3[i], d1)
        ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
        assert abs(ld[i] - ref["logdet"]) <= ltol * abs(ref["logdet"])
        assert np.max(np.abs(diags[i] - ref["diag"]) / np.abs(ref["diag"])) <= dtol
    assert b.kernels() > 0


@pytest.mark.parametrize("precision,ltol,dtol", [("fp64", 1e-12, 1e-10), ("split", 1e-9, 1e-8)])
def test_batch_workload_classes_vs_oracle(rgf, precision, ltol, dtol):
    """One instance of every (ns, nd) class of the batched workload
    (ns in {42, 128, 256, 512}, nd in {0, 2, 6}, nt drawn from [3, 60], seed 4)
    in one batch graph: each equals the instance alone, bitwise, and matches
    the oracle."""
    rng = np.random.default_rng(4)
    inst = []
    for ns in (42, 128, 256, 512):
        for nd in (0, 2, 6):
            nt = int(rng.integers(3, 61))
            ia, ja, a = gen.generate_bta(ns, nt, nd, 400 + len(inst))
            inst.append((ia, ja, a, ns, nt, nd))
    b = rgf.RGFBatch(inst, precision=precision)
    b.run(concurrent=True)
    ld, diags = b.run(concurrent=True)  # replay of the captured graph
    for i, (ia, ja, a, ns, nt, nd) in enumerate(inst):
        s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
        assert ld[i] == s.logDet()
        assert np.array_equal(diags[i], s.RGFdiag())
        s.close()
        ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
        assert abs(ld[i] - ref["logdet"]) <= ltol * abs(ref["logdet"]), (ns, nt, nd)
        assert np.max(np.abs(diags[i] - ref["diag"]) / np.abs(ref["diag"])) <= dtol, (ns, nt, nd)
    b.close()
