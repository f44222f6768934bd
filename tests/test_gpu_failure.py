"""Failure detection without a GPU fault.

* A bounded device wait that runs out: the leaf Cholesky's wait for the
  previous pivot is given a one-poll limit (rgf_set_wait_limit), so a column
  that is not ready at once makes the leaf give up.  The stage must return
  RGF_ETIMEOUT, and the same handle must then factorize correctly with the
  default limit.  (Only this wait is shortened: it holds no asynchronous
  copies.  The split GEMM's mbarrier waits are never made to run out.)
* A device allocation that fails: rgf_debug_fail_alloc_after makes the k-th
  allocation of the library fail; every construction that meets it must
  return RGF_ENOMEM and release what it had allocated, and construction works
  again once the injection is off.
Tolerances as in the parity tests (FP64: logDet 1e-12, RGFdiag 1e-10).
"""
import numpy as np
import pytest

from oracle import rgf_oracle as O
from rgf_gb300 import gen

pytestmark = pytest.mark.gpu

RGF_ENOMEM, RGF_ETIMEOUT = 2, 5


def test_leaf_wait_limit_times_out_and_handle_recovers(rgf):
    ns, nt, nd = 256, 3, 2
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=31)
    s = rgf.RGF(ia, ja, a, ns, nt, nd, device=0)
    s.set_wait_limit(1)
    with pytest.raises(rgf.RGFError) as e:
        s.factorize()
    assert e.value.status == RGF_ETIMEOUT
    s.set_wait_limit(0)
    s.factorize()
    ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
    ld = s.logDet()
    assert abs(ld - ref["logdet"]) <= 1e-12 * abs(ref["logdet"])
    d = s.RGFdiag()
    assert np.max(np.abs(d - ref["diag"]) / np.abs(ref["diag"])) <= 1e-10
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_failed_allocation_returns_enomem_and_releases(rgf, precision):
    torch = pytest.importorskip("torch")
    ns, nt, nd = 512, 3, 4
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=32)
    rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision, device=0).close()  # module loaded
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    failed = 0
    try:
        for k in range(64):
            rgf.debug_fail_alloc_after(k)
            try:
                s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision, device=0)
            except rgf.RGFError as e:
                assert e.status == RGF_ENOMEM, e
                failed += 1
                continue
            s.close()
            break
    finally:
        rgf.debug_fail_alloc_after(-1)
    assert failed >= 5  # several allocations met the injected failure
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info(0)[0]
    assert abs(free1 - free0) <= 8 << 20, (free0, free1)  # nothing leaked
    s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision, device=0)
    ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
    tol = 1e-12 if precision == "fp64" else 1e-9
    assert abs(s.logDet() - ref["logdet"]) <= tol * abs(ref["logdet"])
    s.close()


def test_launch_trace_records_every_launch(rgf, tmp_path, monkeypatch):
    """RGF_GB300_TRACE=<file>: stages run launch by launch and every launch
    leaves one CSV line (stage, index, stream, label, ms since the stage start),
    with completion times in order on each stream; the results are unchanged."""
    ns, nt, nd = 200, 3, 2
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=33)
    path = tmp_path / "trace.csv"
    monkeypatch.setenv("RGF_GB300_TRACE", str(path))
    s = rgf.RGF(ia, ja, a, ns, nt, nd, device=0)
    monkeypatch.delenv("RGF_GB300_TRACE")
    ld = s.logDet()
    s.close()
    rows = [ln.split(",") for ln in path.read_text().splitlines()]
    # (the first factorization finds A already ingested by create: no "ingest")
    assert len(rows) > 20 and {r[3] for r in rows} >= {"leaf", "block end"}
    for side in ("0", "1"):
        t = [float(r[4]) for r in rows if r[0] == "0" and r[2] == side]
        assert t == sorted(t)
    ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
    assert abs(ld - ref["logdet"]) <= 1e-12 * abs(ref["logdet"])
