"""The allocation-free residual entry point against the handle-based one.

rgf_residual_norm_noalloc is for callers that cannot call cudaMalloc (a
framework allocator that owns the device memory, a serving loop that keeps
allocation and its device-wide synchronisation out of the steady state): it
takes device inputs and a device output and keeps its scratch in a fixed
device array.  This test drives it through the C ABI twice in a row and
checks each result against rgf_residual_norm on the same data.  It lives in
its own file, collected last, so that a failure here leaves every other test
already run.
"""
import ctypes as C

import numpy as np
import pytest

from rgf_gb300 import gen

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _noalloc_fn(lib):
    fn = lib.rgf_residual_norm_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_size_t] + [C.c_void_p] * 7
    return fn


def test_noalloc_residual_matches_handle_entry_point(rgf):
    torch = pytest.importorskip("torch")
    lib = rgf.load_library()
    fn = _noalloc_fn(lib)
    ns, nt, nd = 60, 5, 3
    n = ns * nt + nd
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=21)
    solver = rgf.RGF(ia, ja, a, ns, nt, nd, device=0)
    dev = torch.device("cuda", 0)
    d_ia = torch.from_numpy(ia.view(np.int64)).to(dev)
    d_ja = torch.from_numpy(ja.view(np.int64)).to(dev)
    d_a = torch.from_numpy(a).to(dev)
    d_out = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(5)
    for _ in range(2):  # two calls in a row share the scratch array
        x = rng.standard_normal(n)
        b = rng.standard_normal(n)
        want = solver.residualNorm(x, b)
        want_normalized = solver.residualNormNormalized(x, b)
        d_x = torch.from_numpy(x).to(dev)
        d_b = torch.from_numpy(b).to(dev)
        torch.cuda.synchronize()
        st = fn(n, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_x.data_ptr(),
                d_b.data_ptr(), d_out.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.rgf_status_string(st)
        stream.synchronize()
        got, bnorm = d_out.cpu().numpy()
        assert abs(got - want) <= RTOL * want
        assert abs(got / bnorm - want_normalized) <= RTOL * want_normalized


def test_noalloc_rejects_sizes_beyond_the_limit(rgf):
    lib = rgf.load_library()
    fn = _noalloc_fn(lib)
    one = C.c_void_p(8)  # never dereferenced: the size check comes first
    assert fn((1 << 20) + 1, one, one, one, one, one, one, None) == 1
    assert fn(0, one, one, one, one, one, one, None) == 1
