"""The allocation-free residual entry point against the handle-based one.

rgf_residual_norm_noalloc is for callers that cannot call cudaMalloc (a
framework allocator that owns the device memory, a serving loop that keeps
allocation and its device-wide synchronisation out of the steady state): it
takes device inputs and a device output and keeps its scratch in a fixed
device array.  This test drives it through the C ABI twice in a row and
checks each result against rgf_residual_norm on the same data, checks that a
warm call leaves the device's free memory unchanged, and that a row index
outside the matrix is skipped and reported as NaN.  It lives in its own file,
collected last, so that a failure here leaves every other test already run.
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


def _device_csc(torch, ia, ja, a):
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(ia.view(np.int64)).to(dev),
            torch.from_numpy(ja.view(np.int64)).to(dev),
            torch.from_numpy(a).to(dev))


def test_noalloc_residual_matches_handle_entry_point(rgf):
    torch = pytest.importorskip("torch")
    lib = rgf.load_library()
    fn = _noalloc_fn(lib)
    ns, nt, nd = 60, 5, 3
    n = ns * nt + nd
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=21)
    solver = rgf.RGF(ia, ja, a, ns, nt, nd, device=0)
    dev = torch.device("cuda", 0)
    d_ia, d_ja, d_a = _device_csc(torch, ia, ja, a)
    d_out = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rng = np.random.default_rng(5)
    free_after = []
    for _ in range(2):  # two calls in a row share the scratch array
        x = rng.standard_normal(n)
        b = rng.standard_normal(n)
        want = solver.residualNorm(x, b)
        want_normalized = solver.residualNormNormalized(x, b)
        d_x = torch.from_numpy(x).to(dev)
        d_b = torch.from_numpy(b).to(dev)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        st = fn(n, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), d_x.data_ptr(),
                d_b.data_ptr(), d_out.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.rgf_status_string(st)
        stream.synchronize()
        free_after.append((free_before, torch.cuda.mem_get_info(dev)[0]))
        got, bnorm = d_out.cpu().numpy()
        assert abs(got - want) <= RTOL * want
        assert abs(got / bnorm - want_normalized) <= RTOL * want_normalized
    # the first call may load the module (and its array); the second allocates nothing
    assert free_after[1][0] == free_after[1][1], free_after


def test_noalloc_skips_row_indices_outside_the_matrix(rgf):
    torch = pytest.importorskip("torch")
    lib = rgf.load_library()
    fn = _noalloc_fn(lib)
    ns, nt, nd = 20, 3, 2
    n = ns * nt + nd
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=22)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    x = torch.ones(n, dtype=torch.float64, device=dev)
    b = torch.ones(n, dtype=torch.float64, device=dev)
    d_out = torch.zeros(2, dtype=torch.float64, device=dev)
    for bad_row in (n + 7, 0):  # past the last row; above the diagonal of the last column
        ja_bad = ja.copy()
        ja_bad[-1] = bad_row
        d_ia, d_ja, d_a = _device_csc(torch, ia, ja_bad, a)
        torch.cuda.synchronize()
        st = fn(n, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), x.data_ptr(), b.data_ptr(),
                d_out.data_ptr(), C.c_void_p(stream.cuda_stream))
        assert st == 0, lib.rgf_status_string(st)
        stream.synchronize()
        assert np.all(np.isnan(d_out.cpu().numpy()))
    # a valid call afterwards clears the flag
    d_ia, d_ja, d_a = _device_csc(torch, ia, ja, a)
    torch.cuda.synchronize()
    assert fn(n, d_ia.data_ptr(), d_ja.data_ptr(), d_a.data_ptr(), x.data_ptr(), b.data_ptr(),
              d_out.data_ptr(), C.c_void_p(stream.cuda_stream)) == 0
    stream.synchronize()
    assert np.all(np.isfinite(d_out.cpu().numpy()))


def test_noalloc_rejects_sizes_beyond_the_limit(rgf):
    lib = rgf.load_library()
    fn = _noalloc_fn(lib)
    one = C.c_void_p(8)  # never dereferenced: the size check comes first
    assert fn((1 << 20) + 1, one, one, one, one, one, one, None) == 1
    assert fn(0, one, one, one, one, one, one, None) == 1
