"""Device-memory cache (rgf_set_device_cache): handles of one shape created
and destroyed in a loop get their buffers back from the cache -- no new device
memory is taken after the first -- and compute exactly what a handle with
fresh memory computes, although the reused buffers hold the previous
handle's data."""
import numpy as np
import pytest

from rgf_gb300 import gen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_cache_reuses_buffers_and_results_match(rgf, precision):
    torch = pytest.importorskip("torch")
    ns, nt, nd = 512, 4, 3
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=45)
    ia2, ja2, a2 = gen.generate_bta(ns, nt, nd, seed=46)  # same shape, other values
    fresh = {}
    for key, (i, j, v) in {"m1": (ia, ja, a), "m2": (ia2, ja2, a2)}.items():
        s = rgf.RGF(i, j, v, ns, nt, nd, precision=precision)
        fresh[key] = (s.logDet(), s.RGFdiag())
        s.close()
    rgf.set_device_cache(8 << 30)
    try:
        s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
        s.logDet()
        s.RGFdiag()  # the same calls as below: every buffer of the loop exists once
        held_bytes = s.info()["device_bytes"]
        s.close()
        assert rgf.device_cache_bytes() >= held_bytes
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        for k in range(4):  # alternate the matrices: every buffer is reused dirty
            key, (i, j, v) = ("m1", (ia, ja, a)) if k % 2 else ("m2", (ia2, ja2, a2))
            s = rgf.RGF(i, j, v, ns, nt, nd, precision=precision)
            assert s.logDet() == fresh[key][0]
            assert np.array_equal(s.RGFdiag(), fresh[key][1])
            s.close()
        torch.cuda.synchronize()
        assert abs(torch.cuda.mem_get_info(0)[0] - free0) <= 8 << 20  # nothing new taken
        # another shape misses the cache and still computes correctly
        s = rgf.RGF(*gen.generate_bta(300, 3, 2, seed=47), 300, 3, 2, precision=precision)
        t = rgf.RGF(*gen.generate_bta(300, 3, 2, seed=47), 300, 3, 2, precision=precision)
        assert s.logDet() == t.logDet()
        s.close()
        t.close()
    finally:
        rgf.set_device_cache(0)
    assert rgf.device_cache_bytes() == 0
