"""Tuning knobs and the autotuner.  Every knob setting (leaf width, look-ahead
stream, split/FP64 routing bias) gives the oracle's results within the
precision's tolerance (FP64: logDet 1e-12, RGFdiag 1e-10; split: 1e-9 /
1e-8); an autotuned batch is bitwise the same instances run alone with the
same knobs; the process-wide cache returns the same choice; a failed tuning
run leaves the knobs as they were."""
import numpy as np
import pytest

from oracle import rgf_oracle as O
from rgf_gb300 import gen

pytestmark = pytest.mark.gpu

KNOBS = ("leaf_nb", "lookahead", "split_bias", "splitk_max", "fp64_tile")


def _knobs(t):
    return tuple(t[k] for k in KNOBS)


@pytest.mark.parametrize("precision,ns,nt,nd,ltol,dtol", [
    ("fp64", 70, 3, 4, 1e-12, 1e-10),
    ("split", 300, 3, 4, 1e-9, 1e-8),
])
def test_every_knob_setting_matches_the_oracle(rgf, precision, ns, nt, nd, ltol, dtol):
    ia, ja, a = gen.generate_bta(ns, nt, nd, 11)
    ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
    s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
    # split precision cuts its FP64 products into 32 x 32 tiles by default
    assert _knobs(s.tuning()) == (32, 1, 1.0, 0, 32 if precision == "split" else 0)
    biases = (0.5, 1.0, 2.0) if precision == "split" else (1.0,)
    for nb in (16, 32, 64):
        for la in (0, 1):
            for bias in biases:
                s.set_tuning(nb, la, bias)
                assert _knobs(s.tuning()) == (nb, la, bias, 0, 0)
                for _ in range(2):  # a direct run, then the captured graph
                    s.factorize()
                    ld, d = s.logDet(), s.RGFdiag()
                    assert abs(ld - ref["logdet"]) <= ltol * abs(ref["logdet"]), (nb, la, bias)
                    assert np.max(np.abs(d - ref["diag"]) / np.abs(ref["diag"])) <= dtol, \
                        (nb, la, bias)


@pytest.mark.parametrize("precision,ltol,dtol", [("fp64", 1e-12, 1e-10), ("split", 1e-9, 1e-8)])
def test_tile_shape_knobs_match_the_oracle(rgf, precision, ltol, dtol):
    """The autotuner's tile-shape knobs (split-K degree of the tensor-core
    products, FP64 output tile) change how products are cut into CTAs (and,
    through the cost model, which engine runs a product), never the results
    beyond the precision's tolerance."""
    ns, nt, nd = 520, 3, 4
    ia, ja, a = gen.generate_bta(ns, nt, nd, seed=41)
    ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
    s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
    for splitk in (1, 4, 0):
        for tile in (0, 32, 64):
            s.set_tuning(32, 1, 1.0, splitk, tile)
            for _ in range(2):  # a direct run, then the captured graph
                s.factorize()
                ld, d = s.logDet(), s.RGFdiag()
                assert abs(ld - ref["logdet"]) <= ltol * abs(ref["logdet"])
                assert np.max(np.abs(d - ref["diag"]) / np.abs(ref["diag"])) <= dtol
    s.close()


def test_invalid_knobs_rejected(rgf):
    ia, ja, a = gen.generate_bta(20, 2, 1, 3)
    s = rgf.RGF(ia, ja, a, 20, 2, 1)
    for bad in ((8, 1, 1.0), (48, 1, 1.0), (32, 2, 1.0), (32, 1, 0.0), (32, 1, 100.0),
                (32, 1, float("nan")), (32, 1, 1.0, 3, 0), (32, 1, 1.0, 0, 48)):
        with pytest.raises(rgf.RGFError) as e:
            s.set_tuning(*bad)
        assert e.value.status == 1
    assert _knobs(s.tuning()) == (32, 1, 1.0, 0, 0)


def test_autotune_single_instance_and_cache(rgf):
    ns, nt, nd = 96, 4, 2
    ia, ja, a = gen.generate_bta(ns, nt, nd, 21)
    ref = O.run_all(ns, nt, nd, ia, ja, a, exact=True)
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    t = s.autotune(force=True)
    assert t["leaf_nb"] in (16, 32, 64) and t["lookahead"] in (0, 1)
    assert t["split_bias"] == 1.0          # FP64 has no routing to tune
    assert t["ms"] > 0
    assert s.tuning() == t
    ld, d = s.logDet(), s.RGFdiag()
    assert abs(ld - ref["logdet"]) <= 1e-12 * abs(ref["logdet"])
    assert np.max(np.abs(d - ref["diag"]) / np.abs(ref["diag"])) <= 1e-10
    # another instance of the same class takes the cached choice
    ia2, ja2, a2 = gen.generate_bta(ns, nt + 3, nd, 22)
    s2 = rgf.RGF(ia2, ja2, a2, ns, nt + 3, nd)
    assert s2.autotune() == t


def test_failed_autotune_leaves_knobs(rgf):
    ns, nt, nd = 40, 3, 2
    ia, ja, a = gen.generate_bta(ns, nt, nd, 5)
    a = a.copy()
    a[int(ia[45])] = -50.0                  # column 45 is not positive definite
    s = rgf.RGF(ia, ja, a, ns, nt, nd)
    s.set_tuning(64, 0, 1.0)
    with pytest.raises(rgf.RGFError) as e:
        s.autotune(force=True)
    assert e.value.status == 3
    assert _knobs(s.tuning()) == (64, 0, 1.0, 0, 0)


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_autotuned_batch_is_bitwise_alone(rgf, precision):
    shapes = [(64, 3, 2), (64, 5, 2), (64, 4, 0), (300, 2, 2), (300, 3, 2), (130, 1, 3)]
    inst = [(*gen.generate_bta(ns, nt, nd, 30 + i), ns, nt, nd)
            for i, (ns, nt, nd) in enumerate(shapes)]
    b = rgf.RGFBatch(inst, precision=precision)
    b.run(concurrent=True, want_diag=False)        # captured with the default knobs
    b.run(concurrent=True, want_diag=False)
    assert b.autotune(force=True) == 4             # (64,2) (64,0) (300,2) (130,3)
    tun = b.tunings()
    assert _knobs(tun[0]) == _knobs(tun[1]) and _knobs(tun[3]) == _knobs(tun[4])
    assert all(t["ms"] > 0 for t in tun)
    # the untimed members of a class were set, not tuned: the cache gives the same
    assert b.autotune() == 4 and [_knobs(t) for t in b.tunings()] == [_knobs(t) for t in tun]
    ld, diags = b.run(concurrent=True)             # direct launches with the new knobs
    ld2, diags2 = b.run(concurrent=True)           # recaptured graph
    b.set_tuning(0, 16, 0, 2.0)                    # one member changes: the batch recaptures
    ld3, diags3 = b.run(concurrent=True)
    ld4, diags4 = b.run(concurrent=True)
    for i, (ia, ja, a, ns, nt, nd) in enumerate(inst):
        s = rgf.RGF(ia, ja, a, ns, nt, nd, precision=precision)
        s.set_tuning(*_knobs(tun[i]))
        l1, d1 = s.logDet(), s.RGFdiag()
        assert ld[i] == l1 == ld2[i]
        assert np.array_equal(diags[i], d1) and np.array_equal(diags2[i], d1)
        if i == 0:
            s.set_tuning(16, 0, 2.0)
            l1, d1 = s.logDet(), s.RGFdiag()
        assert ld3[i] == l1 == ld4[i]
        assert np.array_equal(diags3[i], d1) and np.array_equal(diags4[i], d1)
