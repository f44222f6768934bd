"""Host-side checks that need no GPU: the C ABI library loads and exports
every entry point include/rgf.h declares; the generator, .dat I/O and flop
counts behave as documented."""
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_entry_points():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(rgf_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    import ctypes
    import rgf_gb300
    lib = rgf_gb300.load_library()
    names = declared_entry_points()
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n
    # a status string call needs no device
    lib.rgf_status_string.restype = ctypes.c_char_p
    assert lib.rgf_status_string(3).startswith(b"RGF_ENOTSPD")


def test_missing_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import rgf_gb300
    from rgf_gb300 import gen
    ia, ja, a = gen.generate_bta(3, 3, 2, 1)
    with pytest.raises(rgf_gb300.RGFError) as e:
        rgf_gb300.RGF(ia, ja, a, 3, 3, 2)
    assert e.value.status == 4


def test_generator_is_seeded_and_spd():
    from oracle import rgf_oracle as O
    from rgf_gb300 import gen
    a1 = gen.generate_bta(6, 4, 2, 9)
    a2 = gen.generate_bta(6, 4, 2, 9)
    for x, y in zip(a1, a2):
        assert np.array_equal(x, y)
    ia, ja, a = a1
    assert len(ja) == gen.bta_nnz(6, 4, 2)
    A = O.to_dense(ia, ja, a)
    assert np.all(np.linalg.eigvalsh(A) > 0)
    # lower CSC, sorted rows, diagonal first
    for c in range(len(ia) - 1):
        rows = ja[ia[c]:ia[c + 1]].astype(int)
        assert rows[0] == c and np.all(np.diff(rows) > 0)


def test_dat_round_trip(tmp_path):
    from rgf_gb300 import gen
    ia, ja, a = gen.generate_bta(4, 3, 1, 2)
    p = tmp_path / "m.dat"
    gen.write_dat(p, ia, ja, a)
    n, ia2, ja2, a2 = gen.read_dat(p)
    assert n == len(ia) - 1
    assert np.array_equal(ia, ia2) and np.array_equal(ja, ja2) and np.array_equal(a, a2)


def test_flop_contract():
    from rgf_gb300.flops import algorithmic_flops
    f = algorithmic_flops(2000, 100, 6)
    assert abs(f["factor"] - 1.858e12) / 1.858e12 < 1e-3
    assert abs(f["selinv"] - 5.049e12) / 5.049e12 < 1e-3
    f = algorithmic_flops(1000, 50, 4)
    assert abs(f["total"] - 4.292e11) / 4.292e11 < 1e-3


def test_tuning_entry_points_reject_null_handles():
    import ctypes
    import rgf_gb300
    lib = rgf_gb300.load_library()
    t = rgf_gb300._Tuning()
    n = ctypes.c_size_t()
    assert lib.rgf_get_tuning(None, ctypes.byref(t)) == 1
    assert lib.rgf_set_tuning(None, ctypes.byref(t)) == 1
    assert lib.rgf_autotune(None, 0, None) == 1
    assert lib.rgf_batch_autotune(None, 0, ctypes.byref(n)) == 1


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every struct the Python mirror passes through the C ABI has the size
    and field offsets the C compiler gives it."""
    import ctypes
    import shutil
    import subprocess
    import rgf_gb300
    if shutil.which("gcc") is None:
        pytest.skip("gcc not present")
    structs = {"rgf_opts": rgf_gb300._Opts, "rgf_info_t": rgf_gb300._Info,
               "rgf_request": rgf_gb300._Request, "rgf_server_stats_t": rgf_gb300._ServerStats,
               "rgf_tuning": rgf_gb300._Tuning}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rgf.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n"):
        if ln:
            c, f, v = ln.split()
            got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])


def test_opts_struct_layout_matches_the_header():
    """rgf_default_opts writes exactly the 16 ints of rgf_opts (precision,
    slices, selinv_mode, device, use_graphs, fp64_diag, async_upload, 9
    reserved), which the ctypes mirror declares in the same order."""
    import ctypes
    import rgf_gb300
    lib = rgf_gb300.load_library()
    assert ctypes.sizeof(rgf_gb300._Opts) == 16 * 4
    buf = (ctypes.c_ubyte * 128)(*([0xAB] * 128))
    assert lib.rgf_default_opts(ctypes.cast(buf, ctypes.POINTER(rgf_gb300._Opts))) == 0
    assert bytes(buf[64:]) == b"\xab" * 64  # nothing written past the struct
    o = rgf_gb300._Opts.from_buffer_copy(bytes(buf[:64]))
    assert (o.precision, o.slices, o.selinv_mode, o.device, o.use_graphs, o.fp64_diag,
            o.async_upload) == (0, 0, 0, -1, 1, 1, 0)


def test_device_cache_api_needs_no_device():
    import rgf_gb300
    rgf_gb300.set_device_cache(1 << 20)
    assert rgf_gb300.device_cache_bytes() == 0  # nothing freed into it yet
    rgf_gb300.set_device_cache(0)
    assert rgf_gb300.device_cache_bytes() == 0
