"""rgf_gb300 -- GB300-native drop-in for the reference ``RGF<double>`` solver.

``RGF`` mirrors the public surface of the reference class (``RGF.H:11-80``):
construct with ``(ia, ja, a, ns, nt, nd)`` on the lower triangle of a
symmetric positive-definite block-tridiagonal-arrowhead matrix in CSC form,
then ``factorize``, ``logDet``, ``solve`` and ``RGFdiag``.  Every call goes
through the C ABI of ``librgf_gb300.so`` (``include/rgf.h``); all arithmetic
runs in hand-written sm_103a kernels.  There is no CPU fallback: without the
built library or a usable GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = ["RGF", "RGFBatch", "RGFServer", "RGFError", "load_library", "library_path",
           "STATUS"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

STATUS = {0: "RGF_OK", 1: "RGF_EINVAL", 2: "RGF_ENOMEM", 3: "RGF_ENOTSPD",
          4: "RGF_ECUDA", 5: "RGF_ETIMEOUT", 6: "RGF_ENOTSUP"}
PRECISION = {"fp64": 0, "split": 1}
SELINV = {"exact": 0, "compat": 1}


class RGFError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, status: int, what: str):
        self.status = status
        msg = _LIB.rgf_status_string(status).decode() if _LIB is not None else STATUS.get(status)
        super().__init__(f"{what}: {msg}")


class _Opts(C.Structure):
    _fields_ = [("precision", C.c_int), ("slices", C.c_int), ("selinv_mode", C.c_int),
                ("device", C.c_int), ("use_graphs", C.c_int), ("fp64_diag", C.c_int),
                ("async_upload", C.c_int), ("reserved", C.c_int * 9)]


class _Info(C.Structure):
    _fields_ = [("n", C.c_size_t), ("nnz", C.c_size_t), ("mf_size", C.c_size_t),
                ("device_bytes", C.c_size_t), ("not_spd_column", C.c_int),
                ("reserved0", C.c_int), ("kernels_launched", C.c_longlong),
                ("reserved", C.c_int * 4)]


class _Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("status", C.c_int), ("factor_id", C.c_longlong),
                ("ia", C.c_void_p), ("ja", C.c_void_p), ("a", C.c_void_p),
                ("ns", C.c_size_t), ("nt", C.c_size_t), ("nd", C.c_size_t),
                ("b", C.c_void_p), ("x", C.c_void_p), ("nrhs", C.c_size_t),
                ("diag", C.c_void_p), ("logdet", C.c_double), ("latency_ms", C.c_double),
                ("reserved_bytes", C.c_size_t)]


class _Tuning(C.Structure):
    _fields_ = [("leaf_nb", C.c_int), ("lookahead", C.c_int), ("split_bias", C.c_double),
                ("ms", C.c_double), ("splitk_max", C.c_int), ("fp64_tile", C.c_int),
                ("reserved", C.c_int * 2)]


TUNE_FORCE = 1


def _tuning_dict(t: _Tuning) -> dict:
    return {"leaf_nb": t.leaf_nb, "lookahead": t.lookahead, "split_bias": t.split_bias,
            "splitk_max": t.splitk_max, "fp64_tile": t.fp64_tile, "ms": t.ms}


def _tuning_struct(leaf_nb: int, lookahead: int, split_bias: float, splitk_max: int = 0,
                   fp64_tile: int = 0) -> _Tuning:
    t = _Tuning()
    t.leaf_nb, t.lookahead, t.split_bias = int(leaf_nb), int(lookahead), float(split_bias)
    t.splitk_max, t.fp64_tile = int(splitk_max), int(fp64_tile)
    return t


class _ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong),
                ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("evicted", C.c_longlong), ("resident_factors", C.c_longlong),
                ("queued", C.c_longlong), ("used_bytes", C.c_size_t),
                ("arena_bytes", C.c_size_t), ("arena_in_use", C.c_size_t),
                ("arena_fallbacks", C.c_longlong)]


def library_path() -> str:
    return os.path.join(_HERE, "librgf_gb300.so")


_SIGS = {
    "rgf_status_string": (C.c_char_p, [C.c_int]),
    "rgf_default_opts": (C.c_int, [C.POINTER(_Opts)]),
    "rgf_create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t,
                             C.c_size_t, C.POINTER(_Opts), C.POINTER(C.c_void_p)]),
    "rgf_destroy": (C.c_int, [C.c_void_p]),
    "rgf_create_hermitian": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                       C.c_size_t, C.c_size_t, C.POINTER(_Opts),
                                       C.POINTER(C.c_void_p)]),
    "rgf_hermitian_embed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t,
                                      C.c_size_t, C.c_size_t, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.POINTER(C.c_size_t)]),
    "rgf_factorize": (C.c_int, [C.c_void_p]),
    "rgf_logdet": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "rgf_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t]),
    "rgf_diag": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgf_residual_norm": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]),
    "rgf_residual_norm_normalized": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.POINTER(C.c_double)]),
    "rgf_export_factor": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgf_export_selinv": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgf_get_info": (C.c_int, [C.c_void_p, C.POINTER(_Info)]),
    "rgf_diag_device": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "rgf_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "rgf_kernel_timer_enable": (C.c_int, [C.c_void_p, C.c_int]),
    "rgf_measure_fp64_peak": (C.c_int, [C.POINTER(C.c_double)]),
    "rgf_batch_create": (C.c_int, [C.c_size_t, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.POINTER(_Opts),
                                   C.POINTER(C.c_void_p)]),
    "rgf_batch_destroy": (C.c_int, [C.c_void_p]),
    "rgf_batch_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_size_t)]),
    "rgf_batch_handle": (C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]),
    "rgf_batch_get_stream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "rgf_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "rgf_batch_kernels": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "rgf_server_create": (C.c_int, [C.POINTER(_Opts), C.c_size_t, C.c_int, C.POINTER(C.c_void_p)]),
    "rgf_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong)]),
    "rgf_server_wait": (C.c_int, [C.c_void_p, C.c_longlong, C.c_double, C.POINTER(C.c_int)]),
    "rgf_server_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgf_server_destroy": (C.c_int, [C.c_void_p]),
    "rgf_dgemm_device": (C.c_int, [C.c_int, C.c_int, C.c_char, C.c_char, C.c_int, C.c_int,
                                   C.c_int, C.c_double, C.c_void_p, C.c_int, C.c_void_p,
                                   C.c_int, C.c_double, C.c_void_p, C.c_int, C.c_void_p]),
    "rgf_kernel_timer_read": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "rgf_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(_Tuning)]),
    "rgf_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(_Tuning)]),
    "rgf_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(_Tuning)]),
    "rgf_batch_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_size_t)]),
    "rgf_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int]),
    "rgf_debug_fail_alloc_after": (C.c_int, [C.c_longlong]),
    "rgf_set_device_cache": (C.c_int, [C.c_size_t]),
    "rgf_device_cache_bytes": (C.c_int, [C.POINTER(C.c_size_t)]),
    "rgf_residual_norm_noalloc": (C.c_int, [C.c_size_t] + [C.c_void_p] * 7),
}


def load_library(path: str | None = None):
    """Load librgf_gb300.so (built by ``rgf_gb300.build``); raise if absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or library_path()
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is not built: run `python -m rgf_gb300.build` "
                           "(requires nvcc); there is no CPU fallback")
    lib = C.CDLL(p)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def hermitian_embed(ia, ja, a, ns: int, nt: int, nd: int):
    """Lower CSC (ia2, ja2, a2) of the real symmetric embedding that a
    Hermitian instance factors: [[X, -Y], [Y, X]] for A = X + iY, unknowns
    ordered per block (Re then Im of each block, then of the arrowhead), a BTA
    matrix with (2ns, nt, 2nd).  Host only."""
    lib = load_library()
    ia = np.ascontiguousarray(ia, dtype=np.uint64)
    ja = np.ascontiguousarray(ja, dtype=np.uint64)
    a = np.ascontiguousarray(a, dtype=np.complex128)
    nnz2 = C.c_size_t()
    _check(lib.rgf_hermitian_embed(_ptr(ia), _ptr(ja), _ptr(a), ns, nt, nd, None, None, None,
                                   C.byref(nnz2)), "rgf_hermitian_embed")
    n2 = 2 * (ns * nt + nd)
    ia2 = np.empty(n2 + 1, dtype=np.uint64)
    ja2 = np.empty(nnz2.value, dtype=np.uint64)
    a2 = np.empty(nnz2.value, dtype=np.float64)
    _check(lib.rgf_hermitian_embed(_ptr(ia), _ptr(ja), _ptr(a), ns, nt, nd, _ptr(ia2), _ptr(ja2),
                                   _ptr(a2), C.byref(nnz2)), "rgf_hermitian_embed")
    return ia2, ja2, a2


def debug_fail_alloc_after(after: int) -> None:
    """Failure injection for tests: the next ``after`` device allocations of
    the library succeed and the one after fails (RGF_ENOMEM); -1 turns it off."""
    _check(load_library().rgf_debug_fail_alloc_after(int(after)), "rgf_debug_fail_alloc_after")


def set_device_cache(max_bytes: int) -> None:
    """Keep freed device buffers (up to ``max_bytes``) for later handles of the
    same shape, so that create / destroy in a loop pay no cudaMalloc / cudaFree;
    0 (the default) returns every cached buffer to the driver."""
    _check(load_library().rgf_set_device_cache(int(max_bytes)), "rgf_set_device_cache")


def device_cache_bytes() -> int:
    """Bytes of device memory the cache holds (buffers not in use)."""
    out = C.c_size_t()
    _check(load_library().rgf_device_cache_bytes(C.byref(out)), "rgf_device_cache_bytes")
    return out.value


def measure_fp64_peak() -> float:
    """FP64 (DMMA) TFLOP/s of the current GPU, measured by the library."""
    lib = load_library()
    out = C.c_double()
    _check(lib.rgf_measure_fp64_peak(C.byref(out)), "rgf_measure_fp64_peak")
    return out.value


def dgemm_device(precision: str, transa: str, transb: str, m: int, n: int, k: int,
                 alpha: float, A_ptr: int, lda: int, B_ptr: int, ldb: int, beta: float,
                 C_ptr: int, ldc: int, stream: int = 0, slices: int = 0) -> None:
    """C := alpha op(A) op(B) + beta C on device pointers (column-major)."""
    lib = load_library()
    _check(lib.rgf_dgemm_device(PRECISION[precision], int(slices), transa.encode(),
                                transb.encode(), m, n, k, alpha, C.c_void_p(A_ptr), lda,
                                C.c_void_p(B_ptr), ldb, beta, C.c_void_p(C_ptr), ldc,
                                C.c_void_p(stream)), "rgf_dgemm_device")


def _tuning_of(lib, h) -> dict:
    t = _Tuning()
    _check(lib.rgf_get_tuning(h, C.byref(t)), "rgf_get_tuning")
    return _tuning_dict(t)


def _check(status: int, what: str) -> None:
    if status != 0:
        raise RGFError(status, what)


def _ptr(arr: np.ndarray) -> C.c_void_p:
    return C.c_void_p(arr.ctypes.data)


class RGF:
    """Drop-in for the reference class ``RGF<double>`` (``RGF.H:11-80``).

    ``ia``/``ja`` are the column pointers and row indices (``size_t``) and
    ``a`` the values of the matrix's lower triangle in CSC form.  With
    ``async_upload`` (the default) and page-locked arrays (e.g. from
    ``torch.Tensor.pin_memory``) the copy to the device overlaps the first
    factorization: the object keeps the arrays, as the reference keeps the
    pointers (RGF.H:87-89), and they must not be changed until the first
    factorize / logDet / RGFdiag / solve / residualNorm returns, which also
    reports a CSC outside the block pattern.  ``async_upload=False`` copies
    and validates them before the constructor returns.  A complex
    ``a`` makes a Hermitian instance (``RGF<complex<double>>``, RGF.H:756-774):
    logDet is then log det A and solve / RGFdiag take and return complex arrays.
    """

    def __init__(self, ia, ja, a, ns: int, nt: int, nd: int, precision: str = "fp64",
                 slices: int = 0, selinv: str = "exact", device: int = -1,
                 use_graphs: bool = True, fp64_diag=1, async_upload: bool = True):
        lib = load_library()
        self._lib = lib
        self._h = C.c_void_p()
        self.ns, self.nt, self.nd = int(ns), int(nt), int(nd)
        self.n = self.ns * self.nt + self.nd
        self._ia = np.ascontiguousarray(ia, dtype=np.uint64)
        self._ja = np.ascontiguousarray(ja, dtype=np.uint64)
        self.hermitian = np.iscomplexobj(a)
        self._a = np.ascontiguousarray(a, dtype=np.complex128 if self.hermitian else np.float64)
        if self._ia.size != self.n + 1:
            raise ValueError(f"ia must have n+1 = {self.n + 1} entries")
        nnz = int(self._ia[-1])
        if self._ja.size < nnz or self._a.size < nnz:
            raise ValueError("ja/a shorter than ia[n]")
        o = _Opts()
        lib.rgf_default_opts(C.byref(o))
        o.precision = PRECISION[precision]
        o.slices = int(slices)
        o.selinv_mode = SELINV[selinv]
        o.device = int(device)
        o.use_graphs = 1 if use_graphs else 0
        # True/1: FP64-accurate emulated diagonal blocks, "native"/2: FP64
        # units, False/0: bulk slice count
        o.fp64_diag = {True: 1, False: 0, "native": 2}.get(fp64_diag, fp64_diag)
        o.async_upload = 1 if async_upload else 0
        create = lib.rgf_create_hermitian if self.hermitian else lib.rgf_create
        _check(create(_ptr(self._ia), _ptr(self._ja), _ptr(self._a), self.ns, self.nt, self.nd,
                      C.byref(o), C.byref(self._h)), "rgf_create")
        self._dt = np.complex128 if self.hermitian else np.float64

    # -- reference methods ----------------------------------------------------
    def factorize(self) -> None:
        """RGF.H:510-546."""
        _check(self._lib.rgf_factorize(self._h), "rgf_factorize")

    def logDet(self) -> float:
        """RGF.H:616-627."""
        out = C.c_double()
        _check(self._lib.rgf_logdet(self._h, C.byref(out)), "rgf_logdet")
        return out.value

    def solve(self, x, b=None, nrhs: int | None = None):
        """``solve(b, nrhs)`` in place (RGF.H:550-554) or ``solve(x, b, nrhs)``
        (RGF.H:559-578).  Arrays are n x nrhs column-major (ld = n); returns x."""
        if b is None:
            b = x
        b = np.asarray(b, dtype=self._dt)
        if nrhs is None:
            nrhs = 1 if b.ndim == 1 else b.shape[1]
        bf = np.asfortranarray(b.reshape(self.n, nrhs) if b.ndim == 1 else b)
        out = np.empty((self.n, nrhs), dtype=self._dt, order="F")
        _check(self._lib.rgf_solve(self._h, _ptr(out), _ptr(bf), int(nrhs)), "rgf_solve")
        if isinstance(x, np.ndarray) and x.size == out.size:
            if x.ndim == 1:
                x[:] = out.ravel(order="F")
            else:
                x[...] = out.reshape(x.shape, order="F")
        return out[:, 0] if b.ndim == 1 else out

    def RGFdiag(self, diag=None) -> np.ndarray:
        """RGF.H:582-612: diag(A^{-1})."""
        out = np.empty(self.n, dtype=self._dt)
        _check(self._lib.rgf_diag(self._h, _ptr(out)), "rgf_diag")
        if diag is not None:
            diag[:] = out
        return out

    def residualNorm(self, x, b) -> float:
        """RGF.H:631-655 (first right-hand side)."""
        xx = np.ascontiguousarray(np.asarray(x, dtype=self._dt).reshape(self.n, -1, order="F")[:, 0])
        bb = np.ascontiguousarray(np.asarray(b, dtype=self._dt).reshape(self.n, -1, order="F")[:, 0])
        out = C.c_double()
        _check(self._lib.rgf_residual_norm(self._h, _ptr(xx), _ptr(bb), C.byref(out)),
               "rgf_residual_norm")
        return out.value

    def residualNormNormalized(self, x, b) -> float:
        """RGF.H:659-663."""
        xx = np.ascontiguousarray(np.asarray(x, dtype=self._dt).reshape(self.n, -1, order="F")[:, 0])
        bb = np.ascontiguousarray(np.asarray(b, dtype=self._dt).reshape(self.n, -1, order="F")[:, 0])
        out = C.c_double()
        _check(self._lib.rgf_residual_norm_normalized(self._h, _ptr(xx), _ptr(bb), C.byref(out)),
               "rgf_residual_norm_normalized")
        return out.value

    # -- extensions -------------------------------------------------------------
    def export_factor(self) -> np.ndarray:
        """The factor in the reference's MF layout (lower triangles defined)."""
        info = self.info()
        out = np.empty(info["mf_size"], dtype=np.float64)
        _check(self._lib.rgf_export_factor(self._h, _ptr(out)), "rgf_export_factor")
        return out

    def export_selinv(self) -> np.ndarray:
        """Selected inverse blocks in the MF layout."""
        info = self.info()
        out = np.empty(info["mf_size"], dtype=np.float64)
        _check(self._lib.rgf_export_selinv(self._h, _ptr(out)), "rgf_export_selinv")
        return out

    def info(self) -> dict:
        i = _Info()
        _check(self._lib.rgf_get_info(self._h, C.byref(i)), "rgf_get_info")
        return {"n": i.n, "nnz": i.nnz, "mf_size": i.mf_size, "device_bytes": i.device_bytes,
                "not_spd_column": i.not_spd_column, "kernels_launched": i.kernels_launched}

    def diag_device_ptr(self) -> int:
        p = C.c_void_p()
        _check(self._lib.rgf_diag_device(self._h, C.byref(p)), "rgf_diag_device")
        return p.value

    def stream(self) -> int:
        p = C.c_void_p()
        _check(self._lib.rgf_get_stream(self._h, C.byref(p)), "rgf_get_stream")
        return p.value or 0

    def tuning(self) -> dict:
        """The knobs of this instance: leaf_nb, lookahead, split_bias and the
        autotuner's measured factorize + RGFdiag time ``ms`` (0 if none)."""
        return _tuning_of(self._lib, self._h)

    def set_tuning(self, leaf_nb: int = 32, lookahead: int = 1, split_bias: float = 1.0,
                   splitk_max: int = 0, fp64_tile: int = 0) -> None:
        """Set the knobs (leaf_nb 16/32/64, lookahead 0/1, split_bias in
        [1/16, 16], tile shapes: splitk_max 0/1/2/4/8/16 and fp64_tile
        0/32/64); the factor is recomputed on next use."""
        t = _tuning_struct(leaf_nb, lookahead, split_bias, splitk_max, fp64_tile)
        _check(self._lib.rgf_set_tuning(self._h, C.byref(t)), "rgf_set_tuning")

    def autotune(self, force: bool = False) -> dict:
        """Measure candidate knobs on this instance (or take the process-wide
        cached choice for its class) and keep the fastest; returns it."""
        t = _Tuning()
        _check(self._lib.rgf_autotune(self._h, TUNE_FORCE if force else 0, C.byref(t)),
               "rgf_autotune")
        return _tuning_dict(t)

    def set_wait_limit(self, polls: int) -> None:
        """Poll limit of the leaf Cholesky's pivot wait (0 = default); a wait
        that runs out makes the stage raise RGFError(RGF_ETIMEOUT)."""
        _check(self._lib.rgf_set_wait_limit(self._h, int(polls)), "rgf_set_wait_limit")

    def kernel_timer(self, enable) -> None:
        """True/1: time bulk GEMMs; 2: also print per-shape totals on reset."""
        _check(self._lib.rgf_kernel_timer_enable(self._h, int(enable)), "timer")

    def kernel_timer_read(self, reset: bool = True) -> dict:
        """Per class: 'all', 'fp64' (DMMA GEMM), 'split' (tensor-core GEMM) with
        ms, launches and FP64-equivalent flops; 'split' also has tensor_flops."""
        out = {}
        for kind, name in ((0, "all"), (1, "fp64"), (2, "split"), (3, "split_tensor")):
            ms, n, fl = C.c_double(), C.c_longlong(), C.c_double()
            _check(self._lib.rgf_kernel_timer_read(self._h, 0, kind, C.byref(ms), C.byref(n),
                                                   C.byref(fl)), "timer")
            out[name] = {"ms": ms.value, "launches": n.value, "flops": fl.value}
        out["split"]["tensor_flops"] = out.pop("split_tensor")["flops"]
        if reset:
            _check(self._lib.rgf_kernel_timer_read(self._h, 1, 0, None, None, None), "timer")
        return out

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.rgf_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class RGFBatch:
    """Many independent instances (uneven ns, nt, nd) factorized together.

    ``instances`` is a sequence of ``(ia, ja, a, ns, nt, nd)``.  ``run()``
    returns ``(logdet[count], [diag_0, ...])``: with ``concurrent=True`` the
    whole batch is one captured CUDA graph with a concurrent branch per
    instance; ``concurrent=False`` runs instance after instance (the
    per-instance baseline).  Options are those of :class:`RGF`.
    """

    def __init__(self, instances, precision: str = "fp64", slices: int = 0,
                 selinv: str = "exact", device: int = -1, fp64_diag=1):
        lib = load_library()
        self._lib = lib
        self._h = C.c_void_p()
        self._keep = []
        cnt = len(instances)
        ia_p = (C.c_void_p * cnt)()
        ja_p = (C.c_void_p * cnt)()
        a_p = (C.c_void_p * cnt)()
        ns = np.empty(cnt, dtype=np.uint64)
        nt = np.empty(cnt, dtype=np.uint64)
        nd = np.empty(cnt, dtype=np.uint64)
        self.sizes = []
        for i, (ia, ja, a, s_, t_, d_) in enumerate(instances):
            ia = np.ascontiguousarray(ia, dtype=np.uint64)
            ja = np.ascontiguousarray(ja, dtype=np.uint64)
            a = np.ascontiguousarray(a, dtype=np.float64)
            self._keep += [ia, ja, a]
            ia_p[i], ja_p[i], a_p[i] = ia.ctypes.data, ja.ctypes.data, a.ctypes.data
            ns[i], nt[i], nd[i] = s_, t_, d_
            self.sizes.append((int(s_), int(t_), int(d_)))
        o = _Opts()
        lib.rgf_default_opts(C.byref(o))
        o.precision = PRECISION[precision]
        o.slices = int(slices)
        o.selinv_mode = SELINV[selinv]
        o.device = int(device)
        o.fp64_diag = {True: 1, False: 0, "native": 2}.get(fp64_diag, fp64_diag)
        _check(lib.rgf_batch_create(cnt, ia_p, ja_p, a_p, _ptr(ns), _ptr(nt), _ptr(nd),
                                    C.byref(o), C.byref(self._h)), "rgf_batch_create")
        self._keep = []  # the library copied the CSC to the device
        self.count = cnt

    def run(self, concurrent: bool = True, want_diag: bool = True):
        logdet = np.empty(self.count, dtype=np.float64)
        diags = [np.empty(s * t + d, dtype=np.float64) for (s, t, d) in self.sizes] if want_diag else []
        ptrs = (C.c_void_p * self.count)(*[x.ctypes.data for x in diags]) if want_diag else None
        _check(self._lib.rgf_batch_run(self._h, 0 if concurrent else 1, _ptr(logdet),
                                       ptrs), "rgf_batch_run")
        return logdet, diags

    def stream(self) -> int:
        p = C.c_void_p()
        _check(self._lib.rgf_batch_get_stream(self._h, C.byref(p)), "rgf_batch_get_stream")
        return p.value or 0

    def kernels(self) -> int:
        k = C.c_longlong()
        _check(self._lib.rgf_batch_kernels(self._h, C.byref(k)), "rgf_batch_kernels")
        return k.value

    def autotune(self, force: bool = False) -> int:
        """Tune every (ns, nd) class of the batch on its instance of median nt
        (or take the cached choice) and set it on all members; returns the
        number of classes."""
        n = C.c_size_t()
        _check(self._lib.rgf_batch_autotune(self._h, TUNE_FORCE if force else 0, C.byref(n)),
               "rgf_batch_autotune")
        return n.value

    def _handle(self, i: int) -> C.c_void_p:
        h = C.c_void_p()
        _check(self._lib.rgf_batch_handle(self._h, int(i), C.byref(h)), "rgf_batch_handle")
        return h

    def tunings(self) -> list:
        """The knobs of every instance (see :meth:`RGF.tuning`)."""
        return [_tuning_of(self._lib, self._handle(i)) for i in range(self.count)]

    def set_tuning(self, i: int, leaf_nb: int = 32, lookahead: int = 1,
                   split_bias: float = 1.0, splitk_max: int = 0, fp64_tile: int = 0) -> None:
        """Set the knobs of instance i; the batch graph is captured again."""
        t = _tuning_struct(leaf_nb, lookahead, split_bias, splitk_max, fp64_tile)
        _check(self._lib.rgf_set_tuning(self._handle(i), C.byref(t)), "rgf_set_tuning")

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.rgf_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RGFServer:
    """Request loop with continuous batching and resident factors.

    ``submit_factor`` / ``submit_solve`` / ``submit_diag`` / ``submit_release``
    return a ticket; ``wait(ticket)`` returns a dict with the request's
    status, latency and results (``factor_id`` and ``logdet`` for factor
    requests, ``x`` for solves, ``diag`` for RGFdiag).
    """

    FACTOR, SOLVE, DIAG, RELEASE = 0, 1, 2, 3

    def __init__(self, hbm_budget_bytes: int, slots: int = 8, precision: str = "fp64",
                 slices: int = 0, selinv: str = "exact", device: int = -1, fp64_diag=1):
        lib = load_library()
        self._lib = lib
        self._h = C.c_void_p()
        o = _Opts()
        lib.rgf_default_opts(C.byref(o))
        o.precision = PRECISION[precision]
        o.slices = int(slices)
        o.selinv_mode = SELINV[selinv]
        o.device = int(device)
        o.fp64_diag = {True: 1, False: 0, "native": 2}.get(fp64_diag, fp64_diag)
        _check(lib.rgf_server_create(C.byref(o), int(hbm_budget_bytes), int(slots),
                                     C.byref(self._h)), "rgf_server_create")
        self._live = {}

    def _submit(self, req, keep):
        t = C.c_longlong()
        _check(self._lib.rgf_server_submit(self._h, C.byref(req), C.byref(t)), "rgf_server_submit")
        self._live[t.value] = (req, keep)
        return t.value

    def submit_factor(self, ia, ja, a, ns, nt, nd) -> int:
        ia = np.ascontiguousarray(ia, dtype=np.uint64)
        ja = np.ascontiguousarray(ja, dtype=np.uint64)
        a = np.ascontiguousarray(a, dtype=np.float64)
        r = _Request(kind=self.FACTOR, ia=ia.ctypes.data, ja=ja.ctypes.data, a=a.ctypes.data,
                     ns=ns, nt=nt, nd=nd)
        return self._submit(r, {"ia": ia, "ja": ja, "a": a})

    def submit_solve(self, factor_id: int, b) -> int:
        b = np.asfortranarray(b, dtype=np.float64)
        if b.ndim == 1:
            b = b.reshape(-1, 1, order="F")
        x = np.empty_like(b, order="F")
        r = _Request(kind=self.SOLVE, factor_id=factor_id, b=b.ctypes.data, x=x.ctypes.data,
                     nrhs=b.shape[1])
        return self._submit(r, {"b": b, "x": x})

    def submit_diag(self, factor_id: int, n: int) -> int:
        d = np.empty(n, dtype=np.float64)
        r = _Request(kind=self.DIAG, factor_id=factor_id, diag=d.ctypes.data)
        return self._submit(r, {"diag": d})

    def submit_release(self, factor_id: int) -> int:
        return self._submit(_Request(kind=self.RELEASE, factor_id=factor_id), {})

    def wait(self, ticket: int, timeout_s: float = 600.0) -> dict:
        st = C.c_int()
        _check(self._lib.rgf_server_wait(self._h, ticket, timeout_s, C.byref(st)), "rgf_server_wait")
        req, keep = self._live.pop(ticket)
        out = {"status": req.status, "latency_ms": req.latency_ms, "kind": req.kind}
        if req.kind == self.FACTOR:
            out.update(factor_id=req.factor_id, logdet=req.logdet)
        if "x" in keep:
            out["x"] = keep["x"]
        if "diag" in keep:
            out["diag"] = keep["diag"]
        return out

    def stats(self) -> dict:
        st = _ServerStats()
        _check(self._lib.rgf_server_stats(self._h, C.byref(st)), "rgf_server_stats")
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.rgf_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
