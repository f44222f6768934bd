"""CPU oracle for the RGF hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy/scipy (host LAPACK/BLAS, FP64), the block
recursion of the reference class ``RGF<double>`` (rjanalik/RGF, ``RGF.H``).
It is the checker: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.
The product library (``rgf_gb300``) never calls it and has no CPU fallback.

Functions and the reference lines they follow:

* ``Layout``              -- ``RGF.H:84-138`` (block map, ``diag_pos``),
                             ``RGF.H:174-229`` (``mf_block_*`` index math)
* ``ingest``              -- ``RGF.H:684-700`` + ``CWC_utility.cu:998-1029``
                             (``getPos``) and ``:1085-1105`` (supernode scatter)
* ``factorize``           -- ``RGF.H:233-340`` (``FirstStageFactor``)
* ``logdet``              -- ``RGF.H:616-627`` + ``Blas.H:1084-1092``
* ``solve``               -- ``RGF.H:344-418`` (``SecondStageSolve``)
* ``selinv_compat``       -- ``RGF.H:422-506`` (``ThirdStageRGF``): the
                             reference's recursion, which drops the arrowhead
                             cross terms when ``nd > 0``
* ``selinv_exact``        -- the exact block selected inversion (derived from
                             ``Sigma L = L^{-T}``); equals ``selinv_compat``
                             when ``nd == 0``
* ``residual_norm``       -- ``RGF.H:631-663``

Deliberate deviation: for ``nt == 1 and nd > 0`` the reference never applies
the TRSM to the arrowhead rows (both TRSMs are guarded by ``nt > 1``,
``RGF.H:258,293``), which yields a wrong factor; this oracle factors that case
correctly.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.linalg import blas as _blas
from scipy.linalg import lapack as _lapack


# --------------------------------------------------------------------------
# Block layout (RGF.H:84-138, 174-229)
# --------------------------------------------------------------------------
class Layout:
    """Offsets of the block-column ("supernode") layout of the factor MF.

    Block column ``i < nt-1`` is a column-major ``(2ns+nd) x ns`` panel
    ``[L_ii; L_{i+1,i}; C_i]``; block column ``nt-1`` is ``(ns+nd) x ns``
    (``[L_ii; C_i]``); the corner is ``nd x nd``.  (RGF.H:95, 114-138)
    """

    def __init__(self, ns: int, nt: int, nd: int):
        if ns < 1 or nt < 1:
            raise ValueError("ns and nt must be >= 1")
        self.ns, self.nt, self.nd = int(ns), int(nt), int(nd)
        self.n = ns * nt + nd
        self.mf_size = 2 * (nt - 1) * ns * ns + ns * ns + self.n * nd  # RGF.H:95

    def lda(self, i: int) -> int:
        """Leading dimension of block column i (RGF.H:183-195)."""
        if i < self.nt - 1:
            return 2 * self.ns + self.nd
        if i < self.nt:
            return self.ns + self.nd
        return self.nd

    def col_offset(self, i: int) -> int:
        """Offset of block column i in MF (RGF.H:121,128,136)."""
        ns, nd = self.ns, self.nd
        if i < self.nt:
            return i * ns * (2 * ns + nd)
        return (self.nt - 1) * ns * (2 * ns + nd) + ns * (ns + nd)

    def dense_row_offset(self, i: int) -> int:
        """Row of C_i inside block column i (RGF.H:213-221)."""
        if i < self.nt - 1:
            return 2 * self.ns
        if i == self.nt - 1:
            return self.ns
        return 0

    def diag_pos(self) -> np.ndarray:
        """Offsets of the diagonal entries of L in MF (RGF.H:114-138)."""
        ns, nt, nd = self.ns, self.nt, self.nd
        pos = np.empty(self.n, dtype=np.int64)
        for i in range(nt):
            pos[i * ns:(i + 1) * ns] = self.col_offset(i) + np.arange(ns) * (self.lda(i) + 1)
        if nd:
            pos[nt * ns:] = self.col_offset(nt) + np.arange(nd) * (nd + 1)
        return pos

    def panel(self, MF: np.ndarray, i: int) -> np.ndarray:
        """Fortran-ordered view of block column i (or the corner, i == nt)."""
        rows = self.lda(i)
        cols = self.ns if i < self.nt else self.nd
        off = self.col_offset(i)
        return MF[off:off + rows * cols].reshape((rows, cols), order="F")


# --------------------------------------------------------------------------
# Ingest: lower CSC -> MF (RGF.H:684-700, CWC_utility.cu:998-1029, 1085-1105)
# --------------------------------------------------------------------------
def mf_position(L: Layout, r: np.ndarray, c: np.ndarray) -> np.ndarray:
    """Offset in MF of the lower-triangle entry (r, c), r >= c.

    Same mapping as the reference's ``getPos`` (CWC_utility.cu:998-1029):
    the column's block column gives the panel, the row's block gives the
    panel row (own block, next block or arrowhead rows).
    """
    ns, nt = L.ns, L.nt
    r = np.asarray(r, dtype=np.int64)
    c = np.asarray(c, dtype=np.int64)
    ib = np.minimum(c // ns, nt)
    jc = np.where(ib < nt, c - ib * ns, c - nt * ns)
    col_off = np.where(ib < nt - 1, ib * ns * (2 * ns + L.nd),
                       np.where(ib == nt - 1, (nt - 1) * ns * (2 * ns + L.nd),
                                (nt - 1) * ns * (2 * ns + L.nd) + ns * (ns + L.nd)))
    lda = np.where(ib < nt - 1, 2 * ns + L.nd, np.where(ib == nt - 1, ns + L.nd, L.nd))
    in_arrow = r >= ns * nt
    row = np.where(in_arrow,
                   np.where(ib < nt - 1, 2 * ns, np.where(ib == nt - 1, ns, 0)) + (r - ns * nt),
                   r - ib * ns)
    return col_off + jc * lda + row


def check_pattern(L: Layout, ia: np.ndarray, ja: np.ndarray) -> None:
    """Raise ValueError unless (ia, ja) is a lower CSC of the BTA pattern."""
    n = L.n
    ia = np.asarray(ia, dtype=np.int64)
    ja = np.asarray(ja, dtype=np.int64)
    if ia.shape != (n + 1,) or ia[0] != 0 or np.any(np.diff(ia) < 0) or ia[-1] != ja.size:
        raise ValueError("malformed column pointers")
    c = np.repeat(np.arange(n, dtype=np.int64), np.diff(ia))
    r = ja
    if np.any(r < c) or np.any(r >= n):
        raise ValueError("row index outside the lower triangle")
    ns, nt = L.ns, L.nt
    rb = np.minimum(r // ns, nt)
    cb = np.minimum(c // ns, nt)
    ok = (rb == cb) | (rb == cb + 1) & (rb < nt) | (rb == nt)
    if not np.all(ok):
        raise ValueError("entry outside the block-tridiagonal-arrowhead pattern")


def ingest(L: Layout, ia, ja, a) -> np.ndarray:
    """Scatter the lower CSC into a zeroed MF array (RGF.H:695-699)."""
    ia = np.asarray(ia, dtype=np.int64)
    ja = np.asarray(ja, dtype=np.int64)
    a = np.asarray(a, dtype=np.float64)
    check_pattern(L, ia, ja)
    MF = np.zeros(L.mf_size, dtype=np.float64)
    c = np.repeat(np.arange(L.n, dtype=np.int64), np.diff(ia))
    MF[mf_position(L, ja, c)] = a
    return MF


# --------------------------------------------------------------------------
# Dense helpers on Fortran views
# --------------------------------------------------------------------------
def _potrf_lower(A: np.ndarray) -> None:
    """In-place lower Cholesky of the square Fortran view A (tpotrf_dev 'L')."""
    c, info = _lapack.dpotrf(A, lower=1, clean=0, overwrite_a=0)
    if info != 0:
        raise np.linalg.LinAlgError(f"dpotrf info={info}")
    A[:, :] = np.tril(c) + np.triu(A, 1)


def _trsm_rltn(Lii: np.ndarray, B: np.ndarray) -> None:
    """B := B * tril(Lii)^{-T} (ttrsm_dev('R','L','T','N'), RGF.H:260,287,317)."""
    if B.shape[0] == 0:
        return
    B[:, :] = _blas.dtrsm(1.0, np.tril(Lii), B, side=1, lower=1, trans_a=1, diag=0)


def _trsm_left(Lii: np.ndarray, X: np.ndarray, trans: bool) -> np.ndarray:
    """tril(Lii)^{-1} X or tril(Lii)^{-T} X (c_ttrsm('L','L','N'|'T','N'))."""
    return _blas.dtrsm(1.0, np.tril(Lii), X, side=0, lower=1, trans_a=int(trans), diag=0)


def _trtri_lower(Lii: np.ndarray) -> np.ndarray:
    inv, info = _lapack.dtrtri(np.tril(Lii), lower=1, unitdiag=0)
    if info != 0:
        raise np.linalg.LinAlgError(f"dtrtri info={info}")
    return np.tril(inv)


# --------------------------------------------------------------------------
# Stage 1: factorize (RGF.H:233-340)
# --------------------------------------------------------------------------
def factorize(L: Layout, MF: np.ndarray) -> None:
    """Block Cholesky in place on MF, lower triangles of the diagonal blocks.

    Step order follows RGF.H:245-339: for block column i the Schur updates
    from block column i-1 (diagonal block, arrowhead rows, corner), then
    POTRF of the diagonal block, then TRSM of the rows below it.  The
    reference applies a full GEMM to the diagonal block; only its lower
    triangle is meaningful, and only that is written here.
    """
    ns, nt, nd = L.ns, L.nt, L.nd
    corner = L.panel(MF, nt) if nd else None
    prev = None
    for i in range(nt):
        P = L.panel(MF, i)
        if prev is not None:
            Bm = prev[ns:2 * ns, :]                       # L_{i,i-1}
            D = P[:ns, :]
            D[:, :] -= np.tril(_blas.dsyrk(1.0, Bm, lower=1))   # RGF.H:276,304
            if nd:
                ro_m = L.dense_row_offset(i - 1)
                Cm = prev[ro_m:ro_m + nd, :]              # C_{i-1}
                ro = L.dense_row_offset(i)
                P[ro:ro + nd, :] -= Cm @ Bm.T             # RGF.H:279,307
                corner[:, :] -= Cm @ Cm.T                 # RGF.H:280,308
        _potrf_lower(P[:ns, :])                           # RGF.H:254,284,312
        if P.shape[0] > ns:
            _trsm_rltn(P[:ns, :], P[ns:, :])              # RGF.H:260,287,317
        prev = P
    if nd:
        ro = L.dense_row_offset(nt - 1)
        Cl = prev[ro:ro + nd, :]
        corner[:, :] -= Cl @ Cl.T                         # RGF.H:332
        _potrf_lower(corner)                              # RGF.H:335


def logdet(L: Layout, MF: np.ndarray) -> float:
    """2 * sum(log L_kk) over the diagonal of the factor (RGF.H:616-627)."""
    return float(2.0 * np.sum(np.log(MF[L.diag_pos()])))


# --------------------------------------------------------------------------
# Stage 2: solve (RGF.H:344-418)
# --------------------------------------------------------------------------
def solve(L: Layout, MF: np.ndarray, b: np.ndarray) -> np.ndarray:
    """x = A^{-1} b by block forward/backward substitution.

    ``b`` is ``n x nrhs`` (or length n); column-major semantics as in the
    reference (ld = n).
    """
    ns, nt, nd = L.ns, L.nt, L.nd
    squeeze = b.ndim == 1
    rhs = np.array(b, dtype=np.float64, copy=True).reshape(L.n, -1)
    blk = lambda i: slice(i * ns, (i + 1) * ns)
    dsl = slice(nt * ns, nt * ns + nd)
    # forward (RGF.H:353-383)
    for i in range(nt):
        P = L.panel(MF, i)
        if i > 0:
            Pm = L.panel(MF, i - 1)
            rhs[blk(i)] -= Pm[ns:2 * ns, :] @ rhs[blk(i - 1)]
        rhs[blk(i)] = _trsm_left(P[:ns, :], rhs[blk(i)], trans=False)
    if nd:
        for i in range(nt):
            P = L.panel(MF, i)
            ro = L.dense_row_offset(i)
            rhs[dsl] -= P[ro:ro + nd, :] @ rhs[blk(i)]
        rhs[dsl] = _trsm_left(L.panel(MF, nt), rhs[dsl], trans=False)
        # backward (RGF.H:386-400)
        rhs[dsl] = _trsm_left(L.panel(MF, nt), rhs[dsl], trans=True)
        for i in range(nt):
            P = L.panel(MF, i)
            ro = L.dense_row_offset(i)
            rhs[blk(i)] -= P[ro:ro + nd, :].T @ rhs[dsl]
    for i in range(nt - 1, -1, -1):                      # RGF.H:402-417
        P = L.panel(MF, i)
        rhs[blk(i)] = _trsm_left(P[:ns, :], rhs[blk(i)], trans=True)
        if i > 0:
            Pm = L.panel(MF, i - 1)
            rhs[blk(i - 1)] -= Pm[ns:2 * ns, :].T @ rhs[blk(i)]
    return rhs[:, 0] if squeeze else rhs


# --------------------------------------------------------------------------
# Stage 3: selected inversion
# --------------------------------------------------------------------------
def selinv_compat(L: Layout, MF: np.ndarray) -> np.ndarray:
    """diag(A^{-1}) by the reference's recursion (RGF.H:422-506).

    Sigma_ii = L_ii^{-T} (I + L_{i+1,i}^T Sigma_{i+1,i+1} L_{i+1,i}
                          + C_i^T Sigma_dd C_i) L_ii^{-1}.
    Exact for nd == 0; drops the arrowhead cross terms for nd > 0.
    """
    ns, nt, nd = L.ns, L.nt, L.nd
    diag = np.empty(L.n)
    Sdd = None
    if nd:
        Ldinv = _trtri_lower(L.panel(MF, nt))             # RGF.H:439-441
        Sdd = Ldinv.T @ Ldinv                             # RGF.H:442
        diag[nt * ns:] = np.diag(Sdd)                     # RGF.H:461
    Snext = None
    for i in range(nt - 1, -1, -1):
        P = L.panel(MF, i)
        Linv = _trtri_lower(P[:ns, :])                    # RGF.H:449-450,486-487
        T1 = np.eye(ns)                                   # RGF.H:452,489
        if Snext is not None:
            Bi = P[ns:2 * ns, :]
            T1 += (Bi.T @ Snext) @ Bi                     # RGF.H:491-492
        if nd:
            ro = L.dense_row_offset(i)
            Ci = P[ro:ro + nd, :]
            T1 += (Ci.T @ Sdd) @ Ci                       # RGF.H:454-455,496-497
        S = (Linv.T @ T1) @ Linv                          # RGF.H:457-458,500-501
        diag[i * ns:(i + 1) * ns] = np.diag(S)            # RGF.H:483,505
        Snext = S
    return diag


def selinv_exact(L: Layout, MF: np.ndarray, blocks: bool = False):
    """Exact selected inversion of the block-tridiagonal-arrowhead factor.

    From Sigma L = L^{-T} restricted to block column i of L
    ([L_ii; L_{i+1,i}; C_i]):
      Sigma_{i+1,i} = -(Sigma_{i+1,i+1} L_{i+1,i} + Sigma_{d,i+1}^T C_i) L_ii^{-1}
      Sigma_{d,i}   = -(Sigma_dd C_i + Sigma_{d,i+1} L_{i+1,i}) L_ii^{-1}
      Sigma_ii      = L_ii^{-T} (L_ii^{-1} - L_{i+1,i}^T Sigma_{i+1,i} - C_i^T Sigma_{d,i})
    with Sigma_dd = L_dd^{-T} L_dd^{-1}.  Returns diag(A^{-1}); with
    ``blocks=True`` also an MF-shaped array holding Sigma_ii (full),
    Sigma_{i+1,i} and Sigma_{d,i} in the factor's block positions and
    Sigma_dd in the corner.
    """
    ns, nt, nd = L.ns, L.nt, L.nd
    diag = np.empty(L.n)
    MS = np.zeros(L.mf_size) if blocks else None
    Sdd = None
    if nd:
        Ldinv = _trtri_lower(L.panel(MF, nt))
        Sdd = Ldinv.T @ Ldinv
        diag[nt * ns:] = np.diag(Sdd)
        if blocks:
            L.panel(MS, nt)[:, :] = Sdd
    Snext = None      # Sigma_{i+1,i+1}
    Sdnext = None     # Sigma_{d,i+1}
    for i in range(nt - 1, -1, -1):
        P = L.panel(MF, i)
        Linv = _trtri_lower(P[:ns, :])
        Z = np.zeros((ns, ns))
        Ssub = None
        if Snext is not None:
            Bi = P[ns:2 * ns, :]
            X = Snext @ Bi
            if nd:
                ro = L.dense_row_offset(i)
                X += Sdnext.T @ P[ro:ro + nd, :]
            Ssub = -X @ Linv
            Z += Bi.T @ Ssub
        Sd = None
        if nd:
            ro = L.dense_row_offset(i)
            Ci = P[ro:ro + nd, :]
            Y = Sdd @ Ci
            if Snext is not None:
                Y += Sdnext @ P[ns:2 * ns, :]
            Sd = -Y @ Linv
            Z += Ci.T @ Sd
        S = Linv.T @ (Linv - Z)
        S = 0.5 * (S + S.T)
        diag[i * ns:(i + 1) * ns] = np.diag(S)
        if blocks:
            Q = L.panel(MS, i)
            Q[:ns, :] = S
            if Ssub is not None:
                Q[ns:2 * ns, :] = Ssub
            if Sd is not None:
                ro = L.dense_row_offset(i)
                Q[ro:ro + nd, :] = Sd
        Snext, Sdnext = S, Sd
    return (diag, MS) if blocks else diag


# --------------------------------------------------------------------------
# Residual (RGF.H:631-663)
# --------------------------------------------------------------------------
def sym_matvec(ia, ja, a, x: np.ndarray) -> np.ndarray:
    """A x for the symmetric matrix stored as its lower CSC (RGF.H:638-648)."""
    ia = np.asarray(ia, dtype=np.int64)
    ja = np.asarray(ja, dtype=np.int64)
    a = np.asarray(a, dtype=np.float64)
    n = ia.size - 1
    x2 = np.asarray(x, dtype=np.float64).reshape(n, -1)
    c = np.repeat(np.arange(n, dtype=np.int64), np.diff(ia))
    y = np.zeros_like(x2)
    np.add.at(y, ja, a[:, None] * x2[c])
    off = ja != c
    np.add.at(y, c[off], a[off, None] * x2[ja[off]])
    return y.reshape(np.shape(x))


def residual_norm(ia, ja, a, x, b) -> float:
    """||b - A x||_2 (first RHS column), RGF.H:631-655."""
    r = np.asarray(b, dtype=np.float64).reshape(len(ia) - 1, -1)[:, 0] - \
        sym_matvec(ia, ja, a, np.asarray(x).reshape(len(ia) - 1, -1)[:, 0])
    return float(np.linalg.norm(r))


def residual_norm_normalized(ia, ja, a, x, b) -> float:
    """residual_norm / ||b||_2 (RGF.H:659-663)."""
    bb = np.asarray(b, dtype=np.float64).reshape(len(ia) - 1, -1)[:, 0]
    return residual_norm(ia, ja, a, x, b) / float(np.linalg.norm(bb))


# --------------------------------------------------------------------------
# Dense LAPACK oracle (small n only)
# --------------------------------------------------------------------------
def to_dense(ia, ja, a) -> np.ndarray:
    ia = np.asarray(ia, dtype=np.int64)
    n = ia.size - 1
    A = np.zeros((n, n))
    c = np.repeat(np.arange(n, dtype=np.int64), np.diff(ia))
    A[np.asarray(ja, dtype=np.int64), c] = a
    return np.tril(A) + np.tril(A, -1).T


def dense_reference(ia, ja, a, b=None) -> dict:
    """logdet, diag(inv(A)) and (optionally) A^{-1} b from dense LAPACK."""
    A = to_dense(ia, ja, a)
    sign, ld = np.linalg.slogdet(A)
    if sign <= 0:
        raise np.linalg.LinAlgError("matrix is not positive definite")
    Ainv = np.linalg.inv(A)
    out = {"logdet": float(ld), "diag": np.diag(Ainv).copy(), "inv": Ainv}
    if b is not None:
        out["x"] = np.linalg.solve(A, np.asarray(b, dtype=np.float64))
    return out


# --------------------------------------------------------------------------
# Whole-pipeline convenience (what one RGF object does)
# --------------------------------------------------------------------------
def run_all(ns, nt, nd, ia, ja, a, b=None, exact=True) -> dict:
    L = Layout(ns, nt, nd)
    MF = ingest(L, ia, ja, a)
    factorize(L, MF)
    out = {"MF": MF, "logdet": logdet(L, MF)}
    if b is not None:
        out["x"] = solve(L, MF, b)
    out["diag"] = selinv_exact(L, MF) if exact else selinv_compat(L, MF)
    return out
