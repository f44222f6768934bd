"""Seeded synthetic block-tridiagonal-arrowhead (BTA) matrices and .dat I/O.

The matrix is symmetric positive definite of size n = ns*nt + nd and is
returned as its lower triangle in CSC form with ``size_t`` indices -- the
input format of the reference's ``RGF(ia, ja, a, ns, nt, nd)`` constructor
(``RGF.H:84-89``; the same arrays ``main.C:49-70`` reads from a ``.dat``
file):

* diagonal blocks   D_i = A_i A_i^T / ns + (ns + 2) I,   A_i ~ N(0, 1)
  (optionally plus kappa^2 I + a 5-point Laplacian on a gx x gy grid,
  gx * gy = ns -- an SPDE-like operator);
* sub-diagonal      B_i ~ N(0, 0.1 / ns)  (block row i+1, block column i);
* arrowhead rows    C_i ~ N(0, 0.1), nd x ns;
* corner            R R^T / nd + (nt + 2) I,   R ~ N(0, 1), nd x nd.

Random draws come from ``numpy.random.default_rng(seed)`` in the order
A_i, B_i (i < nt-1), C_i for i = 0..nt-1, then R.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import blas as _blas


def laplacian_5pt(gx: int, gy: int) -> np.ndarray:
    """Dense 5-point Laplacian (4 on the diagonal, -1 to grid neighbours)."""
    n = gx * gy
    Lp = 4.0 * np.eye(n)
    idx = np.arange(n).reshape(gy, gx)
    for a, b in ((idx[:, :-1], idx[:, 1:]), (idx[:-1, :], idx[1:, :])):
        Lp[a.ravel(), b.ravel()] = -1.0
        Lp[b.ravel(), a.ravel()] = -1.0
    return Lp


def bta_nnz(ns: int, nt: int, nd: int) -> int:
    """Stored (lower) non-zeros of a dense-block BTA matrix."""
    return nt * ns * (ns + 1) // 2 + (nt - 1) * ns * ns + nt * ns * nd + nd * (nd + 1) // 2


def generate_bta(ns: int, nt: int, nd: int, seed: int, spde_grid=None, kappa2: float = 1.0):
    """Return (ia, ja, a): lower CSC of a seeded SPD BTA matrix.

    ``ia``/``ja`` are ``uint64`` (size_t), ``a`` is ``float64``.
    """
    ns, nt, nd = int(ns), int(nt), int(nd)
    rng = np.random.default_rng(seed)
    n = ns * nt + nd
    nnz = bta_nnz(ns, nt, nd)
    ia = np.empty(n + 1, dtype=np.uint64)
    ja = np.empty(nnz, dtype=np.uint64)
    a = np.empty(nnz, dtype=np.float64)
    spde = None
    if spde_grid is not None:
        gx, gy = spde_grid
        if gx * gy != ns:
            raise ValueError("spde grid must have ns points")
        spde = laplacian_5pt(gx, gy) + kappa2 * np.eye(ns)
    pos = 0
    ia[0] = 0
    col = 0
    for i in range(nt):
        last = i == nt - 1
        ro = ns if last else 2 * ns
        lda = ro + nd
        P = np.empty((ns, lda))          # P[j, r] = entry (row r of panel, column j)
        A = rng.standard_normal((ns, ns))
        D = _blas.dsyrk(1.0 / ns, A, lower=1)          # lower triangle of A A^T / ns
        D = np.tril(D) + np.tril(D, -1).T
        D[np.diag_indices(ns)] += ns + 2.0
        if spde is not None:
            D += spde
        P[:, :ns] = D.T
        if not last:
            B = rng.standard_normal((ns, ns)) * np.sqrt(0.1 / ns)
            P[:, ns:2 * ns] = B.T
        if nd:
            C = rng.standard_normal((nd, ns)) * np.sqrt(0.1)
            P[:, ro:] = C.T
        r = np.arange(lda)
        mask = (r[None, :] >= np.arange(ns)[:, None]) | (r[None, :] >= ns)
        rowg = np.where(r < ro, i * ns + r, nt * ns + r - ro).astype(np.uint64)
        cnt = mask.sum(axis=1)
        k = int(cnt.sum())
        a[pos:pos + k] = P[mask]
        ja[pos:pos + k] = np.broadcast_to(rowg, (ns, lda))[mask]
        ia[col + 1:col + ns + 1] = pos + np.cumsum(cnt)
        pos += k
        col += ns
    if nd:
        R = rng.standard_normal((nd, nd))
        Cn = R @ R.T / nd + (nt + 2.0) * np.eye(nd)
        for k in range(nd):
            m = nd - k
            a[pos:pos + m] = Cn[k:, k]
            ja[pos:pos + m] = nt * ns + np.arange(k, nd, dtype=np.uint64)
            pos += m
            ia[col + 1] = pos
            col += 1
    assert pos == nnz and col == n
    return ia, ja, a


def random_rhs(n: int, nrhs: int, seed: int) -> np.ndarray:
    """Column-major (ld = n) right-hand sides ~ N(0, 1), shape (n, nrhs)."""
    rng = np.random.default_rng(seed + 1000003)
    return np.asfortranarray(rng.standard_normal((n, nrhs)))


def read_dat(path):
    """Read the reference's .dat matrix format (main.C:41-72).

    Whitespace-separated: n, n, nnz, ia[n+1], ja[nnz], a[nnz].
    Returns (n, ia, ja, a).
    """
    with open(path) as f:
        tok = f.read().split()
    n = int(tok[0])
    nnz = int(tok[2])
    ia = np.array(tok[3:3 + n + 1], dtype=np.uint64)
    nnz = int(ia[-1])
    ja = np.array(tok[4 + n:4 + n + nnz], dtype=np.uint64)
    a = np.array(tok[4 + n + nnz:4 + n + 2 * nnz], dtype=np.float64)
    return n, ia, ja, a


def write_dat(path, ia, ja, a) -> None:
    n = len(ia) - 1
    with open(path, "w") as f:
        f.write(f"{n}\n{n}\n{int(ia[-1])}\n")
        f.write("\n".join(str(int(v)) for v in ia) + "\n")
        f.write("\n".join(str(int(v)) for v in ja) + "\n")
        f.write("\n".join(repr(float(v)) for v in a) + "\n")


def write_rhs(path, b) -> None:
    """RHS file read by main.C:79-84 (one value per line, column-major)."""
    with open(path, "w") as f:
        f.write("\n".join(repr(float(v)) for v in np.asarray(b).ravel(order="F")) + "\n")


def batch_shapes(count: int, seed: int, ns_choices=(42, 128, 256, 512), nt_range=(3, 60),
                 nd_choices=(0, 2, 6)):
    """Seeded uneven instance sizes: ns from ns_choices, nt uniform in
    nt_range (inclusive), nd from nd_choices."""
    rng = np.random.default_rng(seed)
    return [(int(rng.choice(ns_choices)), int(rng.integers(nt_range[0], nt_range[1] + 1)),
             int(rng.choice(nd_choices))) for _ in range(count)]


def generate_batch(count: int, seed: int, **kw):
    """(ia, ja, a, ns, nt, nd) for `count` seeded uneven instances."""
    out = []
    for i, (ns, nt, nd) in enumerate(batch_shapes(count, seed, **kw)):
        ia, ja, a = generate_bta(ns, nt, nd, seed * 100003 + i)
        out.append((ia, ja, a, ns, nt, nd))
    return out


def generate_bta_hermitian(ns: int, nt: int, nd: int, seed: int):
    """Return (ia, ja, a): lower CSC of a seeded Hermitian positive-definite
    BTA matrix, ``a`` complex128.  Same structure and scales as generate_bta
    with complex N(0, 1) draws: D_i = A_i A_i^H / ns + (ns + 2) I,
    B_i ~ N(0, 0.1/ns), C_i ~ N(0, 0.1), corner R R^H / nd + (nt + 2) I.
    Dense assembly: meant for test sizes."""
    ns, nt, nd = int(ns), int(nt), int(nd)
    rng = np.random.default_rng(seed)
    n = ns * nt + nd

    def cn(*shape):
        return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)

    A = np.zeros((n, n), dtype=np.complex128)
    for i in range(nt):
        s = slice(i * ns, (i + 1) * ns)
        G = cn(ns, ns)
        A[s, s] = G @ G.conj().T / ns + (ns + 2.0) * np.eye(ns)
        if i < nt - 1:
            t = slice((i + 1) * ns, (i + 2) * ns)
            A[t, s] = cn(ns, ns) * np.sqrt(0.1 / ns)
        if nd:
            A[nt * ns:, s] = cn(nd, ns) * np.sqrt(0.1)
    if nd:
        R = cn(nd, nd)
        A[nt * ns:, nt * ns:] = R @ R.conj().T / nd + (nt + 2.0) * np.eye(nd)
    A = np.tril(A)
    A = A + np.tril(A, -1).conj().T
    np.fill_diagonal(A, A.diagonal().real)
    # lower CSC over the full block pattern (explicit zeros kept)
    ia = np.zeros(n + 1, dtype=np.uint64)
    rows, vals = [], []
    for c in range(n):
        if c < ns * nt:
            i = c // ns
            hi = (i + 2) * ns if i < nt - 1 else (i + 1) * ns
            r = np.concatenate([np.arange(c, hi), np.arange(nt * ns, n)])
        else:
            r = np.arange(c, n)
        rows.append(r)
        vals.append(A[r, c])
        ia[c + 1] = ia[c] + len(r)
    return ia, np.concatenate(rows).astype(np.uint64), np.concatenate(vals)
