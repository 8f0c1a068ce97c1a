"""FP64 converged solve of the simpois CG systems (scipy sparse direct).

TEST INFRASTRUCTURE ONLY (the checker).  Builds, for one channel, the system
the reference's CG solves (cleant_cgpois.c:197-264):

* kind 0: A = -Lap restricted to the unknowns, 5-point stencil with
  clamp-to-edge (cleant_cgpois.c:67-89); b = -f_U + Lap_UK g_K.
* kind 1: A = the 13-point bilaplacian with a single clamp
  (cleant_cgpois.c:91-121); b = -f_U - A_UK g_K.

and solves it with a sparse LU factorisation (SuperLU through scipy) in
float64.  The result is the "FP64 converged solve" every GPU result is
compared against.  Large systems are ordered by geometric nested dissection
first (the unknowns are split by separator lines as wide as the stencil's
reach, recursively, separators last): for the 13-point operator on a
1024 x 1024 hole this cuts the factor from 1.2e9 to 4e8 nonzeros and the time
from 23 minutes to under one.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_STENCILS = {
    0: [((0, 0), 4.0), ((1, 0), -1.0), ((0, 1), -1.0), ((-1, 0), -1.0), ((0, -1), -1.0)],
    1: [((0, 0), 20.0),
        ((1, 0), -8.0), ((0, 1), -8.0), ((-1, 0), -8.0), ((0, -1), -8.0),
        ((1, 1), 2.0), ((1, -1), 2.0), ((-1, 1), 2.0), ((-1, -1), 2.0),
        ((2, 0), 1.0), ((0, 2), 1.0), ((-2, 0), 1.0), ((0, -2), 1.0)],
}


def build_system(g, f=None, kind=0):
    """Return (A csr, b, unknown flat indices) for one channel (h, w)."""
    g = np.asarray(g, dtype=np.float32)
    h, w = g.shape
    unk = np.isnan(g).ravel()
    idx = np.flatnonzero(unk)
    n = idx.size
    inv = -np.ones(h * w, np.int64)
    inv[idx] = np.arange(n)
    ii = idx % w
    jj = idx // w
    gk = np.where(unk, 0.0, g.ravel().astype(np.float64))
    rows, cols, vals = [], [], []
    b = np.zeros(n) if f is None else -np.asarray(f, np.float64).ravel()[idx]
    for (di, dj), c in _STENCILS[kind]:
        qi = np.clip(ii + di, 0, w - 1)
        qj = np.clip(jj + dj, 0, h - 1)
        q = qj * w + qi
        qu = inv[q]
        m = qu >= 0
        rows.append(np.arange(n)[m])
        cols.append(qu[m])
        vals.append(np.full(m.sum(), c))
        b[~m] -= c * gk[q[~m]]
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(n, n))
    A.sum_duplicates()
    return A, b, idx


def nested_dissection(ii, jj, reach, leaf=32):
    """Elimination order of the points (ii, jj): the box of a set is cut
    across its longer side by a separator band `reach` pixels wide (no
    stencil couples the two halves through it); halves first, recursively,
    then the band; sets of at most `leaf` points are kept in raster order."""
    out = []
    stack = [(np.arange(ii.size), 0)]
    # explicit stack: (set, state); state 1 = its halves are done, emit the band
    while stack:
        idx, state = stack.pop()
        if state == 1:
            out.append(idx)
            continue
        if idx.size <= leaf:
            out.append(idx)
            continue
        xi, yj = ii[idx], jj[idx]
        x0, x1, y0, y1 = xi.min(), xi.max(), yj.min(), yj.max()
        key, lo, hi = (xi, x0, x1) if x1 - x0 >= y1 - y0 else (yj, y0, y1)
        c = (lo + hi) // 2
        a, b = idx[key < c], idx[key >= c + reach]
        if a.size == 0 or b.size == 0:
            out.append(idx)
            continue
        sep = idx[(key >= c) & (key < c + reach)]
        # popped in the order a, b, then the band
        stack.append((sep, 1))
        stack.append((b, 0))
        stack.append((a, 0))
    return np.concatenate(out) if out else np.zeros(0, np.int64)


def lu_solve(A, b, idx, w, kind):
    """x with A x = b (A symmetric positive definite, unknowns at flat
    indices idx of a width-w grid)."""
    n = idx.size
    if n < 20000:
        return spla.spsolve(A.tocsc(), b)
    p = nested_dissection(idx % w, idx // w, 2 if kind == 1 else 1)
    Ap = A[p][:, p].tocsc()
    lu = spla.splu(Ap, permc_spec="NATURAL", diag_pivot_thresh=0.0, options=dict(SymmetricMode=True))
    x = np.empty(n)
    x[p] = lu.solve(b[p])
    return x


def solve(g, f=None, kind=0):
    """FP64 solution image (h, w): g at the knowns, the exact solve at the unknowns."""
    g = np.asarray(g, dtype=np.float32)
    out = g.astype(np.float64).ravel().copy()
    A, b, idx = build_system(g, f, kind)
    if idx.size:
        out[idx] = lu_solve(A, b, idx, g.shape[1], kind)
    return out.reshape(g.shape)


def rel_residual64(u, g, f=None, kind=0):
    """||b - A u_U|| / ||b|| in float64 for an arbitrary (float or double) u."""
    A, b, idx = build_system(g, f, kind)
    if idx.size == 0:
        return 0.0
    x = np.asarray(u, np.float64).ravel()[idx]
    bn = np.linalg.norm(b)
    return float(np.linalg.norm(b - A @ x) / bn) if bn > 0 else 0.0
