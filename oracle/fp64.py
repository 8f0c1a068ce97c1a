"""FP64 converged solve of the simpois CG systems (scipy sparse direct).

TEST INFRASTRUCTURE ONLY (the checker).  Builds, for one channel, the system
the reference's CG solves (cleant_cgpois.c:197-264):

* kind 0: A = -Lap restricted to the unknowns, 5-point stencil with
  clamp-to-edge (cleant_cgpois.c:67-89); b = -f_U + Lap_UK g_K.
* kind 1: A = the 13-point bilaplacian with a single clamp
  (cleant_cgpois.c:91-121); b = -f_U - A_UK g_K.

and solves it with ``scipy.sparse.linalg.spsolve`` in float64.  The result is
the "FP64 converged solve" every GPU result is compared against.
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


def solve(g, f=None, kind=0):
    """FP64 solution image (h, w): g at the knowns, the exact solve at the unknowns."""
    g = np.asarray(g, dtype=np.float32)
    out = g.astype(np.float64).ravel().copy()
    A, b, idx = build_system(g, f, kind)
    if idx.size:
        out[idx] = spla.spsolve(A.tocsc(), b)
    return out.reshape(g.shape)


def rel_residual64(u, g, f=None, kind=0):
    """||b - A u_U|| / ||b|| in float64 for an arbitrary (float or double) u."""
    A, b, idx = build_system(g, f, kind)
    if idx.size == 0:
        return 0.0
    x = np.asarray(u, np.float64).ravel()[idx]
    bn = np.linalg.norm(b)
    return float(np.linalg.norm(b - A @ x) / bn) if bn > 0 else 0.0
