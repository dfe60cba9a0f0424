"""CPU restatement of the AMG set-up's index work — test infrastructure only.

The device hierarchy of gcge_old_gb300/csrc/gcge_cuda_amg.cu has no counterpart
in the reference (the reference reaches an AMG through hypre, a third-party
library it does not contain, app/hypre/gcge_app_hypre.c:305-331), so this
restates the design's own rules, step by step, for the tests to check the
device result bit-exactly (aggregates are integer work):

* strength graph: the off-diagonal stored entries with a nonzero value and,
  for theta > 0, |a_ij| >= theta sqrt(|d_i d_j|), d the row's diagonal sum
  (`k_diag`, `k_strength`), in the row's entry order;
* distance-2 maximal independent set by iterated two-hop max-propagation of
  64-bit tuples (state << 62 | hash(i) & 0x3FFFFFFF << 32 | i), state 0 out,
  1 undecided, 2 in; an undecided row whose tuple is the largest within two
  hops joins, one that sees a joined tuple within two hops leaves
  (`k_mis_init`, `k_mis_max`, `k_mis_decide`);
* aggregates: roots numbered in row order; then twice, from a snapshot, every
  unaggregated row joins the aggregated neighbour with the largest
  (hash, index) tuple (`k_agg_roots`, `k_agg_join`); rows still alone become
  singletons numbered after the roots (`k_left_*`).

Only tests import this module.
"""
from __future__ import annotations

import numpy as np

MASK32 = np.uint64(0xFFFFFFFF)


def lowbias32(i: np.ndarray) -> np.ndarray:
    """The 32-bit integer finaliser of `amg_hash` (Wellons' "lowbias32")."""
    x = i.astype(np.uint64) & MASK32
    x ^= x >> np.uint64(16)
    x = (x * np.uint64(0x7FEB352D)) & MASK32
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x846CA68B)) & MASK32
    x ^= x >> np.uint64(16)
    return x


def tuples(state: np.ndarray, idx: np.ndarray) -> np.ndarray:
    h = lowbias32(idx) & np.uint64(0x3FFFFFFF)
    return (state.astype(np.uint64) << np.uint64(62)) | (h << np.uint64(32)) | idx.astype(np.uint64)


def diagonal(rowptr, col, val):
    n = len(rowptr) - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    d = np.zeros(n)
    np.add.at(d, rows[col == rows], val[col == rows])
    return d


def strength(rowptr, col, val, theta: float = 0.0):
    """(indptr, indices) of the strength graph, entries in row order."""
    n = len(rowptr) - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    d = diagonal(rowptr, col, val)
    keep = (col != rows) & (val != 0.0)
    if theta > 0.0:
        keep &= np.abs(val) >= theta * np.sqrt(np.abs(d[rows]) * np.abs(d[col]))
    counts = np.bincount(rows[keep], minlength=n)
    indptr = np.concatenate([[0], np.cumsum(counts)])
    return indptr, col[keep].astype(np.int64)


def _closed_max(indptr, indices, t):
    """out_i = max(t_i, max over i's strength neighbours of t_j)."""
    n = len(indptr) - 1
    out = t.copy()
    nb = t[indices]
    nonempty = np.diff(indptr) > 0
    if nb.size:
        starts = indptr[:-1][nonempty]
        red = np.maximum.reduceat(nb, starts)
        out[nonempty] = np.maximum(out[nonempty], red)
    return out


def mis2(indptr, indices, max_rounds: int = 200) -> np.ndarray:
    """States after the distance-2 MIS (2: root, 0: out)."""
    n = len(indptr) - 1
    idx = np.arange(n)
    state = np.ones(n, dtype=np.int64)
    t = tuples(state, idx)
    for _ in range(max_rounds):
        t2 = _closed_max(indptr, indices, _closed_max(indptr, indices, t))
        und = state == 1
        win = und & (t2 == t)
        lose = und & ~win & ((t2 >> np.uint64(62)) == np.uint64(2))
        state[win] = 2
        state[lose] = 0
        t = tuples(state, idx)
        if not np.any(state == 1):
            return state
    raise RuntimeError("distance-2 MIS did not settle")


def _join(indptr, indices, frm):
    """One join pass: an unaggregated row takes the aggregate of its aggregated
    neighbour with the largest (hash, index) tuple."""
    n = len(indptr) - 1
    agg = frm.copy()
    key = tuples(np.ones(n, dtype=np.int64), np.arange(n))
    for i in np.nonzero(frm < 0)[0]:
        nb = indices[indptr[i]:indptr[i + 1]]
        nb = nb[frm[nb] >= 0]
        if nb.size:
            agg[i] = frm[nb[np.argmax(key[nb])]]
    return agg


def aggregates(rowptr, col, val, theta: float = 0.0) -> np.ndarray:
    """The aggregate of every row, as the device set-up numbers them."""
    indptr, indices = strength(np.asarray(rowptr), np.asarray(col), np.asarray(val), theta)
    state = mis2(indptr, indices)
    roots = state == 2
    agg = np.where(roots, np.cumsum(roots) - 1, -1)
    agg = _join(indptr, indices, agg)
    agg = _join(indptr, indices, agg)
    left = agg < 0
    agg[left] = int(roots.sum()) + np.cumsum(left)[left] - 1
    return agg.astype(np.int64)


def mis2_properties(rowptr, col, val, theta: float = 0.0):
    """(roots pairwise more than two hops apart, every row within two hops of a
    root): the defining properties of a distance-2 maximal independent set."""
    indptr, indices = strength(np.asarray(rowptr), np.asarray(col), np.asarray(val), theta)
    state = mis2(indptr, indices)
    n = len(indptr) - 1
    roots = np.nonzero(state == 2)[0]
    import scipy.sparse as sp
    S = sp.csr_matrix((np.ones(len(indices)), indices, indptr), shape=(n, n))
    S = S + sp.identity(n, format="csr")
    S2 = (S @ S).tocsr()
    R = sp.csr_matrix((np.ones(len(roots)), (np.arange(len(roots)), roots)), shape=(len(roots), n))
    reach = (R @ S2).tocsr()
    independent = all(len(set(reach[r].indices) & set(roots)) == 1 for r in range(len(roots)))
    covered = np.asarray(reach.sum(axis=0)).ravel() > 0
    return independent, bool(covered.all())
