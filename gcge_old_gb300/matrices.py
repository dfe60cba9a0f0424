"""Seeded synthetic problem generators for the GCG eigensolver workloads.

Every generator returns a :class:`CSRMatrix` (0-based int32 ``rowptr`` and
``col``, float64 ``val``, columns sorted within each row: the layout of the
reference's ``CSR_MAT``, app/csr/gcge_app_csr.h:27-41) or ``None`` for B = I.
The same arrays feed the CUDA solver, the oracle port and the reference
oracle, so all three see bit-identical inputs.

Workloads (sizes given as defaults, every generator takes a smaller grid for
tests):

* ``laplace2d``      5-point Dirichlet Laplacian [4; -1 x4] on an m x m
                     interior grid, B = I.                 (n = 16,384 at m=128)
* ``laplace3d_mass`` 7-point Laplacian scaled by h (h = 1/(m+1)) and a
                     diagonal lumped mass h^3 (1 + U(-0.1, 0.1)).
                                                           (n = 2,097,152 at m=128)
* ``diffusion27``    trilinear (Q1) finite-element stiffness with per-cell
                     coefficient exp(N(0,1)) on an m^3 interior grid, kept in
                     its full 27-point pattern, and the Q1 consistent mass
                     (centre 8/27, face 2/27, edge 1/54, corner 1/216) h^3.
                                                           (n = 4,096,000 at m=160)
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CSRMatrix:
    n: int
    rowptr: np.ndarray  # int32, n+1
    col: np.ndarray     # int32, nnz
    val: np.ndarray     # float64, nnz

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.rowptr), shape=(self.n, self.n))

    @staticmethod
    def from_scipy(m) -> "CSRMatrix":
        m = m.tocsr()
        m.sort_indices()
        return CSRMatrix(m.shape[0], np.ascontiguousarray(m.indptr, dtype=np.int32),
                         np.ascontiguousarray(m.indices, dtype=np.int32),
                         np.ascontiguousarray(m.data, dtype=np.float64))

    def matvec(self, x: np.ndarray) -> np.ndarray:
        return self.to_scipy() @ x


def _tridiag(m: int, diag: float, off: float):
    import scipy.sparse as sp
    e = np.ones(m)
    return sp.diags([off * e[:-1], diag * e, off * e[:-1]], [-1, 0, 1], format="csr")


def laplace2d(m: int = 128) -> CSRMatrix:
    """5-point stencil [4; -1 x 4] on an m x m interior grid (Dirichlet)."""
    import scipy.sparse as sp
    t = _tridiag(m, 2.0, -1.0)
    i = sp.identity(m, format="csr")
    return CSRMatrix.from_scipy(sp.kron(i, t) + sp.kron(t, i))


def laplace3d(m: int) -> CSRMatrix:
    """Unscaled 7-point stencil [6; -1 x 6] on an m^3 interior grid."""
    import scipy.sparse as sp
    t = _tridiag(m, 2.0, -1.0)
    i = sp.identity(m, format="csr")
    a = sp.kron(sp.kron(i, i), t) + sp.kron(sp.kron(i, t), i) + sp.kron(sp.kron(t, i), i)
    return CSRMatrix.from_scipy(a)


def diag_matrix(d: np.ndarray) -> CSRMatrix:
    n = d.shape[0]
    return CSRMatrix(n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32),
                     np.ascontiguousarray(d, dtype=np.float64))


def laplace3d_mass(m: int = 128, seed: int = 0):
    """A = h * 7-point Laplacian, B = diag(h^3 (1 + U(-0.1, 0.1))), h = 1/(m+1)."""
    h = 1.0 / (m + 1)
    a = laplace3d(m)
    a.val *= h
    rng = np.random.default_rng(seed)
    b = diag_matrix(h ** 3 * (1.0 + rng.uniform(-0.1, 0.1, size=m ** 3)))
    return a, b


def _q1_assemble(m: int, cell_coef: np.ndarray | None, weights) -> CSRMatrix:
    """Assemble a 27-point operator on the m^3 interior nodes of an (m+1)^3
    cell grid.  ``weights[d]`` is the element-matrix entry for two vertices
    that differ in d coordinates; node-pair entries sum over the shared cells,
    weighted by ``cell_coef`` (or 1)."""
    nc = m + 1
    if cell_coef is None:
        cell_coef = np.ones((nc, nc, nc))
    idx = np.arange(m)
    rows, cols, vals = [], [], []
    node = lambda x, y, z: (z * m + y) * m + x
    X, Y, Z = np.meshgrid(idx, idx, idx, indexing="ij")
    for oz in (-1, 0, 1):
        for oy in (-1, 0, 1):
            for ox in (-1, 0, 1):
                d = abs(ox) + abs(oy) + abs(oz)
                # cells shared by node p=(x,y,z) (interior index) and p+o: node
                # interior index i sits at grid point i+1; a cell c touches grid
                # points c..c+1 per axis.  Shared cells per axis: offset 0 ->
                # {i, i+1}; offset +1 -> {i+1}; offset -1 -> {i}.
                sx = [0, 1] if ox == 0 else ([1] if ox > 0 else [0])
                sy = [0, 1] if oy == 0 else ([1] if oy > 0 else [0])
                sz = [0, 1] if oz == 0 else ([1] if oz > 0 else [0])
                xs, ys, zs = X + ox, Y + oy, Z + oz
                valid = (xs >= 0) & (xs < m) & (ys >= 0) & (ys < m) & (zs >= 0) & (zs < m)
                acc = np.zeros((m, m, m))
                for cx in sx:
                    for cy in sy:
                        for cz in sz:
                            acc += cell_coef[cx:cx + m, cy:cy + m, cz:cz + m]
                v = acc * weights[d]
                rows.append(node(X, Y, Z)[valid])
                cols.append(node(xs, ys, zs)[valid])
                vals.append(v[valid])
    import scipy.sparse as sp
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    v = np.concatenate(vals)
    a = sp.coo_matrix((v, (r, c)), shape=(m ** 3, m ** 3)).tocsr()
    # keep structural zeros (face entries of the Q1 stiffness are exactly 0)
    a.sum_duplicates()
    return CSRMatrix.from_scipy(a)


def diffusion27(m: int = 160, seed: int = 0):
    """Q1 FE stiffness with per-cell kappa = exp(N(0,1)) and the Q1 consistent
    mass, both scaled for grid spacing h = 1/(m+1), full 27-point pattern."""
    h = 1.0 / (m + 1)
    rng = np.random.default_rng(seed)
    kappa = np.exp(rng.standard_normal((m + 1, m + 1, m + 1)))
    # trilinear element stiffness / h: d=0: 1/3, d=1: 0, d=2: -1/12, d=3: -1/12
    a = _q1_assemble(m, kappa, [h / 3.0, 0.0, -h / 12.0, -h / 12.0])
    # trilinear element mass: h^3/216 * (8, 4, 2, 1)
    b = _q1_assemble(m, None, [h ** 3 * 8 / 216, h ** 3 * 4 / 216, h ** 3 * 2 / 216, h ** 3 / 216])
    return a, b


def aniso2d(m: int = 512, seed: int = 0, ratio: float = 10.0):
    """2D anisotropic diffusion, 5-point, on the m x m interior nodes of an
    (m+1) x (m+1) cell grid with per-cell kappa ~ U(0.5, 2): the conductance of
    an edge is the mean kappa of the two cells beside it, times ``ratio`` for
    y-edges; edges to the Dirichlet boundary only add to the diagonal.
    B = diag(h^2 (1 + U(-0.1, 0.1))), h = 1/(m+1).

    Returns (A, B, S, kappa) with A.val = S @ kappa: S (nnz x (m+1)^2, CSR) is
    the linear map from cell coefficients to the stored values of A, for
    gradients with respect to kappa."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    nc = m + 1
    kappa = rng.uniform(0.5, 2.0, nc * nc)
    n = m * m
    # edges between grid points; interior node (r, c) is grid point (r+1, c+1),
    # index r*m + c; cell (a, b) has its lower-left corner at grid point (a, b)
    A_, B_ = np.meshgrid(np.arange(m), np.arange(m + 1), indexing="ij")
    # x-edges: grid row a+1, grid columns b -> b+1; cells (a, b) and (a+1, b)
    xi = np.where(B_ >= 1, A_ * m + B_ - 1, -1)
    xj = np.where(B_ < m, A_ * m + B_, -1)
    xc1, xc2 = A_ * nc + B_, (A_ + 1) * nc + B_
    # y-edges: grid rows a -> a+1, grid column b+1; cells (a, b) and (a, b+1)
    Ay, By = np.meshgrid(np.arange(m + 1), np.arange(m), indexing="ij")
    yi = np.where(Ay >= 1, (Ay - 1) * m + By, -1)
    yj = np.where(Ay < m, Ay * m + By, -1)
    yc1, yc2 = Ay * nc + By, Ay * nc + By + 1
    ei = np.concatenate([xi.ravel(), yi.ravel()])
    ej = np.concatenate([xj.ravel(), yj.ravel()])
    c1 = np.concatenate([xc1.ravel(), yc1.ravel()])
    c2 = np.concatenate([xc2.ravel(), yc2.ravel()])
    w = np.concatenate([np.ones(xi.size), np.full(yi.size, ratio)]) / 2.0
    rows, cols, cells, vals = [], [], [], []
    for p_, q_ in ((ei, ej), (ej, ei)):
        d = p_ >= 0                      # diagonal of each interior endpoint
        o = d & (q_ >= 0)                # coupling of two interior endpoints
        for c in (c1, c2):
            rows += [p_[d], p_[o]]
            cols += [p_[d], q_[o]]
            cells += [c[d], c[o]]
            vals += [w[d], -w[o]]
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    key, ent = np.unique(rows * n + cols, return_inverse=True)
    S = sp.csr_matrix((np.concatenate(vals), (ent, np.concatenate(cells))),
                      shape=(len(key), nc * nc))
    S.sum_duplicates()
    r = key // n
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rowptr, r + 1, 1)
    rowptr = np.cumsum(rowptr)
    A = CSRMatrix(n, rowptr.astype(np.int32), (key % n).astype(np.int32), S @ kappa)
    h = 1.0 / (m + 1)
    B = diag_matrix(h * h * (1.0 + rng.uniform(-0.1, 0.1, n)))
    return A, B, S, kappa


def chung_lu(n: int = 8_000_000, mean_deg: float = 16.0, gamma: float = 2.5, seed: int = 0,
             shift: float = 1e-3):
    """Shifted graph Laplacian of a seeded Chung-Lu power-law graph.

    Expected degrees w_i = c (n / (i + 1))^(1 / (gamma - 1)); mean_deg - 2 of
    the mean degree comes from n (mean_deg - 2) / 2 edges whose endpoints are
    drawn with probability proportional to w (self-loops dropped, repeated
    pairs merged), the other 2 from a random recursive tree (node i joins a
    uniform earlier node), which keeps the graph connected so that B = D is
    positive definite.  Node labels are then shuffled.  Edge weights
    U(0.5, 1.5).  A = L + shift I (L = D - W), B = D.

    Returns (A, B, edges) with edges = (i, j, w, pos) for the undirected edges
    i < j: pos = (A index of (i, j), of (j, i), of (i, i), of (j, j), B index of
    i, of j), for gradients with respect to the edge weights."""
    rng = np.random.default_rng(seed)
    t = 1.0 / (gamma - 1.0)
    w = (n / np.arange(1, n + 1, dtype=np.float64)) ** t
    w *= (mean_deg - 2.0) * n / w.sum()
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    m = int(round(n * (mean_deg - 2.0) / 2.0))
    a = np.searchsorted(cdf, rng.random(m), side="right")
    b = np.searchsorted(cdf, rng.random(m), side="right")
    np.minimum(a, n - 1, out=a)
    np.minimum(b, n - 1, out=b)
    tree_child = np.arange(1, n, dtype=np.int64)
    tree_parent = np.floor(rng.random(n - 1) * tree_child).astype(np.int64)
    i = np.concatenate([np.minimum(a, b), np.minimum(tree_child, tree_parent)])
    j = np.concatenate([np.maximum(a, b), np.maximum(tree_child, tree_parent)])
    keep = i != j
    key = np.sort(i[keep] * n + j[keep])
    key = key[np.concatenate([[True], key[1:] != key[:-1]])]
    perm = rng.permutation(n)
    i, j = perm[key // n], perm[key % n]
    i, j = np.minimum(i, j), np.maximum(i, j)
    wt = rng.uniform(0.5, 1.5, len(i))
    deg = np.bincount(i, weights=wt, minlength=n) + np.bincount(j, weights=wt, minlength=n)
    m = len(i)
    rows = np.concatenate([i, j, np.arange(n)])
    cols = np.concatenate([j, i, np.arange(n)])
    vals = np.concatenate([-wt, -wt, deg + shift])
    order = np.argsort(rows * n + cols, kind="stable")
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    rowptr = np.zeros(n + 1, dtype=np.int64)
    rowptr[1:] = np.cumsum(np.bincount(rows, minlength=n))
    Ac = CSRMatrix(n, rowptr.astype(np.int32), cols[order].astype(np.int32), vals[order])
    B = diag_matrix(deg)
    p_ij, p_ji, p_d = inv[:m], inv[m:2 * m], inv[2 * m:]
    p_ii, p_jj = p_d[i], p_d[j]
    return Ac, B, (i, j, wt, (p_ij, p_ji, p_ii, p_jj, i, j))


def initial_block(n: int, nev: int, seed: int = 0) -> np.ndarray:
    """Seeded N(0,1) initial block, column-major n x nev (shape (nev, n) in C
    order, so column j is ``x0[j]``)."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((nev, n))


def read_csr_text(path: str) -> CSRMatrix:
    """Reader for the reference's CSR text format (app/csr/gcge_app_csr.c:185-236):
    ``nrow ncol nnz`` then ``rowptr[n+1]``, ``col[nnz]``, ``val[nnz]``, 0-based."""
    with open(path) as f:
        tok = f.read().split()
    nrow, ncol, nnz = int(tok[0]), int(tok[1]), int(tok[2])
    p = 3
    rowptr = np.array(tok[p:p + nrow + 1], dtype=np.int64); p += nrow + 1
    col = np.array(tok[p:p + nnz], dtype=np.int64); p += nnz
    val = np.array(tok[p:p + nnz], dtype=np.float64)
    assert ncol == nrow
    import scipy.sparse as sp
    m = sp.csr_matrix((val, col, rowptr), shape=(nrow, ncol))
    return CSRMatrix.from_scipy(m)
