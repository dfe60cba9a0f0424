"""Eigenvalue adjoint (GCGE_CUDA_EigGradCSR behind torch.autograd): against a
dense generalized-eigenproblem reference and against finite differences, on a
seeded 2D anisotropic diffusion problem with a diagonal mass matrix."""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

from gcge_old_gb300.matrices import CSRMatrix, initial_block

pytestmark = pytest.mark.gpu


def aniso_problem(m=20, seed=5):
    """5-point anisotropic diffusion on an m x m interior grid: per-edge
    conductivities U(0.5, 2), y-direction weighted 10x; diagonal mass."""
    rng = np.random.default_rng(seed)
    n = m * m
    idx = np.arange(n).reshape(m, m)
    rows, cols, vals = [], [], []
    diag = np.zeros(n)

    def edge(i, j, w):
        rows.extend([i, j]); cols.extend([j, i]); vals.extend([-w, -w])
        diag[i] += w; diag[j] += w

    for a in range(m):
        for b in range(m):
            if b + 1 < m:
                edge(idx[a, b], idx[a, b + 1], rng.uniform(0.5, 2.0))
            if a + 1 < m:
                edge(idx[a, b], idx[a + 1, b], 10.0 * rng.uniform(0.5, 2.0))
            # boundary (Dirichlet) contributions keep A positive definite
            diag[idx[a, b]] += (b == 0) + (b == m - 1) + 10.0 * ((a == 0) + (a == m - 1))
    A = sp.csr_matrix((vals + list(diag), (rows + list(range(n)), cols + list(range(n)))),
                      shape=(n, n))
    A.sum_duplicates()
    A.sort_indices()
    B = sp.diags(rng.uniform(0.9, 1.1, n)).tocsr()
    return CSRMatrix.from_scipy(A), CSRMatrix.from_scipy(B)


def _setup(nev=10):
    import torch
    A, B = aniso_problem()
    x0 = initial_block(A.n, nev, seed=1)
    w = np.random.default_rng(2).uniform(0, 1, nev)
    a = torch.tensor(A.val, dtype=torch.float64, requires_grad=True)
    b = torch.tensor(B.val, dtype=torch.float64, requires_grad=True)
    return torch, A, B, x0, w, a, b


PARAMS = dict(ev_tol=1e-12, ev_max_it=2000, precision="fp64")


def test_eigenvalue_gradient_matches_dense_adjoint(cuda_lib):
    from gcge_old_gb300.autograd import eigvals_csr
    torch, A, B, x0, w, a, b = _setup()
    nev = len(w)
    lam = eigvals_csr(a, A, nev, x0, b_val=b, B_pattern=B, **PARAMS)
    loss = (torch.from_numpy(w) * lam).sum()
    loss.backward()
    ev, X = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray())  # B-normalised
    np.testing.assert_allclose(lam.detach().numpy(), ev[:nev], rtol=1e-10)
    Asp, Bsp = A.to_scipy().tocoo(), B.to_scipy().tocoo()
    gA = sum(w[k] * X[Asp.row, k] * X[Asp.col, k] for k in range(nev))
    gB = -sum(w[k] * ev[k] * X[Bsp.row, k] * X[Bsp.col, k] for k in range(nev))
    # the CSR value order equals scipy's coo order of a sorted CSR matrix
    np.testing.assert_allclose(a.grad.numpy(), gA, rtol=0, atol=1e-8 * np.abs(gA).max())
    np.testing.assert_allclose(b.grad.numpy(), gB, rtol=0, atol=1e-8 * np.abs(gB).max())


def test_eigenvalue_gradient_matches_finite_differences(cuda_lib):
    from gcge_old_gb300.autograd import eigvals_csr
    torch, A, B, x0, w, a, b = _setup()
    nev = len(w)
    lam = eigvals_csr(a, A, nev, x0, b_val=b, B_pattern=B, **PARAMS)
    (torch.from_numpy(w) * lam).sum().backward()

    def loss(av, bv):
        with torch.no_grad():
            l = eigvals_csr(torch.from_numpy(av), A, nev, x0, b_val=torch.from_numpy(bv),
                            B_pattern=B, **PARAMS)
        return float((w * l.numpy()).sum())

    rng = np.random.default_rng(7)
    Asp = A.to_scipy().tocoo()
    offd = np.flatnonzero(Asp.row < Asp.col)
    for e in rng.choice(offd, 3, replace=False):
        i, j = Asp.row[e], Asp.col[e]
        e2 = np.flatnonzero((Asp.row == j) & (Asp.col == i))[0]  # the symmetric twin
        h = 1e-4 * abs(A.val[e])
        ap, am = A.val.copy(), A.val.copy()
        ap[[e, e2]] += h
        am[[e, e2]] -= h
        fd = (loss(ap, B.val) - loss(am, B.val)) / (2 * h)
        an = float(a.grad[e] + a.grad[e2])
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3 * abs(float(a.grad.abs().max()))), (fd, an)
    for e in rng.choice(B.nnz, 2, replace=False):
        h = 1e-4 * abs(B.val[e])
        bp, bm = B.val.copy(), B.val.copy()
        bp[e] += h
        bm[e] -= h
        fd = (loss(A.val, bp) - loss(A.val, bm)) / (2 * h)
        an = float(b.grad[e])
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
