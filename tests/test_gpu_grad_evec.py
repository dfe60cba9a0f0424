"""Eigenvector losses (GCGE_CUDA_EigvecAdjointSolve + GCGE_CUDA_EigGradCSR2 behind
gcge_old_gb300.autograd.eigpairs_csr): against a dense generalized-eigenproblem
adjoint built from all n eigenpairs, against central differences of the GPU
solver, and through a linear coefficient-to-matrix map (per-cell kappa of the
2D anisotropic diffusion problem)."""
import numpy as np
import pytest
import scipy.linalg as sla

from gcge_old_gb300.matrices import aniso2d, initial_block

pytestmark = pytest.mark.gpu

NEV = 8
PARAMS = dict(ev_tol=1e-12, ev_max_it=2000, precision="fp64")


def signed(V):
    """Rows flipped so that the entry of largest magnitude is positive."""
    idx = np.abs(V).argmax(axis=1)
    return V * np.sign(V[np.arange(len(V)), idx])[:, None]


@pytest.fixture(scope="module")
def prob():
    A, B, S, kappa = aniso2d(m=14, seed=3)  # n = 196
    rng = np.random.default_rng(11)
    return dict(A=A, B=B, S=S, kappa=kappa, x0=initial_block(A.n, NEV, seed=1),
                w=rng.uniform(0, 1, NEV), mask=(rng.uniform(size=A.n) < 0.3).astype(float),
                q=rng.standard_normal(A.n))


def loss_np(ev, X, p):
    """sum_k w_k lambda_k + ||x_1 * mask||^2 + (q . x_3)^2 (sign-invariant in x)."""
    return float((p["w"] * ev).sum() + ((X[0] * p["mask"]) ** 2).sum() + (X[2] @ p["q"]) ** 2)


def loss_t(lam, X, p):
    import torch
    w, m, q = (torch.from_numpy(p[k]).to(lam.device) for k in ("w", "mask", "q"))
    return (w * lam).sum() + ((X[0] * m) ** 2).sum() + (X[2] @ q) ** 2


def run(p, a_val, b_val):
    from gcge_old_gb300.autograd import eigpairs_csr
    return eigpairs_csr(a_val, p["A"], NEV, p["x0"], b_val=b_val, B_pattern=p["B"], **PARAMS)


def test_eigpairs_forward_matches_dense(cuda_lib, prob):
    import torch
    A, B = prob["A"], prob["B"]
    lam, X = run(prob, torch.from_numpy(A.val), torch.from_numpy(B.val))
    ev, V = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray())
    np.testing.assert_allclose(lam.numpy(), ev[:NEV], rtol=1e-10)
    np.testing.assert_allclose(X.numpy(), signed(V[:, :NEV].T), atol=1e-8)


def test_eigenvector_adjoint_matches_dense(cuda_lib, prob):
    """Dense reference: mu_k = sum over all j != k of x_j (x_j^T g_k) / (lambda_j - lambda_k)
    from the full dense eigendecomposition of (A, B)."""
    import torch
    A, B = prob["A"], prob["B"]
    a = torch.tensor(A.val, requires_grad=True)
    b = torch.tensor(B.val, requires_grad=True)
    lam, X = run(prob, a, b)
    loss_t(lam, X, prob).backward()

    ev, V = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray())
    V = V.T.copy()
    V[:NEV] = signed(V[:NEV])
    g = np.zeros((NEV, A.n))
    g[0] = 2 * prob["mask"] ** 2 * V[0]
    g[2] = 2 * (V[2] @ prob["q"]) * prob["q"]
    mu = np.zeros((NEV, A.n))
    for k in (0, 2):
        d = ev - ev[k]
        d[k] = np.inf
        mu[k] = ((V @ g[k]) / d) @ V
    Asp, Bsp = A.to_scipy().tocoo(), B.to_scipy().tocoo()
    w = prob["w"]
    gA = sum(w[k] * V[k][Asp.row] * V[k][Asp.col] - mu[k][Asp.row] * V[k][Asp.col]
             for k in range(NEV))
    gB = sum(-w[k] * ev[k] * V[k][Bsp.row] * V[k][Bsp.col]
             + ev[k] * mu[k][Bsp.row] * V[k][Bsp.col]
             - 0.5 * (g[k] @ V[k]) * V[k][Bsp.row] * V[k][Bsp.col] for k in range(NEV))
    np.testing.assert_allclose(a.grad.numpy(), gA, rtol=0, atol=1e-8 * np.abs(gA).max())
    np.testing.assert_allclose(b.grad.numpy(), gB, rtol=0, atol=1e-8 * np.abs(gB).max())


def test_eigenvector_adjoint_matches_finite_differences(cuda_lib, prob):
    import torch
    A, B = prob["A"], prob["B"]
    a = torch.tensor(A.val, requires_grad=True)
    b = torch.tensor(B.val, requires_grad=True)
    lam, X = run(prob, a, b)
    loss_t(lam, X, prob).backward()

    def f(av, bv):
        with torch.no_grad():
            l, Y = run(prob, torch.from_numpy(av), torch.from_numpy(bv))
        return loss_np(l.numpy(), Y.numpy(), prob)

    rng = np.random.default_rng(5)
    Asp = A.to_scipy().tocoo()
    offd = np.flatnonzero(Asp.row < Asp.col)
    scale = float(a.grad.abs().max())
    for e in rng.choice(offd, 3, replace=False):
        i, j = Asp.row[e], Asp.col[e]
        e2 = np.flatnonzero((Asp.row == j) & (Asp.col == i))[0]
        h = 1e-4 * abs(A.val[e])
        ap, am = A.val.copy(), A.val.copy()
        ap[[e, e2]] += h
        am[[e, e2]] -= h
        fd = (f(ap, B.val) - f(am, B.val)) / (2 * h)
        an = float(a.grad[e] + a.grad[e2])
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3 * scale), (fd, an)
    for e in rng.choice(B.nnz, 3, replace=False):
        h = 1e-4 * abs(B.val[e])
        bp, bm = B.val.copy(), B.val.copy()
        bp[e] += h
        bm[e] -= h
        fd = (f(A.val, bp) - f(A.val, bm)) / (2 * h)
        an = float(b.grad[e])
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-3 * float(b.grad.abs().max())), (fd, an)


def test_gradient_through_cell_coefficients(cuda_lib, prob):
    """kappa -> A values is linear (A.val = S kappa); torch carries the chain rule
    from the CSR-value gradient to kappa."""
    import torch
    S = prob["S"].tocoo()
    St = torch.sparse_coo_tensor(np.vstack([S.row, S.col]), S.data, S.shape)
    kap = torch.tensor(prob["kappa"], requires_grad=True)
    a_val = torch.sparse.mm(St, kap[:, None])[:, 0]
    lam, X = run(prob, a_val, torch.from_numpy(prob["B"].val))
    loss_t(lam, X, prob).backward()
    g = kap.grad.numpy()

    def f(kv):
        with torch.no_grad():
            l, Y = run(prob, torch.from_numpy(prob["S"] @ kv), torch.from_numpy(prob["B"].val))
        return loss_np(l.numpy(), Y.numpy(), prob)

    rng = np.random.default_rng(9)
    for c in rng.choice(len(g), 4, replace=False):
        h = 1e-4 * prob["kappa"][c]
        kp, km = prob["kappa"].copy(), prob["kappa"].copy()
        kp[c] += h
        km[c] -= h
        fd = (f(kp) - f(km)) / (2 * h)
        assert abs(fd - g[c]) <= 1e-6 * max(abs(g[c]), 1e-3 * np.abs(g).max()), (c, fd, g[c])


def test_adjoint_rejects_bad_arguments(cuda_lib, prob):
    import ctypes as C
    from gcge_old_gb300 import lib as L
    lib = L.load()
    ev = np.array([1.0, 1.0])
    assert lib.GCGE_CUDA_EigvecAdjointSolve(None, None, None, ev.ctypes.data_as(L.c_double_p), 2,
                                            None, None, None, 10, 1e-8, None) == 1
    assert lib.GCGE_CUDA_EigvecAdjointSolveAMG(None, None, None, ev.ctypes.data_as(L.c_double_p),
                                               2, None, None, None, 10, 1e-8, None, None) == 1


def test_eigenvector_adjoint_amg_matches_jacobi(cuda_lib):
    """The projected CG preconditioned by an AMG V-cycle of A (adjoint_amg=True)
    gives the gradients of the Jacobi-preconditioned solve in fewer steps."""
    import torch
    from gcge_old_gb300 import autograd as AG
    A, B, _, _ = aniso2d(m=96, seed=5)  # n = 9216
    nev = 8
    x0 = initial_block(A.n, nev, seed=2)
    rng = np.random.default_rng(4)
    mask = torch.from_numpy((rng.uniform(size=A.n) < 0.3).astype(float))
    q = torch.from_numpy(rng.standard_normal(A.n))
    out = {}
    for amg in (None, True):
        a = torch.tensor(A.val, requires_grad=True)
        b = torch.tensor(B.val, requires_grad=True)
        lam, X = AG.eigpairs_csr(a, A, nev, x0, b_val=b, B_pattern=B, adjoint_amg=amg, **PARAMS)
        (((X[0] * mask) ** 2).sum() + (X[2] @ q) ** 2).backward()
        out[amg] = (a.grad.numpy(), b.grad.numpy(), dict(AG.last_adjoint))
    (ga_j, gb_j, st_j), (ga_a, gb_a, st_a) = out[None], out[True]
    assert st_j["preconditioner"] == "jacobi" and st_a["preconditioner"] == "amg"
    assert st_a["columns"] == st_j["columns"] == 2
    np.testing.assert_allclose(ga_a, ga_j, rtol=0, atol=1e-7 * np.abs(ga_j).max())
    np.testing.assert_allclose(gb_a, gb_j, rtol=0, atol=1e-7 * np.abs(gb_j).max())
    assert st_a["steps"] <= st_j["steps"] / 2, (st_a, st_j)


def test_eigenvector_adjoint_amg_rejects_another_size(cuda_lib, prob):
    """A hierarchy whose finest level is not A's size is an argument error."""
    import ctypes as C
    from gcge_old_gb300 import lib as L
    from gcge_old_gb300 import solver as S
    lib = L.load()
    A2, _, _, _ = aniso2d(m=20, seed=1)
    dA2 = S.DeviceMatrix(A2)
    amg = S.AMG(dA2)
    dA = S.DeviceMatrix(prob["A"])
    ev = np.arange(1.0, NEV + 1.0)
    xs = (C.c_void_p * NEV)()
    assert lib.GCGE_CUDA_EigvecAdjointSolveAMG(dA.handle, None, xs,
                                               ev.ctypes.data_as(L.c_double_p), NEV, xs, xs,
                                               None, 10, 1e-8, None, amg.handle) == 1
    assert "finest level" in lib.GCGE_CUDA_GetLastErrorMessage().decode()
    amg.close()
    dA.close()
    dA2.close()
