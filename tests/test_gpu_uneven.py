"""Uneven rows: products and solves on a shifted power-law graph Laplacian
(seeded Chung-Lu graph, rows from 1 to thousands of entries), where rows of
more than 64 entries go through the chunked warp pass (gcge_cuda_heavy.cu)."""
import ctypes as C

import numpy as np
import pytest

from gcge_old_gb300 import matrices as M
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph():
    A, B, edges = M.chung_lu(50_000, seed=1)
    d = np.diff(A.rowptr)
    assert d.max() > 1000 and (d > 64).sum() > 100  # heavy rows present
    return A, B, edges


def test_spmm_f64_heavy_rows(cuda_lib, graph):
    import torch
    from gcge_old_gb300.solver import DeviceMatrix
    A = graph[0]
    rng = np.random.default_rng(0)
    k = 13
    X = torch.from_numpy(rng.standard_normal((k, A.n))).cuda()
    Y = torch.zeros_like(X)
    dA = DeviceMatrix(A)
    xp = (C.c_void_p * k)(*[C.c_void_p(X[j].data_ptr()) for j in range(k)])
    yp = (C.c_void_p * k)(*[C.c_void_p(Y[j].data_ptr()) for j in range(k)])
    assert cuda_lib.GCGE_CUDA_MatDotMultiVec(dA.handle, xp, yp, k) == 0
    ref = (A.to_scipy() @ X.cpu().numpy().T).T
    err = np.abs(Y.cpu().numpy() - ref).max() / np.abs(ref).max()
    assert err < 1e-13, err
    dA.close()


@pytest.mark.parametrize("k", [4, 13, 28])
def test_spmm_rows_f32_heavy_rows(cuda_lib, graph, k):
    import torch
    from gcge_old_gb300.solver import DeviceMatrix
    A = graph[0]
    kw = (k + 3) // 4 * 4
    rng = np.random.default_rng(k)
    Xc = rng.standard_normal((A.n, k)).astype(np.float32)
    Xr = np.zeros((A.n, kw), np.float32)
    Xr[:, :k] = Xc
    X = torch.from_numpy(Xr).cuda()
    Y = torch.zeros_like(X)
    dA = DeviceMatrix(A)
    assert cuda_lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(X.data_ptr()),
                                                 C.c_void_p(Y.data_ptr()), k, None) == 0
    torch.cuda.synchronize()
    ref = A.to_scipy() @ Xc.astype(np.float64)
    scale = np.abs(A.to_scipy()) @ np.abs(Xc.astype(np.float64))
    err = (np.abs(Y.cpu().numpy()[:, :k] - ref) / np.maximum(scale, 1e-30)).max()
    assert err < 1e-5, err
    dA.close()


def _edge_rows_matrix():
    """n = 3000 with empty rows (first and last among them), rows of exactly 64 and
    65 entries (either side of the heavy-row threshold), 256 and 257 entries (either
    side of a chunk boundary) and one row holding every column."""
    from gcge_old_gb300.matrices import CSRMatrix
    n = 3000
    rng = np.random.default_rng(7)
    lens = rng.integers(0, 9, n)
    lens[[0, 17, 1500, n - 1]] = 0
    lens[[5, 6]] = [64, 65]
    lens[[100, 101, 102]] = [256, 257, 513]
    lens[2000] = n
    cols = [np.sort(rng.choice(n, L, replace=False)) for L in lens]
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate(cols).astype(np.int32)
    val = rng.uniform(-1.0, 1.0, rp[-1])
    return CSRMatrix(n, rp, ci, val)


@pytest.mark.parametrize("k", [1, 8, 13])
def test_spmm_edge_rows(cuda_lib, k):
    import torch
    from gcge_old_gb300.solver import DeviceMatrix
    A = _edge_rows_matrix()
    rng = np.random.default_rng(k)
    dA = DeviceMatrix(A)
    # FP64 columns
    X = torch.from_numpy(rng.standard_normal((k, A.n))).cuda()
    Y = torch.full_like(X, float("nan"))
    xp = (C.c_void_p * k)(*[C.c_void_p(X[j].data_ptr()) for j in range(k)])
    yp = (C.c_void_p * k)(*[C.c_void_p(Y[j].data_ptr()) for j in range(k)])
    assert cuda_lib.GCGE_CUDA_MatDotMultiVec(dA.handle, xp, yp, k) == 0
    ref = (A.to_scipy() @ X.cpu().numpy().T).T
    scale = (abs(A.to_scipy()) @ np.abs(X.cpu().numpy().T)).T
    got = Y.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert (np.abs(got - ref) <= 2e-14 * np.maximum(scale, 1e-300)).all()
    assert (got[:, [0, 17, 1500, A.n - 1]] == 0).all()  # empty rows give exact zeros
    # FP32 row-interleaved blocks
    kw = (k + 3) // 4 * 4
    Xr = np.zeros((A.n, kw), np.float32)
    Xr[:, :k] = rng.standard_normal((A.n, k))
    Xd = torch.from_numpy(Xr).cuda()
    Yd = torch.full_like(Xd, float("nan"))
    assert cuda_lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(Xd.data_ptr()),
                                                 C.c_void_p(Yd.data_ptr()), k, None) == 0
    torch.cuda.synchronize()
    got = Yd.cpu().numpy()[:, :k]
    ref = A.to_scipy() @ Xr[:, :k].astype(np.float64)
    scale = abs(A.to_scipy()) @ np.abs(Xr[:, :k].astype(np.float64))
    assert (np.abs(got - ref) <= 1e-5 * np.maximum(scale, 1e-30)).all()
    assert (got[[0, 17, 1500, A.n - 1]] == 0).all()
    dA.close()


@pytest.mark.parametrize("fp32", [0, 1])
def test_block_cg_heavy_rows(cuda_lib, fp32):
    """The column block CG (GCGE_CUDA_BlockCG, FP64 and FP32) on a power-law graph:
    the same step count and iterate as the oracle's restatement of GCGE_BCG.  The shift
    (100) keeps the system well conditioned: with the 1e-3 shift of the solver
    tests, 20 CG steps turn one-ulp differences in the products (the heavy rows
    are summed chunk-wise, in another order than a row loop) into differences of
    about 1e-2 in the iterate, in the oracle itself."""
    from gcge_old_gb300.solver import DeviceMatrix
    from gpu_util import dev_cols, host
    from oracle import ops_ref as R
    A = M.chung_lu(50_000, seed=1, shift=100.0)[0]
    assert (np.diff(A.rowptr) > 64).sum() > 100
    k = 13
    rng = np.random.default_rng(8)
    rhs = rng.standard_normal((k, A.n))
    x0 = rng.standard_normal((k, A.n)) * 0.1
    rs, rp = dev_cols(rhs)
    xs, xp = dev_cols(x0)
    dA = DeviceMatrix(A)
    steps = C.c_int(0)
    assert cuda_lib.GCGE_CUDA_BlockCG(dA.handle, rp, xp, k, A.n, 20, 1e-2, fp32,
                                      C.byref(steps)) == 0
    X, _, niter = R.block_cg(A, rhs, x0, 20, 1e-2)
    got = host(xs)
    if not fp32:
        assert steps.value == niter
        np.testing.assert_allclose(got, X, rtol=0, atol=1e-7 * np.abs(X).max())
    else:
        # FP32 columns and values: the same stopping rule.  The iterates are not
        # compared: one-ulp changes of the FP64 products already move the
        # oracle's own iterate by 1e-8 here (an amplification of ~1e7), so FP32
        # rounding moves it by O(1e-2); the residual bound below is the check.
        assert abs(steps.value - niter) <= 2
    a = A.to_scipy()
    for j in range(k):
        r0 = np.linalg.norm(rhs[j] - a @ x0[j])
        bound = 1e-2 * r0 * (1.05 if fp32 else 1.0001)
        assert np.linalg.norm(rhs[j] - a @ got[j]) <= bound or steps.value == 20
    dA.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nev,bs", [(16, 10), (40, 36)])
def test_solve_hub_localised_power_law_graph(cuda_lib, precision, nev, bs):
    """A shifted power-law graph (shift 100, 117 heavy rows) whose lowest
    eigenvectors sit on hub nodes, against the oracle port: block size 10 (the
    mixed solve on row-interleaved FP32 blocks) and 36 (above their 32 columns:
    the FP32 column block CG).  The mixed W step hands the FP32 correction
    alone to the orthogonalisation; with w0 + e the mixed solve broke down on
    this problem (spurious eigenvalues near 1e-6)."""
    from gcge_old_gb300 import solver as S
    A, B, _ = M.chung_lu(5000, seed=2, shift=100.0)
    assert (np.diff(A.rowptr) > 64).sum() > 100
    x0 = M.initial_block(A.n, nev, seed=3)
    kw = dict(ev_tol=1e-8, ev_max_it=150, block_size=bs)
    ev, vec, st = S.solve(A, B, nev, x0, precision=precision, **kw)
    ref = O.port_solve(A, B, nev, x0, O.default_para(nev, **kw), threads=8)
    assert np.max(np.abs(ev - ref["eval"]) / np.abs(ref["eval"])) < 1e-9
    crit = O.true_residuals(A, B, ev, vec) * np.abs(ev) / np.maximum(1.0, np.abs(ev))
    assert crit.max() < 1.5e-8, crit


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solve_power_law_graph(cuda_lib, precision):
    from gcge_old_gb300 import solver as S
    A, B, _ = M.chung_lu(20_000, seed=2)
    nev = 16
    x0 = M.initial_block(A.n, nev, seed=3)
    ev, vec, st = S.solve(A, B, nev, x0, ev_tol=1e-10, ev_max_it=500, precision=precision)
    ref = O.port_solve(A, B, nev, x0, O.default_para(nev, ev_tol=1e-10, ev_max_it=500),
                       threads=4)
    assert np.max(np.abs(ev - ref["eval"]) / np.abs(ref["eval"])) < 1e-9
    # the reference's criterion ||A x - lambda B x|| / (||x|| max(1, |lambda|)): the
    # smallest eigenvalue (~ shift n / sum(d)) is far below 1 here
    crit = O.true_residuals(A, B, ev, vec) * np.abs(ev) / np.maximum(1.0, np.abs(ev))
    assert crit.max() < 2e-10, crit


def test_edge_weight_gradient(cuda_lib):
    """dlambda_k / dw_e = (x_i - x_j)^2 - lambda_k (x_i^2 + x_j^2) on an edge (i, j)
    (A = L + shift I, B = D), assembled from the CSR-value adjoints of A and B."""
    import torch
    from gcge_old_gb300.autograd import eigvals_csr
    A, B, (i, j, w, pos) = M.chung_lu(3_000, seed=4)
    nev = 8
    x0 = M.initial_block(A.n, nev, seed=5)
    a = torch.tensor(A.val, requires_grad=True)
    b = torch.tensor(B.val, requires_grad=True)
    lam = eigvals_csr(a, A, nev, x0, b_val=b, B_pattern=B, ev_tol=1e-12, ev_max_it=2000,
                      precision="fp64")
    lam[nev - 1].backward()
    p_ij, p_ji, p_ii, p_jj, bi, bj = pos
    ga, gb = a.grad.numpy(), b.grad.numpy()
    gw = -ga[p_ij] - ga[p_ji] + ga[p_ii] + ga[p_jj] + gb[bi] + gb[bj]
    rng = np.random.default_rng(6)
    for e in rng.choice(len(w), 3, replace=False):
        h = 1e-4 * w[e]

        def lam_at(dw):
            av, bv = A.val.copy(), B.val.copy()
            av[[p_ij[e], p_ji[e]]] -= dw
            av[[p_ii[e], p_jj[e]]] += dw
            bv[[bi[e], bj[e]]] += dw
            with torch.no_grad():
                l = eigvals_csr(torch.from_numpy(av), A, nev, x0, b_val=torch.from_numpy(bv),
                                B_pattern=B, ev_tol=1e-12, ev_max_it=2000, precision="fp64")
            return float(l[nev - 1])

        fd = (lam_at(h) - lam_at(-h)) / (2 * h)
        assert abs(fd - gw[e]) <= 1e-6 * max(abs(gw[e]), 1e-3 * np.abs(gw).max()), (e, fd, gw[e])
