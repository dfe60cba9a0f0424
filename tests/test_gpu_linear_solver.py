"""The MultiLinearSolver hook (GCGE_OPS.MultiLinearSolver, src/gcge_ops.h:77,
called at src/gcge_xpw.c:178-191): a user block solver for the W step in place
of the built-in block CG, and the stock GPU solver GCGE_CUDA_JacobiPCG behind
it.  Eigenvalues with the hook match the built-in path's to the solve tolerance;
a failing callback fails the solve; fn=NULL restores the built-in path."""
import ctypes as C

import numpy as np
import pytest

from gcge_old_gb300 import lib as L
from gcge_old_gb300.matrices import diffusion27, initial_block
from gcge_old_gb300.solver import GCGESolver

pytestmark = pytest.mark.gpu

NEV = 8
PARAMS = dict(ev_tol=1e-10, ev_max_it=300, precision="fp64")


@pytest.fixture(scope="module")
def problem():
    A, B = diffusion27(m=20, seed=3)  # n = 8000, exp(N(0,1)) coefficients, consistent mass
    return A, B, initial_block(A.n, NEV, seed=4)


def _solve(A, B, x0, setup=None, **kw):
    s = GCGESolver(A, B, NEV, **{**PARAMS, **kw})
    try:
        if setup:
            setup(s)
        ev, _ = s.solve(x0)
        return ev, s.residuals(), s.stats()
    finally:
        s.close()


def test_jacobi_pcg_matches_builtin(cuda_lib, problem):
    A, B, x0 = problem
    ev0, r0, _ = _solve(A, B, x0)
    ev1, r1, st = _solve(A, B, x0, setup=lambda s: s.use_jacobi_pcg(max_it=30, rate=1e-2))
    assert r0.max() < 1e-10 and r1.max() < 1e-10, (r0, r1)
    np.testing.assert_allclose(ev1, ev0, rtol=1e-9)


def test_python_callback_sees_the_block(cuda_lib, problem):
    """A callback written in Python gets k <= block size columns of length n on the
    solver's stream, and may delegate to the stock solver."""
    A, B, x0 = problem
    calls = []
    prm = L.PCGParam(30, 1e-2)
    lib = L.load()

    @L.MultiLinearSolver
    def cb(ctx, mat, rhs, x, k, n, stream):
        calls.append((k, n))
        return lib.GCGE_CUDA_JacobiPCG(C.cast(C.pointer(prm), C.c_void_p), mat, rhs, x, k, n,
                                       stream)

    ev, r, _ = _solve(A, B, x0, setup=lambda s: s.set_linear_solver(cb))
    assert calls and all(n == A.n and 1 <= k <= NEV for k, n in calls), calls[:5]
    assert r.max() < 1e-10
    ev0, _, _ = _solve(A, B, x0)
    np.testing.assert_allclose(ev, ev0, rtol=1e-9)


def test_failing_callback_fails_the_solve(cuda_lib, problem):
    A, B, x0 = problem

    @L.MultiLinearSolver
    def bad(ctx, mat, rhs, x, k, n, stream):
        return 7

    with pytest.raises(L.GcgeCudaError, match="linear solver returned 7"):
        _solve(A, B, x0, setup=lambda s: s.set_linear_solver(bad))


def test_null_restores_builtin(cuda_lib, problem):
    A, B, x0 = problem

    @L.MultiLinearSolver
    def bad(ctx, mat, rhs, x, k, n, stream):
        return 1

    def setup(s):
        s.set_linear_solver(bad)
        s.set_linear_solver(None)

    ev, r, _ = _solve(A, B, x0, setup=setup)
    assert r.max() < 1e-10


def test_jacobi_pcg_direct(cuda_lib):
    """GCGE_CUDA_JacobiPCG alone on a diagonally dominant system: k columns, each
    reaches the requested relative residual."""
    import torch
    from gcge_old_gb300.solver import DeviceMatrix
    A, _ = diffusion27(m=16, seed=1)
    n, k = A.n, 5
    rng = np.random.default_rng(0)
    b = torch.from_numpy(rng.standard_normal((k, n))).cuda()
    x = torch.zeros((k, n), dtype=torch.float64, device="cuda")
    rhs = b.clone()
    dA = DeviceMatrix(A)
    bp = (C.c_void_p * k)(*[C.c_void_p(rhs[j].data_ptr()) for j in range(k)])
    xp = (C.c_void_p * k)(*[C.c_void_p(x[j].data_ptr()) for j in range(k)])
    prm = L.PCGParam(500, 1e-8)
    L.check(L.load().GCGE_CUDA_JacobiPCG(C.cast(C.pointer(prm), C.c_void_p), dA.handle, bp, xp,
                                         k, n, None), "JacobiPCG")
    torch.cuda.synchronize()
    As = A.to_scipy()
    xs, bs = x.cpu().numpy(), b.cpu().numpy()
    for j in range(k):
        res = np.linalg.norm(bs[j] - As @ xs[j]) / np.linalg.norm(bs[j])
        assert res < 1e-7, (j, res)
    dA.close()


def _residual_after(lib, A, b, steps, degree, rate=1e-14):
    """||b - A x|| / ||b|| after `steps` Chebyshev-PCG steps from x = 0."""
    from gpu_util import dev_cols, host
    from gcge_old_gb300.solver import DeviceMatrix
    dA = DeviceMatrix(A)
    rs, rp = dev_cols(b[None, :].copy())
    xs, xp = dev_cols(np.zeros((1, A.n)))
    prm = L.ChebParam(steps, rate, degree, 0.05)
    rc = lib.GCGE_CUDA_ChebyshevPCG(C.cast(C.pointer(prm), C.c_void_p), dA.handle, rp, xp, 1, A.n,
                                    None)
    assert rc == 0, lib.GCGE_CUDA_GetLastErrorMessage()
    x = host(xs)[0]
    return np.linalg.norm(b - A.to_scipy() @ x) / np.linalg.norm(b)


def test_chebyshev_preconditioner_reduces_the_residual_faster(cuda_lib, problem):
    """On the log-normal-coefficient 27-point matrix the polynomial preconditioner
    takes the residual further in the same number of CG steps than diag(A)
    alone, and the solve converges to the target."""
    A, _, _ = problem
    b = np.random.default_rng(0).standard_normal(A.n)
    r_jac = _residual_after(cuda_lib, A, b, 12, 0)
    r_cheb = _residual_after(cuda_lib, A, b, 12, 4)
    assert r_cheb < 0.5 * r_jac, (r_cheb, r_jac)
    assert _residual_after(cuda_lib, A, b, 200, 4, rate=1e-10) < 1e-10


def test_chebyshev_pcg_w_step_matches_builtin(cuda_lib, problem):
    """The W step by ChebyshevPCG (device-resident step scalars) gives the
    built-in block CG's eigenpairs to the solve tolerance."""
    A, B, x0 = problem
    ev0, r0, st0 = _solve(A, B, x0)
    ev1, r1, st1 = _solve(A, B, x0, setup=lambda s: s.use_chebyshev_pcg(max_it=40, rate=1e-3,
                                                                       degree=4))
    assert r0.max() < 1e-10 and r1.max() < 1e-10, (r0, r1)
    np.testing.assert_allclose(ev1, ev0, rtol=1e-9)
    assert st1["num_iter"] <= st0["num_iter"] + 2, (st1["num_iter"], st0["num_iter"])
