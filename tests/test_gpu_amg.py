"""The AMG hierarchy (GCGE_CUDA_AMG) and its W-step solver GCGE_CUDA_AMGPCG,
the GPU counterpart of the hypre app's BoomerAMG-preconditioned solvers behind
MultiLinearSolver (app/hypre/gcge_app_hypre.c:305-331, src/gcge_xpw.c:178-191).

The set-up is checked algebraically against scipy on the host: the
aggregates partition the rows, P is the damped-Jacobi-smoothed tentative
prolongation of those aggregates, R = P^T, and every coarse operator is the
Galerkin product P^T A P.  The V-cycle is checked as a symmetric, contracting
preconditioner, AMG-PCG against plain CG, and the W step by AMG-PCG against the
built-in block CG's eigenpairs."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from gcge_old_gb300 import lib as L
from gcge_old_gb300.matrices import diffusion27, initial_block, laplace3d_mass
from gcge_old_gb300.solver import AMG, DeviceMatrix, GCGESolver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def diff27():
    A, B = diffusion27(m=16, seed=5)  # n = 4096, exp(N(0,1)) cell coefficients
    return A, B


def _hierarchy_checks(A, amg):
    nlev = amg.num_levels
    assert nlev >= 2
    Al = A.to_scipy().tocsr()
    for l in range(nlev - 1):
        info = amg.level_info(l)
        agg = amg.aggregates(l)
        nagg = amg.level_info(l + 1)["n"]
        # a partition of the rows into nagg non-empty aggregates
        assert agg.min() == 0 and agg.max() == nagg - 1
        assert np.all(np.bincount(agg, minlength=nagg) > 0)
        assert nagg < info["n"]
        # P = (I - omega D^-1 A) T with T_{i, agg(i)} = 1, omega = 4 / (3 lmax)
        T = sp.csr_matrix((np.ones(info["n"]), (np.arange(info["n"]), agg)),
                          shape=(info["n"], nagg))
        omega = 4.0 / (3.0 * info["lmax"])
        Dinv = sp.diags(1.0 / Al.diagonal())
        P_ref = (T - omega * (Dinv @ (Al @ T))).tocsr()
        # rows of more than 256 stored entries keep their tentative row
        long_rows = np.diff(Al.indptr) > 256
        if long_rows.any():
            keep = sp.diags((~long_rows).astype(float))
            P_ref = (keep @ P_ref + sp.diags(long_rows.astype(float)) @ T).tocsr()
        P = amg.level_csr(l, "P")
        assert abs(P - P_ref).max() < 1e-13 * abs(P_ref).max()
        R = amg.level_csr(l, "R")
        assert abs(R - P.T).max() == 0.0
        # Galerkin operator
        Ac_ref = (P.T @ Al @ P).tocsr()
        Ac = amg.level_csr(l + 1, "A")
        assert abs(Ac - Ac_ref).max() < 1e-12 * abs(Ac_ref).max()
        # rows sorted by column (canonical order)
        for i in range(min(Ac.shape[0], 200)):
            cols = Ac.indices[Ac.indptr[i]:Ac.indptr[i + 1]]
            assert np.all(np.diff(cols) > 0)
        # the smoother's bound lies above the spectral radius of D^-1 A (power
        # iteration x 1.1), not far above it
        if info["n"] <= 5000:
            ev = np.linalg.eigvals((Dinv @ Al).toarray()).real.max()
            assert 0.999 * ev <= info["lmax"] <= 1.5 * ev, (ev, info["lmax"])
        Al = Ac_ref


def test_hierarchy_is_galerkin(cuda_lib, diff27):
    A, _ = diff27
    dA = DeviceMatrix(A)
    amg = AMG(dA, coarse_size=64)
    _hierarchy_checks(A, amg)
    # the coarsest level is small enough for its dense inverse
    assert amg.level_info(amg.num_levels - 1)["n"] <= 512
    amg.close()
    dA.close()


def test_hierarchy_with_strength_threshold(cuda_lib, diff27):
    A, _ = diff27
    dA = DeviceMatrix(A)
    amg = AMG(dA, coarse_size=64, strength=0.1)
    _hierarchy_checks(A, amg)
    amg.close()
    dA.close()


def test_plain_aggregation(cuda_lib, diff27):
    """smooth_p = 0: P is the tentative prolongation itself."""
    A, _ = diff27
    dA = DeviceMatrix(A)
    amg = AMG(dA, coarse_size=64, smooth_p=0)
    agg = amg.aggregates(0)
    P = amg.level_csr(0, "P")
    assert P.nnz == A.n and np.array_equal(P.indices, agg) and np.all(P.data == 1.0)
    Ac = amg.level_csr(1, "A")
    ref = (P.T @ A.to_scipy() @ P).tocsr()
    assert abs(Ac - ref).max() < 1e-12 * abs(ref).max()
    amg.close()
    dA.close()


def _apply(amg, B):
    from gpu_util import dev_cols, host
    bs, bp = dev_cols(B)
    xs, xp = dev_cols(np.zeros_like(B))
    lib = L.load()
    assert lib.GCGE_CUDA_AMG_Apply(amg.handle, bp, xp, B.shape[0], None) == 0, \
        lib.GCGE_CUDA_GetLastErrorMessage()
    from gpu_util import torch_cuda
    torch_cuda().cuda.synchronize()
    return host(xs)


def test_vcycle_symmetric_and_contracting(cuda_lib):
    A, _ = laplace3d_mass(24, seed=2)  # n = 13,824
    dA = DeviceMatrix(A)
    amg = AMG(dA)
    As = A.to_scipy()
    rng = np.random.default_rng(3)
    U = rng.standard_normal((2, A.n))
    MU = _apply(amg, U)
    # symmetric preconditioner: u^T M v = v^T M u (FP32 V-cycle)
    a, b = U[0] @ MU[1], U[1] @ MU[0]
    assert abs(a - b) < 1e-5 * np.sqrt(abs(U[0] @ MU[0]) * abs(U[1] @ MU[1])), (a, b)
    # positive definite on these vectors
    assert U[0] @ MU[0] > 0 and U[1] @ MU[1] > 0
    # stationary iteration x <- x + M (b - A x) contracts the A-norm error
    x_true = rng.standard_normal(A.n)
    rhs = As @ x_true
    x = np.zeros(A.n)
    err = []
    for _ in range(6):
        x = x + _apply(amg, (rhs - As @ x)[None, :])[0]
        e = x - x_true
        err.append(np.sqrt(e @ (As @ e)))
    rates = np.array(err[1:]) / np.array(err[:-1])
    assert rates.max() < 0.6, rates
    amg.close()
    dA.close()


def _pcg(lib, dA, amg_or_none, b, steps, rate):
    from gpu_util import dev_cols, host
    rs, rp = dev_cols(b)
    xs, xp = dev_cols(np.zeros_like(b))
    if amg_or_none is None:
        prm = L.ChebParam(steps, rate, 0, 0.05)  # diag(A)-preconditioned CG
        rc = lib.GCGE_CUDA_ChebyshevPCG(C.cast(C.pointer(prm), C.c_void_p), dA.handle, rp, xp,
                                        b.shape[0], dA.n, None)
    else:
        rc = lib.GCGE_CUDA_AMGPCG(amg_or_none.handle, dA.handle, rp, xp, b.shape[0], dA.n, None)
    assert rc == 0, lib.GCGE_CUDA_GetLastErrorMessage()
    return host(xs)


def test_amg_pcg_converges_much_faster_than_jacobi_pcg(cuda_lib):
    A, _ = diffusion27(m=32, seed=7)  # n = 32,768, coefficient jumps of e^{+-4}
    dA = DeviceMatrix(A)
    As = A.to_scipy()
    lib = L.load()
    rng = np.random.default_rng(1)
    b = rng.standard_normal((3, A.n))
    amg = AMG(dA, pcg_max_it=60, pcg_rate=1e-5)
    x = _pcg(lib, dA, amg, b, 60, 1e-5)
    steps_amg = amg.last_steps
    res = [np.linalg.norm(b[j] - As @ x[j]) / np.linalg.norm(b[j]) for j in range(3)]
    assert max(res) < 2e-5, res
    # diag(A)-preconditioned CG in FP64 after the same number of steps is far behind
    xj = _pcg(lib, dA, None, b, steps_amg, 1e-14)
    res_j = [np.linalg.norm(b[j] - As @ xj[j]) / np.linalg.norm(b[j]) for j in range(3)]
    assert min(res_j) > 100 * max(res), (res_j, res, steps_amg)
    assert steps_amg <= 30, steps_amg
    # a nonzero start: the FP64 residual of x0 is what gets reduced
    from gpu_util import dev_cols, host
    x0 = 0.5 * x
    rs, rp = dev_cols(b)
    xs, xp = dev_cols(x0)
    assert lib.GCGE_CUDA_AMGPCG(amg.handle, dA.handle, rp, xp, 3, dA.n, None) == 0
    x1 = host(xs)
    res1 = [np.linalg.norm(b[j] - As @ x1[j]) / np.linalg.norm(b[j]) for j in range(3)]
    assert max(res1) < 2e-5, res1
    amg.close()
    dA.close()


NEV = 8


def _solve(A, B, x0, setup=None, **kw):
    params = dict(ev_tol=1e-10, ev_max_it=300, precision="fp64")
    params.update(kw)
    s = GCGESolver(A, B, NEV, **params)
    try:
        if setup:
            setup(s)
        ev, _ = s.solve(x0)
        return ev, s.residuals(), s.stats()
    finally:
        s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_amg_w_step_matches_builtin_in_fewer_iterations(cuda_lib, precision):
    """At n = 110,592 the built-in block CG's 20 steps fall short on the
    coefficient jumps and the GCG iteration needs more outer steps; with the
    AMG-PCG W step it needs fewer, to the same eigenpairs (ev_tol 1e-11: both
    paths take different iterates, and the residual bound with a mass matrix of
    size h^3 leaves the eigenvalues free by more than the bound itself)."""
    A, B = diffusion27(m=48, seed=3)
    x0 = initial_block(A.n, NEV, seed=4)
    ev0, r0, st0 = _solve(A, B, x0, precision=precision, ev_tol=1e-11)
    ev1, r1, st1 = _solve(A, B, x0, precision=precision, ev_tol=1e-11,
                          setup=lambda s: s.use_amg_pcg())
    assert r0.max() < 1e-10 and r1.max() < 1e-10, (r0.max(), r1.max())
    np.testing.assert_allclose(ev1, ev0, rtol=1e-10)
    assert st1["num_iter"] < 0.8 * st0["num_iter"], (st1["num_iter"], st0["num_iter"])


def test_power_law_graph_stops_before_fill_in(cuda_lib):
    """On a power-law graph (hubs make every aggregate a neighbour of every other)
    the Galerkin operator fills in: at 300,000 nodes the first coarse operator
    would hold 13,863 rows and 169 M entries (a two-minute set-up).  The
    hierarchy stops coarsening before such a level, and AMG-PCG still reduces
    the residual."""
    import time
    A, B, _ = M_chung_lu(300000)
    dA = DeviceMatrix(A)
    t0 = time.time()
    amg = AMG(dA, pcg_max_it=80, pcg_rate=1e-3)
    assert time.time() - t0 < 60
    for l in range(amg.num_levels):
        info = amg.level_info(l)
        if info["n"] > 4096:
            assert info["nnz_a"] <= 0.3 * info["n"] ** 2, (l, info)
    lib = L.load()
    b = np.random.default_rng(2).standard_normal((2, A.n))
    x = _pcg(lib, dA, amg, b, 40, 1e-3)
    As = A.to_scipy()
    res = [np.linalg.norm(b[j] - As @ x[j]) / np.linalg.norm(b[j]) for j in range(2)]
    assert max(res) < 1e-2, res
    amg.close()
    dA.close()


def M_chung_lu(n):
    from gcge_old_gb300.matrices import chung_lu
    return chung_lu(n, seed=4)


def test_amg_w_step_diffusion27_workload_matches_oracle_port(cuda_lib):
    """The full-size 27-point workload (160^3, n = 4,096,000, nev 100) with the
    AMG-PCG W step in mixed precision at ev_tol 3e-12 (its iterates differ from
    the reference's, so the residual bound is set tighter than the reference's
    run): every eigenvalue within 1e-10 of the oracle port's solve
    (tests/golden/cfg3_port_summary.json), every pair at residual <= 1e-10, in
    far fewer GCG iterations than the port's 170."""
    import json
    import os
    from conftest import GOLDEN
    from gcge_old_gb300 import matrices as Mx
    from oracle import oracle as O
    path = os.path.join(GOLDEN, "cfg3_port_summary.json")
    if not os.path.exists(path):
        pytest.skip("no oracle summary of the 27-point workload")
    ref = json.load(open(path))
    A, B = Mx.diffusion27(160, seed=0)
    x0 = Mx.initial_block(A.n, 100, seed=0)
    s = GCGESolver(A, B, 100, ev_tol=3e-12, ev_max_it=1000, precision="mixed")
    try:
        s.use_amg_pcg()
        ev, vec = s.solve(x0)
        st = s.stats()
    finally:
        s.close()
    rel = np.abs(ev - np.array(ref["eval"])) / np.abs(np.array(ref["eval"]))
    assert rel.max() < 1e-10, rel.max()
    assert O.true_residuals(A, B, ev, vec).max() <= 1e-10
    assert st["num_iter"] < 0.5 * ref["iters"], st["num_iter"]


@pytest.mark.parametrize("make,theta", [("diffusion27", 0.0), ("diffusion27", 0.1),
                                        ("laplace3d_mass", 0.0), ("chung_lu", 0.0)])
def test_aggregates_match_the_oracle_exactly(cuda_lib, make, theta):
    """The device's distance-2 MIS aggregation is index work: on every level
    with a prolongation, its aggregates equal the CPU restatement's
    (oracle/amg_ref.py) exactly, computed from that level's operator."""
    from oracle import amg_ref as R
    from gcge_old_gb300.matrices import chung_lu
    A = {"diffusion27": lambda: diffusion27(m=20, seed=5)[0],
         "laplace3d_mass": lambda: laplace3d_mass(24, seed=2)[0],
         "chung_lu": lambda: chung_lu(5000, seed=6)[0]}[make]()
    dA = DeviceMatrix(A)
    amg = AMG(dA, coarse_size=32, strength=theta)
    Al = A.to_scipy().tocsr()
    for l in range(amg.num_levels - 1):
        ref = R.aggregates(Al.indptr, Al.indices, Al.data, theta)
        got = amg.aggregates(l)
        assert np.array_equal(got, ref), (l, int(np.sum(got != ref)))
        Al = amg.level_csr(l + 1, "A")
    amg.close()
    dA.close()


def test_amg_pcg_wider_than_32_columns(cuda_lib):
    """Blocks over 32 columns (a W step with a block size above 32) run 32
    columns at a time; every column reaches the residual target."""
    A, _ = laplace3d_mass(16, seed=4)
    dA = DeviceMatrix(A)
    amg = AMG(dA, pcg_max_it=60, pcg_rate=1e-4)
    lib = L.load()
    b = np.random.default_rng(5).standard_normal((40, A.n))
    x = _pcg(lib, dA, amg, b, 60, 1e-4)
    As = A.to_scipy()
    res = [np.linalg.norm(b[j] - As @ x[j]) / np.linalg.norm(b[j]) for j in range(40)]
    assert max(res) < 1e-3, max(res)
    amg.close()
    dA.close()
