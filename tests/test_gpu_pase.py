"""The multilevel eigensolver (GCGE_CUDA_PASE_Solve), the GPU form of the
reference's PASE add-on (pase/src/pase_solver.c): the pairs it returns are
checked against the GCG solver's pairs of the same problem (and against the
closed form for the 2D Laplacian), with every pair at relative residual
below the tolerance in an FP64 check on the host and B-orthonormal vectors."""
import numpy as np
import pytest

from gcge_old_gb300 import matrices as M
from gcge_old_gb300 import solver as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _b_orth(B, X):
    BX = np.stack([B.to_scipy() @ x for x in X]) if B is not None else X
    return np.abs(X @ BX.T - np.eye(len(X))).max()


@pytest.mark.parametrize("make", ["diffusion27", "laplace3d_mass"])
def test_pase_matches_gcg(cuda_lib, make):
    A, B = M.diffusion27(24, seed=3) if make == "diffusion27" else M.laplace3d_mass(32, seed=5)
    nev = 12
    ev, vec, st = S.pase_solve(A, B, nev, tol=1e-10)
    x0 = M.initial_block(A.n, nev, seed=9)
    ref, _, _ = S.solve(A, B, nev, x0, ev_tol=1e-12, ev_max_it=500)
    np.testing.assert_allclose(ev, ref, rtol=1e-9)
    res = O.true_residuals(A, B, ev, vec)
    assert res.max() < 1e-10, (res.max(), st)
    assert _b_orth(B, vec) < 1e-9
    assert 1 <= st["cycles"] <= 60 and st["max_residual"] < 1e-10


def test_pase_identity_mass_closed_form(cuda_lib):
    m, nev = 64, 8
    A = M.laplace2d(m)
    ev, vec, st = S.pase_solve(A, None, nev, tol=1e-10)
    t = 2.0 - 2.0 * np.cos(np.arange(1, m + 1) * np.pi / (m + 1))
    exact = np.sort((t[:, None] + t[None, :]).ravel())[:nev]
    np.testing.assert_allclose(ev, exact, rtol=1e-9)
    assert O.true_residuals(A, None, ev, vec).max() < 1e-10


def test_pase_deeper_auxiliary_level(cuda_lib):
    """The auxiliary space on level 2 (two prolongations, B carried down twice)."""
    A, B = M.laplace3d_mass(40, seed=6)
    dA = S.DeviceMatrix(A)
    amg = S.AMG(dA, coarse_size=64)
    if amg.num_levels < 3 or amg.level_info(2)["n"] < 60:
        pytest.skip("hierarchy too shallow for a level-2 auxiliary space")
    nev = 8
    ev, vec, st = S.pase_solve(dA, B, nev, amg=amg, aux_level=2, more_nev=4, tol=1e-10,
                               max_cycles=60)
    x0 = M.initial_block(A.n, nev, seed=2)
    ref, _, _ = S.solve(A, B, nev, x0, ev_tol=1e-12, ev_max_it=500)
    np.testing.assert_allclose(ev, ref, rtol=1e-9)
    assert O.true_residuals(A, B, ev, vec).max() < 1e-10
    amg.close()


def test_pase_rejects_bad_parameters(cuda_lib):
    A, B = M.laplace3d_mass(12, seed=1)
    with pytest.raises(Exception, match="PASE"):
        S.pase_solve(A, B, 4, aux_level=0)
    with pytest.raises(Exception, match="PASE"):
        S.pase_solve(A, B, 4, tol=-1.0)


def test_pase_leaves_the_hierarchy_settings(cuda_lib):
    """The smoothing runs AMG-PCG with its own step count; the hierarchy's
    settings are back afterwards (an AMG-PCG call then runs its own 7 steps)."""
    import ctypes as C
    from gpu_util import dev_cols
    from gcge_old_gb300 import lib as L
    A, B = M.laplace3d_mass(24, seed=3)
    dA = S.DeviceMatrix(A)
    amg = S.AMG(dA, pcg_max_it=7, pcg_rate=1e-12)
    S.pase_solve(dA, B, 6, amg=amg, more_nev=4, tol=1e-10)
    lib = L.load()
    rs, rp = dev_cols(np.random.default_rng(0).standard_normal((2, A.n)))
    xs, xp = dev_cols(np.zeros((2, A.n)))
    assert lib.GCGE_CUDA_AMGPCG(amg.handle, dA.handle, rp, xp, 2, A.n, None) == 0
    assert amg.last_steps == 7
    amg.close()
    dA.close()
