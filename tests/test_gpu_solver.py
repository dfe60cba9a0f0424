"""GPU parity of the whole GCG solve through the C ABI: against the golden
outputs of the reference (tests/golden/), against the oracle port on fresh
seeds, and edge cases.  Eigenvalues must agree to 1e-10 relative, every
returned pair must reach the residual the reference reached, and
eigenvectors are compared by B-principal angles per eigenvalue cluster."""
import numpy as np
import pytest

from conftest import GOLDEN_NAMES, load_golden
from gcge_old_gb300 import matrices as M
from gcge_old_gb300 import solver as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

EV_RTOL = 1e-10


def gpu_params(flags, precision):
    p = {"precision": precision}
    for k, v in flags.items():
        if k == "fixed_shift":
            p["if_shift"], p["shift"] = 1, float(v)
        elif k in ("eval_type", "conv_type"):
            p[k] = v
        else:
            p[k] = int(v) if k in ("block_size", "ev_max_it", "cg_max_it", "use_shift") else float(v)
    return p


def b_orthonormality(B, X):
    b = B.to_scipy() if B is not None else None
    BX = np.stack([b @ x for x in X]) if b is not None else X
    return np.abs(X @ BX.T - np.eye(len(X))).max()


def cluster_angles(ev, X, Y, B, gap=1e-8):
    """Largest sine of the B-principal angles between span(X_c), span(Y_c)
    over clusters c of eigenvalues closer than gap (relative)."""
    b = B.to_scipy() if B is not None else None
    worst = 0.0
    i = 0
    while i < len(ev):
        j = i + 1
        while j < len(ev) and abs(ev[j] - ev[j - 1]) <= gap * abs(ev[j]):
            j += 1
        Xc, Yc = X[i:j], Y[i:j]
        BY = np.stack([b @ y for y in Yc]) if b is not None else Yc
        s = np.linalg.svd(Xc @ BY.T, compute_uv=False)
        worst = max(worst, float(np.sqrt(max(0.0, 1.0 - min(s.min(), 1.0) ** 2))))
        i = j
    return worst


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_solver_matches_reference_golden(cuda_lib, name, precision):
    A, B, nev, x0, d = load_golden(name)
    ev, vec, st = S.solve(A, B, nev, x0, **gpu_params(d["flags_dict"], precision))
    rel = np.abs(ev - d["eval"]) / np.abs(d["eval"])
    assert rel.max() < EV_RTOL, (rel.max(), st)
    tr = O.true_residuals(A, B, ev, vec)
    if "evec" in d:
        tr_ref = O.true_residuals(A, B, d["eval"], d["evec"])
    else:  # the reference's "R" values are divided by max(1, |lambda|), not |lambda|
        lam = np.abs(d["eval"])
        tr_ref = d["res"] * np.maximum(1.0, lam) / lam
    assert tr.max() <= max(10 * tr_ref.max(), 1e-13), (tr.max(), tr_ref.max())
    assert b_orthonormality(B, vec) < 1e-10
    if "evec" in d:
        assert cluster_angles(ev, vec, d["evec"], B) < 1e-5
    if precision == "fp64":
        assert abs(st["num_iter"] - int(d["iters"])) <= 2, (st["num_iter"], int(d["iters"]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_vs_oracle_port_fresh_seed(cuda_lib, precision):
    A, B = M.laplace3d_mass(16, seed=42)
    nev = 16
    x0 = M.initial_block(A.n, nev, seed=77)
    ev, vec, st = S.solve(A, B, nev, x0, ev_tol=1e-10, ev_max_it=200, precision=precision)
    ref = O.port_solve(A, B, nev, x0, O.default_para(nev, ev_tol=1e-10, ev_max_it=200), threads=4)
    assert np.max(np.abs(ev - ref["eval"]) / ref["eval"]) < EV_RTOL
    assert O.true_residuals(A, B, ev, vec).max() < 1e-10
    assert cluster_angles(ev, vec, ref["evec"], B) < 1e-5


def test_solver_identity_b_equals_no_b(cuda_lib):
    A = M.laplace2d(20)
    nev = 10
    x0 = M.initial_block(A.n, nev, seed=1)
    I = M.diag_matrix(np.ones(A.n))
    e1, v1, _ = S.solve(A, None, nev, x0, ev_tol=1e-12, ev_max_it=100)
    e2, v2, _ = S.solve(A, I, nev, x0, ev_tol=1e-12, ev_max_it=100)
    np.testing.assert_allclose(e1, e2, rtol=1e-12)


def test_solver_single_eigenpair(cuda_lib):
    A, B = M.laplace3d_mass(10, seed=3)
    x0 = M.initial_block(A.n, 1, seed=2)
    ev, vec, st = S.solve(A, B, 1, x0, ev_tol=1e-10, ev_max_it=200)
    import scipy.sparse.linalg as sla
    w = sla.eigsh(A.to_scipy(), k=1, M=B.to_scipy(), sigma=0, which="LM")[0]
    assert abs(ev[0] - w[0]) / w[0] < 1e-10


def test_solver_stops_at_max_iterations(cuda_lib):
    A = M.laplace2d(64)
    x0 = M.initial_block(A.n, 12, seed=8)
    ev, vec, st = S.solve(A, None, 12, x0, ev_tol=1e-14, ev_max_it=3)
    assert st["num_iter"] == 3
    assert np.all(np.isfinite(ev))


def test_solver_without_inner_cg(cuda_lib):
    """cg_max_it = 1: W is the scaled X (the block CG does no step)."""
    A = M.laplace2d(16)
    x0 = M.initial_block(A.n, 10, seed=4)
    ev, vec, st = S.solve(A, None, 10, x0, ev_tol=1e-6, ev_max_it=400, cg_max_it=1)
    assert np.all(np.isfinite(ev))


def test_solver_rejects_bad_arguments(cuda_lib):
    A = M.laplace2d(4)
    with pytest.raises(Exception):
        S.GCGESolver(A, None, 40)  # nev larger than n
    with pytest.raises(Exception):
        S.GCGESolver(A, None, 2, no_such_parameter=1)


def test_solver_nonfinite_input_returns(cuda_lib):
    """A NaN in the matrix must not hang the device: the solve ends at
    ev_max_it (or with an error status)."""
    A = M.laplace2d(12)
    A.val = A.val.copy()
    A.val[7] = np.nan
    x0 = M.initial_block(A.n, 4, seed=3)
    try:
        ev, vec, st = S.solve(A, None, 4, x0, ev_tol=1e-10, ev_max_it=5)
        assert st["num_iter"] <= 5
    except Exception as e:  # an error status is an acceptable outcome
        assert "Solve" in str(e)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_solver_headline_workload_matches_reference(cuda_lib, precision):
    """The full-size workload (128^3 7-point Laplacian with diagonal mass,
    nev 50, 1e-10): eigenvalues against the reference's own run
    (tests/golden/cfg2_reference_summary.json) to 1e-10 relative, every pair
    at relative residual <= 1e-10 (FP64 post-check), B-orthonormal vectors."""
    import json
    import os
    from conftest import GOLDEN
    ref = json.load(open(os.path.join(GOLDEN, "cfg2_reference_summary.json")))
    A, B = M.laplace3d_mass(128, seed=0)
    x0 = M.initial_block(A.n, 50, seed=0)
    ev, vec, st = S.solve(A, B, 50, x0, ev_tol=1e-10, ev_max_it=1000, precision=precision)
    rel = np.abs(ev - np.array(ref["eval"])) / np.abs(np.array(ref["eval"]))
    assert rel.max() < EV_RTOL, rel.max()
    assert O.true_residuals(A, B, ev, vec).max() <= 1e-10
    assert b_orthonormality(B, vec) < 1e-9
    assert abs(st["num_iter"] - ref["iters"]) <= 5


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_solver_diffusion27_workload_matches_oracle_port(cuda_lib, precision):
    """The full-size 27-point workload (160^3 Q1 diffusion with log-normal
    cell coefficients and its consistent mass, n = 4,096,000, nev 100) at
    ev_tol 1e-11: eigenvalues against the oracle port's solve of the same
    matrices and start (tests/golden/cfg3_port_summary.json, ev_tol 1e-11) to
    1e-10 relative per pair, every pair at relative residual <= 1e-10."""
    import json
    import os
    from conftest import GOLDEN
    path = os.path.join(GOLDEN, "cfg3_port_summary.json")
    if not os.path.exists(path):
        pytest.skip("no oracle summary of the 27-point workload")
    ref = json.load(open(path))
    A, B = M.diffusion27(160, seed=0)
    x0 = M.initial_block(A.n, 100, seed=0)
    ev, vec, st = S.solve(A, B, 100, x0, ev_tol=1e-11, ev_max_it=1000, precision=precision)
    rel = np.abs(ev - np.array(ref["eval"])) / np.abs(np.array(ref["eval"]))
    assert rel.max() < EV_RTOL, rel.max()
    assert O.true_residuals(A, B, ev, vec).max() <= 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_nev128_analytic(cuda_lib, precision):
    """nev = 128 (a 198-column basis: the projected matrices and the Cholesky
    of the initial block no longer fit in one CTA's shared memory) on the 2D
    Laplacian, whose eigenvalues are known in closed form."""
    m, nev = 100, 128
    A = M.laplace2d(m)
    t = 2.0 - 2.0 * np.cos(np.arange(1, m + 1) * np.pi / (m + 1))
    exact = np.sort((t[:, None] + t[None, :]).ravel())[:nev]
    x0 = M.initial_block(A.n, nev, seed=11)
    ev, vec, st = S.solve(A, None, nev, x0, ev_tol=1e-10, ev_max_it=400, precision=precision)
    np.testing.assert_allclose(ev, exact, rtol=1e-9)
    crit = O.true_residuals(A, None, ev, vec) * np.abs(ev) / np.maximum(1.0, np.abs(ev))
    assert crit.max() < 2e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_rank_deficient_initial_block(cuda_lib, precision):
    """Dependent and zero columns in the given block are dropped by the
    orthonormalisation and replaced by pseudo-random ones (the reference's
    completion of a short initial block); the solve then finds the same pairs."""
    A, B = M.laplace3d_mass(12, seed=1)
    nev = 8
    x0 = M.initial_block(A.n, nev, seed=5)
    x0[3] = x0[1]
    x0[5] = 2.0 * x0[1] - x0[2]
    x0[6] = 0.0
    ev, vec, st = S.solve(A, B, nev, x0, ev_tol=1e-10, ev_max_it=300, precision=precision)
    import scipy.linalg as sla
    ref = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray(), eigvals_only=True)[:nev]
    np.testing.assert_allclose(ev, ref, rtol=1e-9)
    assert O.true_residuals(A, B, ev, vec).max() < 1e-9


def test_solver_indefinite_b_returns(cuda_lib):
    """An indefinite B (negative diagonal entries) breaks the B-orthonormalisation:
    the solve must end with a status or at ev_max_it, never hang."""
    A = M.laplace2d(12)
    d = np.ones(A.n)
    d[::7] = -1.0
    B = M.diag_matrix(d)
    x0 = M.initial_block(A.n, 4, seed=3)
    try:
        ev, vec, st = S.solve(A, B, 4, x0, ev_tol=1e-10, ev_max_it=5)
        assert st["num_iter"] <= 5
    except Exception as e:  # an error status is an acceptable outcome
        assert "Solve" in str(e)


def test_random_start_with_omega_criterion(cuda_lib):
    """num_init_evec = 0: the start block is pseudo-random (src/gcge_eigsol.c:134-140),
    and the "O" criterion takes its omega norm from that block (:141-177).  The
    pairs found are the reference's (golden fixture from another start)."""
    A, B, nev, x0, d = load_golden("ref_diff27_m10_nev10")
    s = S.GCGESolver(A, B, nev, num_init_evec=0, conv_type="O", ev_tol=1e-12, ev_max_it=300)
    try:
        ev, vec = s.solve()
        res = s.residuals()
    finally:
        s.close()
    rel = np.abs(ev - d["eval"]) / np.abs(d["eval"])
    assert rel.max() < EV_RTOL, rel.max()
    assert res.max() < 1e-12
    assert O.true_residuals(A, B, ev, vec).max() < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_partial_start_block(cuda_lib, precision):
    """num_init_evec < nev: the given columns first, pseudo-random ones after."""
    A, B = M.laplace3d_mass(12, seed=1)
    nev = 10
    x0 = M.initial_block(A.n, nev, seed=5)
    ev, vec, st = S.solve(A, B, nev, x0, num_init_evec=4, ev_tol=1e-11, ev_max_it=300,
                          precision=precision)
    import scipy.linalg as sla
    ref = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray(), eigvals_only=True)[:nev]
    np.testing.assert_allclose(ev, ref, rtol=1e-10)


def test_fp64_correction_w_form(cuda_lib):
    """-gcge_w_form correction: the FP64 block CG hands the correction e to the
    W orthogonalisation instead of w0 + e (the mixed form's W step in FP64);
    same pairs as the reference."""
    A, B, nev, x0, d = load_golden("ref_lap3d_m12_nev12")
    ev, vec, st = S.solve(A, B, nev, x0, w_form="correction",
                          **gpu_params(d["flags_dict"], "fp64"))
    rel = np.abs(ev - d["eval"]) / np.abs(d["eval"])
    assert rel.max() < EV_RTOL, rel.max()
    assert O.true_residuals(A, B, ev, vec).max() < 1e-9
    assert st["num_iter"] <= int(d["iters"]) + 3


def test_final_report_in_reference_layout(cuda_lib, capfd):
    """print_result / print_conv / print_final_part_time write the report of
    GCGE_PrintFinalInfo (src/gcge_para.c:577-699) to stdout."""
    A, B, nev, x0, d = load_golden("ref_lap2d_m32_nev10")
    capfd.readouterr()
    ev, vec, st = S.solve(A, B, nev, x0, print_result=1, print_conv=1, print_final_part_time=1,
                          **gpu_params(d["flags_dict"], "fp64"))
    out = capfd.readouterr().out
    assert "Final eigenvalues and residual information:" in out
    assert "relative residual" in out
    rows = [l for l in out.splitlines() if l.strip().endswith("(converged)")]
    assert len(rows) == nev
    first = rows[0].split()
    assert first[0] == "1" and abs(float(first[1]) - ev[0]) <= 1e-14 * abs(ev[0])
    assert "Total gcg iteration: %d" % st["num_iter"] in out
    assert "All %d eigenpairs converged!" % nev in out
    assert "Section Name        w_lsol       w_orth       rr_eig       rr_mat" in out


def test_command_line_after_setup_is_a_state_error(cuda_lib):
    import ctypes as C
    A = M.laplace2d(16)
    s = S.GCGESolver(A, None, 4)
    try:
        args = [b"-gcge_precision", b"mixed"]
        argv = (C.c_char_p * 2)(*args)
        assert cuda_lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s.handle, 2, argv) == 4
        assert cuda_lib.GCGE_CUDA_SOLVER_SetParamInt(s.handle, b"nev", 5) == 4
        ev, vec = s.solve(M.initial_block(A.n, 4, seed=1))
        assert np.all(np.isfinite(ev))
    finally:
        s.close()
