"""CPU tests: the oracle port against the reference's golden outputs, the
reference against the port where the reference is built here, and the
seeded generators."""
import numpy as np
import pytest
import scipy.linalg as sl

from conftest import GOLDEN_NAMES, load_golden
from gcge_old_gb300 import matrices as M
from oracle import oracle as O


def para_for(nev, flags):
    kw = {}
    for k, v in flags.items():
        if k in ("ev_tol", "cg_rate"):
            kw[k] = float(v)
        elif k in ("block_size", "ev_max_it", "cg_max_it", "use_shift"):
            kw[k] = int(v)
        elif k == "eval_type":
            kw["eval_sm"] = int(v == "sm")
        elif k == "fixed_shift":
            kw["if_shift"], kw["shift"] = 1, float(v)
        elif k == "conv_type":
            kw["conv_type"] = {"R": 0, "O": 1, "A": 2}[v]
        elif k == "conv_omega_norm":
            kw["conv_omega_norm"] = float(v)
    return O.default_para(nev, **kw)


@pytest.mark.parametrize("name", [n for n in GOLDEN_NAMES if "m128" not in n])
def test_port_matches_reference_golden(name):
    A, B, nev, x0, d = load_golden(name)
    r = O.port_solve(A, B, nev, x0, para_for(nev, d["flags_dict"]), threads=2)
    rel = np.max(np.abs(r["eval"] - d["eval"]) / np.abs(d["eval"]))
    assert rel < 1e-10, rel
    assert abs(r["iters"] - int(d["iters"])) <= 1
    # same converged residuals (criterion values) up to rounding
    tr = O.true_residuals(A, B, r["eval"], r["evec"])
    tr_ref = O.true_residuals(A, B, d["eval"], d["evec"])
    assert tr.max() < 10 * max(tr_ref.max(), 1e-14)


@pytest.mark.parametrize("name", [n for n in GOLDEN_NAMES if "m128" not in n and "3x3" not in n])
def test_port_mixed_w_step_matches_reference_golden(name):
    """The port's mixed W step (FP32 block CG, W = the FP32 correction) reaches the
    reference's eigenvalues and residual bound on the golden fixtures."""
    A, B, nev, x0, d = load_golden(name)
    para = para_for(nev, d["flags_dict"])
    para.mixed = 1
    para.ev_max_it = max(para.ev_max_it, 2 * int(d["iters"]) + 10)
    r = O.port_solve(A, B, nev, x0, para, threads=2)
    rel = np.max(np.abs(r["eval"] - d["eval"]) / np.abs(d["eval"]))
    assert rel < 1e-9, rel
    assert r["iters"] <= int(d["iters"]) + 5
    tr = O.true_residuals(A, B, r["eval"], r["evec"])
    tr_ref = O.true_residuals(A, B, d["eval"], d["evec"])
    assert tr.max() < 10 * max(tr_ref.max(), 1e-14)


def test_port_matches_reference_golden_headline_cpu_case():
    """128 x 128 Laplacian, nev 20, block 20, tol 1e-13 (the CPU-runnable case)."""
    A, B, nev, x0, d = load_golden("ref_lap2d_m128_nev20")
    r = O.port_solve(A, B, nev, x0, para_for(nev, d["flags_dict"]), threads=4)
    rel = np.max(np.abs(r["eval"] - d["eval"]) / np.abs(d["eval"]))
    assert rel < 1e-10, rel
    assert abs(r["iters"] - int(d["iters"])) <= 1
    assert O.true_residuals(A, B, r["eval"], r["evec"]).max() < 1e-10


def test_golden_against_dense_eigh():
    """The reference's eigenvalues on the small fixtures are the exact ones."""
    for name in ("ref_testAB_3x3", "ref_lap2d_m32_nev10", "ref_lap3d_m12_nev12",
                 "ref_diff27_m10_nev10"):
        A, B, nev, x0, d = load_golden(name)
        a = A.to_scipy().toarray()
        b = B.to_scipy().toarray() if B is not None else None
        w = sl.eigh(a, b, eigvals_only=True, subset_by_index=[0, nev - 1])
        assert np.max(np.abs(d["eval"] - w) / np.abs(w)) < 1e-9, name


@pytest.mark.skipif(not O.ref_available(), reason="reference not built in this checkout")
def test_reference_vs_port_fresh_seed():
    A, B = M.laplace3d_mass(10, seed=9)
    nev = 10
    x0 = M.initial_block(A.n, nev, seed=21)
    ref = O.ref_solve(A, B, nev, x0, {"-gcge_ev_tol": 1e-11, "-gcge_ev_max_it": 100})
    port = O.port_solve(A, B, nev, x0, O.default_para(nev, ev_tol=1e-11, ev_max_it=100))
    assert np.max(np.abs(ref["eval"] - port["eval"]) / ref["eval"]) < 1e-10
    assert ref["iters"] == port["iters"]


def test_port_mixed_w_step_hub_localised_spectrum():
    """The port's emulation of the CUDA solver's mixed W step (FP32 block CG on
    the FP64 residual, W = the FP32 correction) converges like the FP64 solve
    on a shifted power-law graph whose lowest eigenvectors sit on hub nodes
    (handing w0 + e instead of e to the orthogonalisation lost the basis's
    B-orthonormality there and gave spurious eigenvalues near 1e-6)."""
    A, B, _ = M.chung_lu(5000, seed=2, shift=100.0)
    nev = 16
    x0 = M.initial_block(A.n, nev, seed=3)
    para = dict(ev_tol=1e-8, ev_max_it=150, block_size=10)
    f64 = O.port_solve(A, B, nev, x0, O.default_para(nev, **para), threads=4)
    mix = O.port_solve(A, B, nev, x0, O.default_para(nev, mixed=1, **para), threads=4)
    assert f64["iters"] < 60 and abs(mix["iters"] - f64["iters"]) <= 5
    np.testing.assert_allclose(mix["eval"], f64["eval"], rtol=1e-10)
    crit = O.true_residuals(A, B, mix["eval"], mix["evec"]) * mix["eval"] / np.maximum(1, mix["eval"])
    assert crit.max() < 1.5e-8


def test_port_bounded_sample():
    """max_outer bounds the outer loop (used for the timed CPU sample)."""
    A = M.laplace2d(40)
    x0 = M.initial_block(A.n, 10, seed=1)
    r = O.port_solve(A, None, 10, x0, O.default_para(10, ev_tol=1e-13, ev_max_it=100), max_outer=2)
    assert r["iters"] == 4  # RR on X, the [X, W] step, then 2 loop iterations


def test_generators_shapes_and_symmetry():
    A = M.laplace2d(128)
    assert A.n == 16384 and A.nnz == 5 * 128 * 128 - 4 * 128
    A2, B2 = M.laplace3d_mass(16, seed=0)
    assert A2.nnz == 7 * 16 ** 3 - 6 * 16 ** 2
    assert B2.nnz == B2.n and np.all(B2.val > 0)
    h = 1.0 / 17
    assert np.all(np.abs(B2.val / h ** 3 - 1.0) <= 0.1 + 1e-12)
    A3, B3 = M.diffusion27(8, seed=0)
    assert A3.nnz == (3 * 8 - 2) ** 3 and B3.nnz == (3 * 8 - 2) ** 3
    for m in (A2, A3, B3):
        s = m.to_scipy()
        assert abs(s - s.T).max() < 1e-15
    # Q1 mass row sums of an interior node equal h^3 (8 cells x 1/8)
    h = 1.0 / 9
    s = B3.to_scipy()
    i = (4 * 8 + 4) * 8 + 4
    assert abs(s[i].sum() - h ** 3) < 1e-15


def test_generator_is_seeded():
    a1, b1 = M.laplace3d_mass(6, seed=3)
    a2, b2 = M.laplace3d_mass(6, seed=3)
    assert np.array_equal(b1.val, b2.val)
    assert np.array_equal(M.initial_block(100, 3, seed=5), M.initial_block(100, 3, seed=5))
