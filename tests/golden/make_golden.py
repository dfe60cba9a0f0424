"""Generates the golden fixtures of tests/golden/ from the REAL reference.

Run in a checkout where the reference is present (oracle/build_ref.sh builds
it into oracle/_ref/).  Each fixture stores the exact inputs (CSR arrays,
initial block) and the reference's outputs (eigenvalues, eigenvectors for
small cases, iteration count, convergence residuals) so the tests can check
the oracle port and the CUDA solver without the reference on the machine.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gcge_old_gb300 import matrices as M  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
# the reference checkout (oracle.REFERENCE_DIR: $GCGE_REFERENCE_DIR or the
# build container's checkout); the recipe runs only where it exists
REF_DATA = os.path.join(O.REFERENCE_DIR, "test", "data")


def save(name, A, B, nev, x0, flags, keep_vecs=True):
    r = O.ref_solve(A, B, nev, x0, flags)
    d = dict(a_rowptr=A.rowptr, a_col=A.col, a_val=A.val, nev=nev, x0=x0,
             eval=r["eval"], res=r["res"], iters=r["iters"],
             flags=np.array([f"{k}={v}" for k, v in flags.items()]))
    if B is not None:
        d.update(b_rowptr=B.rowptr, b_col=B.col, b_val=B.val)
    if keep_vecs:
        d["evec"] = r["evec"]
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **d)
    tr = O.true_residuals(A, B, r["eval"], r["evec"])
    print(f"{name}: n={A.n} nev={nev} iters={r['iters']} seconds={r['seconds']:.2f} "
          f"max true residual {tr.max():.2e}")


def main():
    if not O.ref_available():
        O.build_ref()
    # 3x3 SPD pair of the reference's test data (test/data/testA, testB)
    A3 = M.read_csr_text(REF_DATA + "/testA")
    B3 = M.read_csr_text(REF_DATA + "/testB")
    save("ref_testAB_3x3", A3, B3, 1, M.initial_block(3, 1, seed=5),
         {"-gcge_ev_tol": 1e-12, "-gcge_ev_max_it": 50})
    # (the 81x81 FE data A_3.txt/M_3.txt is not used: M_3 is singular, and
    # A_3's eigenvalue 1 from its 32 Dirichlet rows has multiplicity above
    # nev + 20, where the reference itself returns no valid pair)
    # 27-point Q1 diffusion with log-normal coefficients and Q1 mass, 10^3
    A, B = M.diffusion27(10, seed=2)
    save("ref_diff27_m10_nev10", A, B, 10, M.initial_block(A.n, 10, seed=4),
         {"-gcge_ev_tol": 1e-11, "-gcge_ev_max_it": 100})
    # 2D 5-point Laplacian, 32 x 32, B = I
    A = M.laplace2d(32)
    save("ref_lap2d_m32_nev10", A, None, 10, M.initial_block(A.n, 10, seed=3),
         {"-gcge_ev_tol": 1e-12, "-gcge_ev_max_it": 100})
    # 3D 7-point Laplacian with diagonal mass, 12^3
    A, B = M.laplace3d_mass(12, seed=1)
    save("ref_lap3d_m12_nev12", A, B, 12, M.initial_block(A.n, 12, seed=3),
         {"-gcge_ev_tol": 1e-10, "-gcge_ev_max_it": 100})
    # the CPU-runnable headline case: 128 x 128 Laplacian, nev 20, block 20
    A = M.laplace2d(128)
    save("ref_lap2d_m128_nev20", A, None, 20, M.initial_block(A.n, 20, seed=0),
         {"-gcge_ev_tol": 1e-13, "-gcge_block_size": 20, "-gcge_ev_max_it": 100},
         keep_vecs=False)

    shifted()
    more_structures()
    criteria()


def shifted():
    """The shift options (use_shift, a fixed if_shift/shift) and eval_type "sm"
    on indefinite problems A - c B; c is off the midpoint of two eigenvalues so
    no two |lambda - c| tie.  "-ref_fixed_shift" is a flag of
    oracle/ref_driver.c that sets para->if_shift = 1, para->shift = value."""
    import scipy.linalg as sla
    import scipy.sparse as sp
    A, B = M.diffusion27(10, seed=2)
    base = {"-gcge_ev_tol": 1e-11, "-gcge_ev_max_it": 150}
    x0 = M.initial_block(A.n, 10, seed=4)
    save("ref_diff27_m10_nev10_useshift", A, B, 10, x0, {**base, "-gcge_use_shift": 1})
    ev = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray(), eigvals_only=True)
    c = 0.5 * (ev[2] + ev[3]) + 0.37
    Ac = M.CSRMatrix.from_scipy(A.to_scipy() - c * B.to_scipy())
    save("ref_diff27c_m10_nev10_fixedshift", Ac, B, 10, x0, {**base, "-ref_fixed_shift": 2 * c})
    save("ref_diff27c_m10_nev10_sm", Ac, B, 10, x0, {**base, "-gcge_eval_type": "sm"})
    L = M.laplace2d(32).to_scipy()
    Lc = M.CSRMatrix.from_scipy(L - 0.1 * sp.identity(L.shape[0]))
    base = {"-gcge_ev_tol": 1e-10, "-gcge_ev_max_it": 150}
    x0 = M.initial_block(Lc.n, 10, seed=4)
    save("ref_lap2dc_m32_nev10_useshift", Lc, None, 10, x0, {**base, "-gcge_use_shift": 1})
    save("ref_lap2dc_m32_nev10_sm", Lc, None, 10, x0, {**base, "-gcge_eval_type": "sm"})


def more_structures():
    """Small instances of the anisotropic (per-cell kappa, diagonal mass) and the
    power-law graph (A = L + 1e-3 I, B = D, rows of very different lengths)
    problem families."""
    A, B, _, _ = M.aniso2d(24, seed=5)
    save("ref_aniso2d_m24_nev10", A, B, 10, M.initial_block(A.n, 10, seed=6),
         {"-gcge_ev_tol": 1e-11, "-gcge_ev_max_it": 150})
    A, B, _ = M.chung_lu(3000, seed=7)
    save("ref_chunglu_n3000_nev10", A, B, 10, M.initial_block(A.n, 10, seed=8),
         {"-gcge_ev_tol": 1e-10, "-gcge_ev_max_it": 300})


def criteria():
    """The "O" (omega-norm) and absolute convergence criteria
    (src/gcge_eigsol.c:713-721) with a given start, where the omega norm is the
    -gcge_conv_omega_norm value."""
    A, B = M.diffusion27(10, seed=2)
    save("ref_diff27_m10_nev10_convO", A, B, 10, M.initial_block(A.n, 10, seed=4),
         {"-gcge_ev_tol": 1e-12, "-gcge_ev_max_it": 150, "-gcge_conv_type": "O",
          "-gcge_conv_omega_norm": 0.5})
    A = M.laplace2d(32)
    save("ref_lap2d_m32_nev10_convA", A, None, 10, M.initial_block(A.n, 10, seed=3),
         {"-gcge_ev_tol": 1e-12, "-gcge_ev_max_it": 150, "-gcge_conv_type": "A"})


def make_cfg2_summary(out_path=os.path.join(OUT, "cfg2_reference_summary.json")):
    """Full-size headline workload (about 40 minutes on one core): writes the
    reference's eigenvalues, criterion values, iteration count and time."""
    import json
    import platform
    A, B = M.laplace3d_mass(128, seed=0)
    x0 = M.initial_block(A.n, 50, seed=0)
    flags = {"-gcge_ev_tol": 1e-10, "-gcge_ev_max_it": 1000}
    r = O.ref_solve(A, B, 50, x0, flags)
    tr = O.true_residuals(A, B, r["eval"], r["evec"])
    json.dump({"workload": "laplace3d_7pt_128^3_diagmass_nev50_tol1e-10 (seed 0 matrix, seed 0 initial block)",
               "generator": "gcge_old_gb300.matrices.laplace3d_mass(128, seed=0), initial_block(n, 50, seed=0)",
               "flags": dict(flags, **{"-gcge_num_init_evec": 50}), "iters": r["iters"],
               "seconds": r["seconds"], "host": "1 core, %s" % platform.machine(),
               "max_true_residual": float(tr.max()), "eval": [float(x) for x in r["eval"]],
               "res": [float(x) for x in r["res"]]}, open(out_path, "w"), indent=1)


def make_cfg3_summary(ev_tol=1e-11, out_path=os.path.join(OUT, "cfg3_port_summary.json")):
    """The 27-point mixed-precision workload at full size (160^3, n = 4,096,000,
    nev 100, block 20) solved by the oracle port on all host threads (the
    reference itself would take days on one core): writes its eigenvalues,
    criterion values, true residuals, iteration count and time.  ev_tol is
    tighter than the residual target 1e-10 because with a mass matrix of size
    h^3 that residual bound leaves the eigenvalues free by up to ~1e-9
    relative; the eigenvalue error falls with the square of the residual."""
    import json
    import platform
    import time
    threads = os.cpu_count() or 1
    t0 = time.time()
    A, B = M.diffusion27(160, seed=0)
    x0 = M.initial_block(A.n, 100, seed=0)
    gen = time.time() - t0
    p = O.default_para(100, ev_tol=ev_tol, ev_max_it=1000)
    r = O.port_solve(A, B, 100, x0, p, threads=threads)
    tr = O.true_residuals(A, B, r["eval"], r["evec"])
    json.dump({"workload": "diffusion27_q1_lognormal_160^3_consistent_mass_nev100 (seed 0 matrix, "
                           "seed 0 initial block)",
               "generator": "gcge_old_gb300.matrices.diffusion27(160, seed=0), initial_block(n, 100, seed=0)",
               "solver": "oracle port (oracle/gcge_port.c), reference default parameters, block size 20",
               "ev_tol": ev_tol, "iters": r["iters"], "seconds": r["seconds"],
               "generator_seconds": gen,
               "host": "%d threads, %s" % (threads, platform.machine()),
               "max_true_residual": float(tr.max()), "eval": [float(x) for x in r["eval"]],
               "res": [float(x) for x in r["res"]], "true_res": [float(x) for x in tr]},
              open(out_path, "w"), indent=1)
    print("cfg3: iters %d, %.0f s, max true residual %.2e" % (r["iters"], r["seconds"], tr.max()))


if __name__ == "__main__":
    # python tests/golden/make_golden.py [shifted|structures|criteria|cfg2|cfg3]
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what == "shifted":
        shifted()
    elif what == "structures":
        more_structures()
    elif what == "criteria":
        criteria()
    elif what == "cfg2":
        make_cfg2_summary()
    elif what == "cfg3":
        make_cfg3_summary(*[float(a) for a in sys.argv[2:3]])
    else:
        main()

