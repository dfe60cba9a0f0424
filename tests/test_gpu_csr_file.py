"""A matrix loaded from the reference's own data files straight to the GPU
(GCGE_CUDA_MatCreateFromFile, text and PETSc binary) and solved: the eigenvalues
match a dense solve of the same file."""
import os

import numpy as np
import pytest
import scipy.linalg as sla

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
DATA = os.path.join(GOLDEN, "csr_files")


@pytest.mark.parametrize("fname", ["A_5.txt", "A_5.petsc.bin"])
def test_solve_matrix_from_file(cuda_lib, fname):
    from gcge_old_gb300.matrices import initial_block, read_csr_text
    from gcge_old_gb300.solver import DeviceMatrix, GCGESolver
    dA = DeviceMatrix.from_file(os.path.join(DATA, fname))
    assert dA.n == 1089
    nev = 8  # the 8th and 9th eigenvalues are 0.1245 and 0.1619: no pair is split
    s = GCGESolver(dA, None, nev, ev_tol=1e-10, ev_max_it=500, precision="fp64")
    try:
        ev, _ = s.solve(initial_block(dA.n, nev, seed=6))
        res = s.residuals()
    finally:
        s.close()
        dA.close()
    ref = sla.eigvalsh(read_csr_text(os.path.join(DATA, "A_5.txt")).to_scipy().toarray())[:nev]
    assert res.max() < 1e-10
    np.testing.assert_allclose(ev, ref, rtol=1e-9)
