"""The C callers of the library (tests/c/solve_c_api.c, amg_c_api.c,
ops_table_gpu.c) compile with -Wall -Werror against include/*.h and link with
-lgcge_cuda on a machine without a GPU; run there, each stops with a non-zero
status and the library's error message (no CPU fallback, no crash).  The
Python path likewise: a missing library is an error, and so is the first
device call without a GPU."""
import subprocess

import pytest

from test_c_programs import _exe

CALLERS = [("solve_c_api.c", ["32", "10", "fp64"]), ("amg_c_api.c", ["48", "10", "mixed"]),
           ("ops_table_gpu.c", [])]


def _has_gpu():
    import torch
    return torch.cuda.is_available()


@pytest.mark.parametrize("src,args", CALLERS)
def test_c_caller_builds_and_fails_loudly_without_a_gpu(tmp_path, src, args):
    exe = _exe(src, tmp_path / src[:-2])
    if _has_gpu():
        pytest.skip("a GPU is present: the GPU tests run these programs")
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=120)
    assert r.returncode > 0, (r.returncode, r.stdout, r.stderr)
    assert "fail" in (r.stdout + r.stderr).lower(), r.stdout + r.stderr


def test_python_path_fails_loudly_without_the_library(monkeypatch, tmp_path):
    """A missing library is an error naming the build step, not a fallback."""
    from gcge_old_gb300 import lib as L
    monkeypatch.setattr(L, "_lib", None)
    monkeypatch.setattr(L, "LIB_PATH", str(tmp_path / "libgcge_cuda.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        L.load()


def test_python_solve_fails_loudly_without_a_gpu():
    """With the library built but no GPU, the first device call is an error."""
    from gcge_old_gb300 import lib as L
    from gcge_old_gb300 import matrices as M
    from gcge_old_gb300 import solver as S
    L.load(build_if_missing=True)
    if _has_gpu():
        pytest.skip("a GPU is present: the GPU tests run the solver")
    A = M.laplace2d(8)
    with pytest.raises(L.GcgeCudaError, match="MatCreate"):
        S.solve(A, None, 4, M.initial_block(A.n, 4, seed=0))
