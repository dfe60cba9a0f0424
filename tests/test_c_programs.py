"""C callers of the library, compiled with gcc against include/*.h and linked
with -lgcge_cuda, run on the GPU: the device-resident solver through the C
API (tests/c/solve_c_api.c), the same with the W step handed to AMG-PCG on a
device-built AMG hierarchy (tests/c/amg_c_api.c), and the GCGE_OPS table
driven through its function pointers (tests/c/ops_table_gpu.c)."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CDIR = os.path.join(ROOT, "tests", "c")


def _exe(src, out):
    from gcge_old_gb300 import build as B
    libdir = os.path.dirname(B.build())
    cmd = ["gcc", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I", CDIR,
           os.path.join(CDIR, src), "-L", libdir, "-Wl,-rpath," + libdir, "-o", str(out),
           "-lgcge_cuda", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return str(out)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c_program_solves_through_the_c_api(tmp_path, precision):
    exe = _exe("solve_c_api.c", tmp_path / "solve_c_api")
    r = subprocess.run([exe, "32", "10", precision], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "c api: OK" in r.stdout
    # the final report in the reference's layout (GCGE_PrintFinalInfo)
    assert "Final eigenvalues and residual information:" in r.stdout
    assert "All 10 eigenpairs converged!" in r.stdout


def test_c_program_drives_the_gcge_ops_table(tmp_path):
    exe = _exe("ops_table_gpu.c", tmp_path / "ops_table_gpu")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ops table: OK" in r.stdout


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_c_program_solves_with_the_amg_preconditioner(tmp_path, precision):
    exe = _exe("amg_c_api.c", tmp_path / "amg_c_api")
    r = subprocess.run([exe, "48", "10", precision], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "amg c api: OK" in r.stdout
