"""CPU checks of the GCGE_OPS plugin surface (include/gcge_cuda_ops.h) against
the reference itself, where its checkout is present: the table has the
reference's struct GCGE_OPS layout field by field, and the unmodified
reference core compiles and links with the CUDA app's set-up
(gcge_old_gb300/app/gcge_app_cuda.c) and library.  Without a GPU the linked
program stops at its first device allocation with its no-device status."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle import oracle as O

REF_DEFS = ["-D_GCGE_CONFIG_H_", "-DGCGE_DOUBLE=double", "-DGCGE_INT=int", "-DGET_PART_TIME=1",
            "-DGCGE_USE_MPI=0", "-include", "float.h"]


def _need_reference():
    if not O.reference_present():
        pytest.skip("reference checkout not present")


def test_ops_table_has_the_reference_layout():
    _need_reference()
    r = subprocess.run(["gcc", "-fsyntax-only", "-Wall", "-Werror", *REF_DEFS,
                        "-I", os.path.join(O.REFERENCE_DIR, "src"), "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "c", "ops_layout.c")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_core_links_with_the_cuda_ops(tmp_path):
    _need_reference()
    ref_so = O.build_ref()
    if ref_so is None:
        pytest.skip("reference build failed")
    from gcge_old_gb300 import build as B
    libdir = os.path.dirname(B.build())
    refdir = os.path.dirname(ref_so)
    exe = str(tmp_path / "ops_ref_driver")
    cmd = ["gcc", "-O2", "-Wall", "-Werror", *REF_DEFS, "-I", os.path.join(O.REFERENCE_DIR, "src"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "gcge_old_gb300", "app"),
           "-I", os.path.join(ROOT, "tests", "c"),
           os.path.join(ROOT, "tests", "c", "ops_ref_driver.c"),
           os.path.join(ROOT, "gcge_old_gb300", "app", "gcge_app_cuda.c"),
           "-L", refdir, "-Wl,-rpath," + refdir, "-L", libdir, "-Wl,-rpath," + libdir,
           "-o", exe, "-lgcge_ref", "-lgcge_cuda", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "16", "4", "-gcge_ev_tol", "1e-10"], capture_output=True, text=True,
                       timeout=300)
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stdout + r.stderr
    else:
        assert r.returncode == 3, r.stdout + r.stderr
        assert "no usable CUDA device" in r.stdout
