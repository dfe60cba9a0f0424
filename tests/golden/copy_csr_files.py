"""Copies the reference's own matrix files (test/data of the reference) into
tests/golden/csr_files/ as fixtures for the CSR file readers: the same 1089 x 1089
FE stiffness matrix as CSR text (A_5.txt) and as PETSc binary (A_5.petsc.bin),
and the 81 x 81 text matrix A_3.txt.  Run once where the reference is present:

    python tests/golden/copy_csr_files.py REFERENCE_DIR
"""
import os
import shutil
import sys

FILES = ["A_3.txt", "A_5.txt", "A_5.petsc.bin"]


def main(ref_root):
    src = os.path.join(ref_root, "test", "data")
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csr_files")
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        shutil.copyfile(os.path.join(src, f), os.path.join(dst, f))
        print("copied", f)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: copy_csr_files.py REFERENCE_DIR")
    main(sys.argv[1])
