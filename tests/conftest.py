import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    """Returns (A, B, nev, x0, data) for a fixture written by make_golden.py."""
    from gcge_old_gb300.matrices import CSRMatrix
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    n = len(d["a_rowptr"]) - 1
    A = CSRMatrix(n, d["a_rowptr"].astype(np.int32), d["a_col"].astype(np.int32), d["a_val"])
    B = None
    if "b_rowptr" in d:
        B = CSRMatrix(n, d["b_rowptr"].astype(np.int32), d["b_col"].astype(np.int32), d["b_val"])
    flags = {}
    for f in d["flags"]:
        k, v = str(f).split("=")
        k = k.replace("-gcge_", "").replace("-ref_", "")  # -ref_fixed_shift: oracle driver flag
        try:
            flags[k] = float(v)
        except ValueError:
            flags[k] = v  # eval_type
    d["flags_dict"] = flags
    return A, B, int(d["nev"]), d["x0"], d


GOLDEN_NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built if needed (GPU tests only)."""
    from gcge_old_gb300 import lib
    return lib.load(build_if_missing=True)
