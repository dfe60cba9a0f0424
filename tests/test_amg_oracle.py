"""The CPU restatement of the AMG set-up's index work (oracle/amg_ref.py):
the distance-2 maximal independent set has its defining properties and the
aggregates partition the rows.  The GPU test in test_gpu_amg.py compares the
device's aggregates with it bit-exactly."""
import numpy as np
import pytest

from gcge_old_gb300 import matrices as M
from oracle import amg_ref as R


CASES = [("laplace3d_mass", lambda: M.laplace3d_mass(12, seed=1)[0], 0.0),
         ("diffusion27", lambda: M.diffusion27(8, seed=2)[0], 0.0),
         ("diffusion27_strength", lambda: M.diffusion27(8, seed=2)[0], 0.1),
         ("chung_lu", lambda: M.chung_lu(2000, seed=3)[0], 0.0)]


@pytest.mark.parametrize("name,make,theta", CASES, ids=[c[0] for c in CASES])
def test_mis2_and_aggregates(name, make, theta):
    A = make()
    independent, covered = R.mis2_properties(A.rowptr, A.col, A.val, theta)
    assert independent and covered
    agg = R.aggregates(A.rowptr, A.col, A.val, theta)
    nagg = agg.max() + 1
    assert agg.min() == 0 and np.all(np.bincount(agg, minlength=nagg) > 0)
    assert nagg < A.n


def test_hash_matches_its_definition():
    # lowbias32 on a few values, computed by hand with 32-bit wrap-around
    def ref(x):
        x &= 0xFFFFFFFF
        x ^= x >> 16
        x = (x * 0x7FEB352D) & 0xFFFFFFFF
        x ^= x >> 15
        x = (x * 0x846CA68B) & 0xFFFFFFFF
        x ^= x >> 16
        return x
    xs = np.array([0, 1, 2, 12345, 2**31 - 1, 4000000])
    assert [int(v) for v in R.lowbias32(xs)] == [ref(int(x)) for x in xs]
