"""The allocation-free inner product (GCGE_CUDA_MultiVecInnerProdNoAlloc)
against the allocating one (GCGE_CUDA_MultiVecInnerProd), through the C ABI,
and both against V W^T computed by numpy on the host.

Kept in its own file, collected last, so that it runs both alone in a fresh
process and after every other test has used the library's other scratch.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import dev_cols, torch_cuda


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def _reference(lib, vp, k1, wp, k2, n, sym):
    a = np.zeros((k2, k1))
    assert lib.GCGE_CUDA_MultiVecInnerProd(vp, k1, wp, k2, n, _ptr(a), k1, sym) == 0
    return a.T


def _no_alloc(lib, vp, k1, wp, k2, n, sym, lda):
    torch = torch_cuda()
    # output sentinel: entries outside the k1 x k2 block must stay untouched
    out = torch.full((k2, lda), -7.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.GCGE_CUDA_MultiVecInnerProdNoAlloc(vp, k1, wp, k2, n, C.c_void_p(out.data_ptr()), lda,
                                                sym, C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.GCGE_CUDA_GetLastErrorMessage()
    stream.synchronize()
    got = out.cpu().numpy()
    assert np.all(got[:, k1:] == -7.0)
    return got[:, :k1].T


@pytest.mark.gpu
def test_no_alloc_inner_prod_matches_two_calls_in_a_row(cuda_lib):
    # first call: the widest block the scratch array takes (64 x 64, sym);
    # second call: a narrower, non-symmetric product of another length, whose
    # partials land on top of what the first call left in the shared array.
    cases = [(64, 64, 1, 50_000, 70), (10, 37, 0, 123_457, 12)]
    for idx, (k1, k2, sym, n, lda) in enumerate(cases):
        rng = np.random.default_rng(100 + idx)
        V = rng.standard_normal((k1, n))
        W = V[:k2].copy() if sym else rng.standard_normal((k2, n))
        vs, vp = dev_cols(V)
        ws, wp = dev_cols(W)
        ref = _reference(cuda_lib, vp, k1, wp, k2, n, sym)
        got = _no_alloc(cuda_lib, vp, k1, wp, k2, n, sym, lda)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.sqrt(n))
        # independent check: the same products from numpy (FP64 on the host)
        host = V @ W.T
        np.testing.assert_allclose(got, host, rtol=1e-12, atol=1e-12 * np.sqrt(n))
        np.testing.assert_allclose(ref, host, rtol=1e-12, atol=1e-12 * np.sqrt(n))
        if sym:
            assert np.array_equal(got, got.T)


@pytest.mark.gpu
def test_no_alloc_inner_prod_rejects_blocks_beyond_its_scratch(cuda_lib):
    k1, k2, n = 65, 64, 1000  # 4160 outputs > GCGE_CUDA_NOALLOC_MAX_OUTPUTS
    vs, vp = dev_cols(np.ones((k1, n)))
    ws, wp = dev_cols(np.ones((k2, n)))
    torch = torch_cuda()
    out = torch.zeros((k2, k1), dtype=torch.float64, device="cuda")
    rc = cuda_lib.GCGE_CUDA_MultiVecInnerProdNoAlloc(vp, k1, wp, k2, n, C.c_void_p(out.data_ptr()),
                                                     k1, 0, None)
    assert rc == 1
    assert b"GCGE_CUDA_NOALLOC_MAX_OUTPUTS" in cuda_lib.GCGE_CUDA_GetLastErrorMessage()
