"""Helpers for GPU tests: device columns held by torch (memory only) and
passed to the C ABI as arrays of column pointers."""
import ctypes as C

import numpy as np


def torch_cuda():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return torch


def dev_cols(X: np.ndarray):
    """Upload rows of X (k, n) as k separate device columns; returns
    (list of tensors, ctypes pointer array)."""
    torch = torch_cuda()
    ts = [torch.from_numpy(np.ascontiguousarray(x)).to("cuda") for x in X]
    arr = (C.c_void_p * max(1, len(ts)))(*[C.c_void_p(t.data_ptr()) for t in ts])
    return ts, arr


def host(ts):
    return np.stack([t.cpu().numpy() for t in ts]) if ts else np.zeros((0, 0))
