"""Eigenvalues of A x = lambda B x as a differentiable function of the CSR
values of A and B (fixed sparsity patterns), for torch.autograd.

The forward pass runs the GPU GCG solver (GCGESolver); the backward pass runs
the adjoint kernel GCGE_CUDA_EigGradCSR on the B-normalised eigenvectors:
for a loss L(lambda), dL/dA_e = sum_k g_k x_k[i] x_k[j] and
dL/dB_e = -sum_k g_k lambda_k x_k[i] x_k[j] over the stored entries e = (i, j),
g_k = dL/dlambda_k.  Every stored value is an independent parameter: for a
symmetric matrix stored in full, perturbing A_ij and A_ji together changes L
by grad[ij] + grad[ji].  Simple (non-repeated) eigenvalues are assumed.

    lam = eigvals_csr(a_val, A_pattern, nev, x0, b_val=b_val, B_pattern=B_pattern)
    (w * lam).sum().backward()
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import lib as L
from .matrices import CSRMatrix
from .solver import DeviceMatrix, GCGESolver


def _with_values(pattern: CSRMatrix, values) -> CSRMatrix:
    v = values.detach().to("cpu", torch.float64).numpy()
    if v.shape != (pattern.nnz,):
        raise ValueError("values must have one entry per stored element of the pattern")
    return CSRMatrix(pattern.n, pattern.rowptr, pattern.col, v.copy())


def _adjoint(pattern: CSRMatrix, evec: np.ndarray, coef: np.ndarray) -> torch.Tensor:
    """grad[e] = sum_k coef[k] evec[k][row(e)] evec[k][col(e)] on the GPU."""
    lib = L.load()
    k = evec.shape[0]
    cols = [torch.from_numpy(np.ascontiguousarray(evec[j])).to("cuda") for j in range(k)]
    xp = (C.c_void_p * k)(*[C.c_void_p(t.data_ptr()) for t in cols])
    grad = torch.zeros(pattern.nnz, dtype=torch.float64, device="cuda")
    dM = DeviceMatrix(pattern)
    c = np.ascontiguousarray(coef, dtype=np.float64)
    L.check(lib.GCGE_CUDA_EigGradCSR(dM.handle, xp, C.c_void_p(c.ctypes.data), k,
                                     C.c_void_p(grad.data_ptr())), "EigGradCSR")
    dM.close()
    return grad


class _EigvalsCSR(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a_val, b_val, A_pattern, B_pattern, nev, x0, params):
        A = _with_values(A_pattern, a_val)
        B = _with_values(B_pattern, b_val) if b_val is not None else None
        s = GCGESolver(A, B, nev, **params)
        try:
            ev, vec = s.solve(x0)
        finally:
            s.close()
        ctx.A_pattern, ctx.B_pattern = A_pattern, B_pattern
        ctx.ev, ctx.vec = ev, vec
        ctx.has_b = b_val is not None
        return torch.from_numpy(ev.copy()).to(a_val.device)

    @staticmethod
    def backward(ctx, g):
        gl = g.detach().to("cpu", torch.float64).numpy()
        ga = _adjoint(ctx.A_pattern, ctx.vec, gl) if ctx.needs_input_grad[0] else None
        gb = None
        if ctx.has_b and ctx.needs_input_grad[1]:
            gb = _adjoint(ctx.B_pattern, ctx.vec, -gl * ctx.ev)
        dev = g.device
        return (ga.to(dev) if ga is not None else None, gb.to(dev) if gb is not None else None,
                None, None, None, None, None)


def eigvals_csr(a_val: torch.Tensor, A_pattern: CSRMatrix, nev: int, x0: np.ndarray,
                b_val: torch.Tensor | None = None, B_pattern: CSRMatrix | None = None,
                **params) -> torch.Tensor:
    """The nev smallest eigenvalues of A x = lambda B x (B = I without b_val), with
    a_val / b_val the CSR values over A_pattern / B_pattern.  params: solver
    parameters of GCGESolver (ev_tol, precision, ...)."""
    if (b_val is None) != (B_pattern is None):
        raise ValueError("b_val and B_pattern go together")
    return _EigvalsCSR.apply(a_val, b_val, A_pattern, B_pattern, nev, x0, params)
