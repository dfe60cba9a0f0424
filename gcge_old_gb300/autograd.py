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

eigpairs_csr also returns the eigenvectors (rows of X, B-normalised, each
signed so that its entry of largest magnitude is positive) for losses that
use them.  Their adjoint (GCGE_CUDA_EigvecAdjointSolve + GCGE_CUDA_EigGradCSR2)
solves, for each eigenvector the loss touches, the projected system
(A - lambda_k B) mu_k = g_k - B x_k (x_k^T g_k) with mu_k B-orthogonal to x_k,
and gives dL/dA_ij = -mu_k[i] x_k[j], dL/dB_ij = lambda_k mu_k[i] x_k[j]
- 1/2 (g_k^T x_k) x_k[i] x_k[j].  It needs lambda_k < lambda_{nev+1}, which
holds for every returned pair.

    lam, X = eigpairs_csr(a_val, A_pattern, nev, x0, b_val=b_val, B_pattern=B_pattern)
    ((X[0] * mask) ** 2).sum().backward()
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import lib as L
from .matrices import CSRMatrix
from .solver import AMG, DeviceMatrix, GCGESolver


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


# step count and column count of the last eigenvector-adjoint solve
last_adjoint = {"steps": 0, "columns": 0, "preconditioner": "jacobi"}


def _signed(vec: np.ndarray) -> np.ndarray:
    """Each row flipped so that its entry of largest magnitude is positive."""
    idx = np.abs(vec).argmax(axis=1)
    sgn = np.sign(vec[np.arange(len(vec)), idx])
    sgn[sgn == 0] = 1.0
    return vec * sgn[:, None]


def _cols(t: torch.Tensor):
    return (C.c_void_p * t.shape[0])(*[C.c_void_p(t[j].data_ptr()) for j in range(t.shape[0])])


class _EigpairsCSR(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a_val, b_val, A_pattern, B_pattern, nev, x0, params, adj):
        A = _with_values(A_pattern, a_val)
        B = _with_values(B_pattern, b_val) if b_val is not None else None
        s = GCGESolver(A, B, nev, **params)
        try:
            ev, vec = s.solve(x0)
        finally:
            s.close()
        vec = _signed(vec)
        ctx.A, ctx.B = A, B
        ctx.ev, ctx.vec, ctx.adj = ev, vec, adj
        ctx.has_b = b_val is not None
        dev = a_val.device
        return torch.from_numpy(ev.copy()).to(dev), torch.from_numpy(vec.copy()).to(dev)

    @staticmethod
    def backward(ctx, g_lam, g_vec):
        lib = L.load()
        ev, nev = ctx.ev, len(ctx.ev)
        gl = (g_lam.detach().to("cpu", torch.float64).numpy() if g_lam is not None
              else np.zeros(nev))
        X = torch.from_numpy(np.ascontiguousarray(ctx.vec)).to("cuda")
        xp = _cols(X)
        mu = None
        gx = np.zeros(nev)
        want = np.zeros(nev, dtype=bool)
        dA = DeviceMatrix(ctx.A)
        dB = DeviceMatrix(ctx.B) if ctx.B is not None else None
        try:
            if g_vec is not None:
                G = g_vec.detach().to("cuda", torch.float64).contiguous()
                want = (G.abs().amax(dim=1) > 0).cpu().numpy()
            if want.any():
                mu = torch.zeros_like(X)
                gp = (C.c_void_p * nev)(*[C.c_void_p(G[j].data_ptr()) if want[j] else None
                                          for j in range(nev)])
                it = C.c_int(0)
                amg = None
                if ctx.adj["amg"] is not None:
                    amg = AMG(dA, **ctx.adj["amg"])
                try:
                    L.check(lib.GCGE_CUDA_EigvecAdjointSolveAMG(
                        dA.handle, dB.handle if dB else None, xp, _dptr(ev), nev, gp, _cols(mu),
                        _dptr(gx), int(ctx.adj["max_it"]), float(ctx.adj["tol"]), C.byref(it),
                        amg.handle if amg else None), "EigvecAdjointSolve")
                finally:
                    if amg:
                        amg.close()
                last_adjoint["steps"] = it.value
                last_adjoint["columns"] = int(want.sum())
                last_adjoint["preconditioner"] = "amg" if amg else "jacobi"
            mp = _cols(mu) if mu is not None else None
            ga = gb = None
            if ctx.needs_input_grad[0]:
                ga = torch.zeros(ctx.A.nnz, dtype=torch.float64, device="cuda")
                a = np.ascontiguousarray(gl)
                b = np.where(want, -1.0, 0.0)
                L.check(lib.GCGE_CUDA_EigGradCSR2(dA.handle, xp, mp, _dptr(a), _dptr(b), nev,
                                                  C.c_void_p(ga.data_ptr())), "EigGradCSR2")
            if ctx.has_b and ctx.needs_input_grad[1]:
                gb = torch.zeros(ctx.B.nnz, dtype=torch.float64, device="cuda")
                a = np.ascontiguousarray(-ev * gl - 0.5 * gx)
                b = np.where(want, ev, 0.0)
                L.check(lib.GCGE_CUDA_EigGradCSR2(dB.handle, xp, mp, _dptr(a), _dptr(b), nev,
                                                  C.c_void_p(gb.data_ptr())), "EigGradCSR2")
        finally:
            dA.close()
            if dB:
                dB.close()
        dev = (g_lam if g_lam is not None else g_vec).device
        return (ga.to(dev) if ga is not None else None, gb.to(dev) if gb is not None else None,
                None, None, None, None, None, None)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(L.c_double_p)


def eigpairs_csr(a_val: torch.Tensor, A_pattern: CSRMatrix, nev: int, x0: np.ndarray,
                 b_val: torch.Tensor | None = None, B_pattern: CSRMatrix | None = None,
                 adjoint_tol: float = 1e-10, adjoint_max_it: int = 100000,
                 adjoint_amg: dict | bool | None = None, **params):
    """(lambda, X): the nev smallest eigenpairs of A x = lambda B x, X of shape
    (nev, n) with B-normalised rows, differentiable in a_val / b_val for losses
    of both.  adjoint_tol / adjoint_max_it: stopping rule of the projected CG of
    the eigenvector adjoint (relative residual per column).  adjoint_amg: True
    or a dict of GCGE_CUDA_AMG_PARAM fields preconditions that CG by a V-cycle
    of an AMG hierarchy of A built in the backward pass (GCGE_CUDA_AMG_Create);
    None / False: diag(A)."""
    if (b_val is None) != (B_pattern is None):
        raise ValueError("b_val and B_pattern go together")
    amg = None if adjoint_amg in (None, False) else ({} if adjoint_amg is True else dict(adjoint_amg))
    adj = {"tol": adjoint_tol, "max_it": adjoint_max_it, "amg": amg}
    return _EigpairsCSR.apply(a_val, b_val, A_pattern, B_pattern, nev, x0, params, adj)
