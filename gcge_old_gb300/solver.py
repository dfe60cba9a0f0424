"""Python mirror of the GCGE solver interface over the CUDA C ABI.

``GCGESolver`` follows GCGE_SOLVER (src/gcge_solver.h:42-60): build it from
CSR matrices, set -gcge_* parameters (names of src/gcge_para.c:128-407),
give the initial block, ``solve()``, read eigenvalues/eigenvectors.  The
matrices are copied to the device once (``GCGE_CUDA_MatCreate``); inputs and
outputs of ``solve`` are host arrays, as for the reference CSR app.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as L
from .matrices import CSRMatrix


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class DeviceMatrix:
    """A CSR matrix resident on the GPU (GCGE_CUDA_MAT)."""

    def __init__(self, m: CSRMatrix):
        self._lib = L.load()
        self.n = m.n
        self._h = (np.ascontiguousarray(m.rowptr, dtype=np.int32),
                   np.ascontiguousarray(m.col, dtype=np.int32),
                   np.ascontiguousarray(m.val, dtype=np.float64))
        h = C.c_void_p()
        L.check(self._lib.GCGE_CUDA_MatCreate(C.byref(h), m.n, _ptr(self._h[0]), _ptr(self._h[1]),
                                              _ptr(self._h[2]), 0), "MatCreate")
        self.handle = h

    @classmethod
    def from_file(cls, path) -> "DeviceMatrix":
        """A square matrix read straight from a CSR text or PETSc binary file
        (GCGE_CUDA_MatCreateFromFile)."""
        import os
        self = cls.__new__(cls)
        self._lib = L.load()
        h = C.c_void_p()
        L.check(self._lib.GCGE_CUDA_MatCreateFromFile(C.byref(h), os.fsencode(path)),
                "MatCreateFromFile")
        self.handle = h
        n = C.c_int()
        L.check(self._lib.GCGE_CUDA_MatGetSize(h, C.byref(n), None), "MatGetSize")
        self.n = n.value
        return self

    def close(self):
        if self.handle:
            h = self.handle
            self._lib.GCGE_CUDA_MatDestroy(C.byref(h))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AMG:
    """Smoothed-aggregation AMG hierarchy of a DeviceMatrix (GCGE_CUDA_AMG),
    built on the GPU; the GPU counterpart of the BoomerAMG hierarchy the
    reference reaches through its hypre app.  ``params``: fields of
    GCGE_CUDA_AMG_PARAM (max_levels, coarse_size, strength, smooth_p,
    cheb_degree, cheb_ratio, pcg_max_it, pcg_rate); the rest keep their
    defaults.  The matrix must outlive the hierarchy."""

    def __init__(self, A: DeviceMatrix, **params):
        self._lib = L.load()
        self.A = A
        self.param = L.AMGParam()
        self._lib.GCGE_CUDA_AMG_DefaultParam(C.byref(self.param))
        for k, v in params.items():
            if k not in dict(L.AMGParam._fields_):
                raise ValueError("unknown AMG parameter %r" % k)
            setattr(self.param, k, v)
        h = C.c_void_p()
        L.check(self._lib.GCGE_CUDA_AMG_Create(C.byref(h), A.handle, C.byref(self.param)),
                "AMG_Create")
        self.handle = h

    @property
    def num_levels(self) -> int:
        n = C.c_int()
        L.check(self._lib.GCGE_CUDA_AMG_GetNumLevels(self.handle, C.byref(n)), "AMG_GetNumLevels")
        return n.value

    def level_info(self, l: int) -> dict:
        n, na, npp, lm = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        L.check(self._lib.GCGE_CUDA_AMG_GetLevelInfo(self.handle, l, C.byref(n), C.byref(na),
                                                     C.byref(npp), C.byref(lm)), "AMG_GetLevelInfo")
        return {"n": n.value, "nnz_a": na.value, "nnz_p": npp.value, "lmax": lm.value}

    def level_csr(self, l: int, which: str = "A"):
        """A_l, P_l or R_l (= P_l^T) as a scipy CSR matrix."""
        import scipy.sparse as sp
        info = self.level_info(l)
        nxt = self.level_info(l + 1)["n"] if which in ("P", "R") else info["n"]
        rows, cols, nnz = {"A": (info["n"], info["n"], info["nnz_a"]),
                           "P": (info["n"], nxt, info["nnz_p"]),
                           "R": (nxt, info["n"], info["nnz_p"])}[which]
        rp = np.zeros(rows + 1, dtype=np.int32)
        ci = np.zeros(max(nnz, 1), dtype=np.int32)
        v = np.zeros(max(nnz, 1))
        L.check(self._lib.GCGE_CUDA_AMG_GetLevelCSR(
            self.handle, l, {"A": 0, "P": 1, "R": 2}[which], rp.ctypes.data_as(L.c_int_p),
            ci.ctypes.data_as(L.c_int_p), v.ctypes.data_as(L.c_double_p)), "AMG_GetLevelCSR")
        return sp.csr_matrix((v[:nnz], ci[:nnz], rp), shape=(rows, cols))

    def aggregates(self, l: int = 0) -> np.ndarray:
        a = np.zeros(self.level_info(l)["n"], dtype=np.int32)
        L.check(self._lib.GCGE_CUDA_AMG_GetAggregates(self.handle, l, a.ctypes.data_as(L.c_int_p)),
                "AMG_GetAggregates")
        return a

    @property
    def last_steps(self) -> int:
        s = C.c_int()
        L.check(self._lib.GCGE_CUDA_AMG_GetLastSteps(self.handle, C.byref(s)), "AMG_GetLastSteps")
        return s.value

    def close(self):
        if self.handle:
            h = self.handle
            self._lib.GCGE_CUDA_AMG_Destroy(C.byref(h))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def pase_solve(A, B, nev: int, amg: "AMG | None" = None, amg_params: dict | None = None,
               evec_device=None, **params):
    """The multilevel eigensolver (GCGE_CUDA_PASE_Solve, the GPU form of the
    reference's PASE_EigenSolver, pase/src/pase_solver.c:17-82) on the AMG
    hierarchy of A.  A, B: CSRMatrix or DeviceMatrix (B None: identity);
    params: fields of GCGE_CUDA_PASE_PARAM.  evec_device: optional torch
    tensor (nev, n) on cuda to receive the eigenvectors (else they are copied
    to the host).  Returns (eval, evec (nev, n) or the tensor, stats dict)."""
    lib = L.load()
    dA = A if isinstance(A, DeviceMatrix) else DeviceMatrix(A)
    dB = None if B is None else (B if isinstance(B, DeviceMatrix) else DeviceMatrix(B))
    own = amg is None
    if own:
        amg = AMG(dA, **(amg_params or {}))
    prm = L.PASEParam()
    lib.GCGE_CUDA_PASE_DefaultParam(C.byref(prm))
    for k, v in params.items():
        if k not in dict(L.PASEParam._fields_):
            raise ValueError("unknown PASE parameter %r" % k)
        setattr(prm, k, v)
    ev = np.zeros(nev)
    st = L.PASEStats()
    if evec_device is None:
        import torch
        out = torch.empty((nev, dA.n), dtype=torch.float64, device="cuda")
    else:
        out = evec_device
    try:
        L.check(lib.GCGE_CUDA_PASE_Solve(dA.handle, dB.handle if dB else None, amg.handle, nev,
                                         C.byref(prm), ev.ctypes.data_as(L.c_double_p),
                                         C.c_void_p(out.data_ptr()), C.byref(st)), "PASE_Solve")
    finally:
        if own:
            amg.close()
    stats = {f: getattr(st, f) for f, _ in L.PASEStats._fields_}
    return ev, (out if evec_device is not None else out.cpu().numpy()), stats


class GCGESolver:
    """GCG eigensolver for A x = lambda B x on one GPU.

    params: mapping of GCGE_PARA names (``nev``, ``ev_tol``, ``block_size``,
    ``ev_max_it``, ``cg_max_it``, ``cg_rate``, ...) plus ``precision``
    ("fp64" or "mixed": FP32 block CG on FP32 copies of A).
    """

    INT_PARAMS = {"nev", "ev_max_it", "block_size", "num_init_evec", "cg_max_it",
                  "max_reorth_time", "print_level", "gemm", "use_shift", "if_shift",
                  "eval_type", "conv_type", "w_form", "print_result", "print_conv",
                  "print_final_part_time", "print_eval", "print_para"}
    NAMED = {"precision": {"fp64": 0, "mixed": 1}, "eval_type": {"sa": 0, "sm": 1},
             "gemm": {"fp64": 0, "ozaki": 1}, "conv_type": {"R": 0, "O": 1, "A": 2},
             "w_form": {"reference": 0, "correction": 1}}

    def __init__(self, A, B=None, nev: int = 1, **params):
        self._lib = L.load()
        self.A = A if isinstance(A, DeviceMatrix) else DeviceMatrix(A)
        self.B = None if B is None else (B if isinstance(B, DeviceMatrix) else DeviceMatrix(B))
        self.n = self.A.n
        self.nev = nev
        h = C.c_void_p()
        L.check(self._lib.GCGE_CUDA_SOLVER_Create(C.byref(h)), "SOLVER_Create")
        self.handle = h
        L.check(self._lib.GCGE_CUDA_SOLVER_SetMatA(h, self.A.handle), "SetMatA")
        L.check(self._lib.GCGE_CUDA_SOLVER_SetMatB(h, self.B.handle if self.B else None), "SetMatB")
        L.check(self._lib.GCGE_CUDA_SOLVER_SetNumEigen(h, nev), "SetNumEigen")
        params.setdefault("num_init_evec", nev)
        for k, v in params.items():
            if k in self.NAMED:
                v = self.NAMED[k].get(v, v)
                L.check(self._lib.GCGE_CUDA_SOLVER_SetParamInt(h, k.encode(), int(v)), k)
            elif k in self.INT_PARAMS:
                L.check(self._lib.GCGE_CUDA_SOLVER_SetParamInt(h, k.encode(), int(v)), k)
            else:
                L.check(self._lib.GCGE_CUDA_SOLVER_SetParamDouble(h, k.encode(), float(v)), k)
        self.eval = np.zeros(nev)
        self.evec = np.zeros((nev, self.n))  # column j of the n x nev block is evec[j]
        L.check(self._lib.GCGE_CUDA_SOLVER_SetEigenvalues(h, _ptr(self.eval)), "SetEigenvalues")
        L.check(self._lib.GCGE_CUDA_SOLVER_SetEigenvectors(h, _ptr(self.evec)), "SetEigenvectors")
        L.check(self._lib.GCGE_CUDA_SOLVER_Setup(h), "Setup")

    def set_linear_solver(self, fn, ctx=None):
        """Replace the built-in block CG of the W step (GCGE_OPS.MultiLinearSolver,
        src/gcge_ops.h:77) by fn, a lib.MultiLinearSolver or a C function address;
        fn=None restores the built-in block CG.  fn and ctx must outlive the solves."""
        self._mls = (fn, ctx)
        if fn is not None and not isinstance(fn, L.MultiLinearSolver):
            fn = C.cast(fn, L.MultiLinearSolver)
        cp = C.cast(C.pointer(ctx), C.c_void_p) if isinstance(ctx, C.Structure) else ctx
        L.check(self._lib.GCGE_CUDA_SOLVER_SetMultiLinearSolver(
            self.handle, C.cast(fn, C.c_void_p) if fn is not None else None, cp),
            "SetMultiLinearSolver")

    def use_jacobi_pcg(self, max_it: int = 20, rate: float = 1e-2):
        """W step by GCGE_CUDA_JacobiPCG: block CG preconditioned by diag(A)."""
        self._pcg = L.PCGParam(max_it, rate)
        self.set_linear_solver(self._lib.GCGE_CUDA_JacobiPCG, self._pcg)

    def use_chebyshev_pcg(self, max_it: int = 20, rate: float = 1e-2, degree: int = 4,
                          lower_frac: float = 0.05):
        """W step by GCGE_CUDA_ChebyshevPCG: block CG preconditioned by a
        Chebyshev polynomial in diag(A)^-1 A."""
        self._cheb = L.ChebParam(max_it, rate, degree, lower_frac)
        self.set_linear_solver(self._lib.GCGE_CUDA_ChebyshevPCG, self._cheb)

    def use_amg_pcg(self, amg: "AMG | None" = None, **params):
        """W step by GCGE_CUDA_AMGPCG: CG preconditioned by one V-cycle of an AMG
        hierarchy of A (built here from ``params`` when not given)."""
        self._amg = amg if amg is not None else AMG(self.A, **params)
        self.set_linear_solver(self._lib.GCGE_CUDA_AMGPCG, self._amg.handle)
        return self._amg

    def solve(self, x0: np.ndarray | None = None):
        """x0: initial block, shape (nev, n) (= column-major n x nev); its first
        num_init_evec columns are used and the rest start pseudo-random (x0 =
        None with num_init_evec = 0: a random start)."""
        if x0 is not None:
            self.evec[...] = np.asarray(x0, dtype=np.float64).reshape(self.nev, self.n)
        L.check(self._lib.GCGE_CUDA_SOLVER_Solve(self.handle), "Solve")
        return self.eval.copy(), self.evec.copy()

    def residuals(self) -> np.ndarray:
        r = np.zeros(self.nev)
        L.check(self._lib.GCGE_CUDA_SOLVER_GetResiduals(self.handle, _ptr(r)), "GetResiduals")
        return r

    def stats(self) -> dict:
        st = L.Stats()
        L.check(self._lib.GCGE_CUDA_SOLVER_GetStats(self.handle, C.byref(st)), "GetStats")
        return st.as_dict()

    def close(self):
        if getattr(self, "handle", None):
            h = self.handle
            self._lib.GCGE_CUDA_SOLVER_Free(C.byref(h))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve(A, B, nev, x0, **params):
    """One-shot solve: returns (eigenvalues, eigenvectors (nev x n), stats)."""
    s = GCGESolver(A, B, nev, **params)
    try:
        ev, vec = s.solve(x0)
        return ev, vec, s.stats()
    finally:
        s.close()
