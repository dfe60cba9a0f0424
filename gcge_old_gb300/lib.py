"""ctypes binding of include/gcge_cuda.h.

``load()`` returns the CDLL of ``_build/libgcge_cuda.so`` with argument and
return types declared for every exported symbol.  It raises when the library
is missing; nothing here falls back to a CPU path.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_pp = C.POINTER(C.c_void_p)


class CSRHost(C.Structure):
    """GCGE_CUDA_CSR_HOST, layout of the reference CSR_MAT."""
    _fields_ = [("N_Rows", C.c_int), ("N_Columns", C.c_int), ("N_Entries", C.c_int),
                ("KCol", c_int_p), ("RowPtr", c_int_p), ("Entries", c_double_p)]


class PCGParam(C.Structure):
    """GCGE_CUDA_PCG_PARAM: steps and relative residual target of GCGE_CUDA_JacobiPCG."""
    _fields_ = [("max_it", C.c_int), ("rate", C.c_double)]


class ChebParam(C.Structure):
    """GCGE_CUDA_CHEB_PARAM: steps, residual target, polynomial degree and the
    lower end of the Chebyshev interval (a fraction of the Gershgorin bound)."""
    _fields_ = [("max_it", C.c_int), ("rate", C.c_double), ("degree", C.c_int),
                ("lower_frac", C.c_double)]


class AMGParam(C.Structure):
    """GCGE_CUDA_AMG_PARAM: hierarchy depth and coarsest size, aggregation
    strength, smoothed (1) or plain (0) prolongation, Chebyshev smoother degree
    and interval ratio, AMG-PCG step cap and residual target."""
    _fields_ = [("max_levels", C.c_int), ("coarse_size", C.c_int), ("strength", C.c_double),
                ("smooth_p", C.c_int), ("cheb_degree", C.c_int), ("cheb_ratio", C.c_double),
                ("pcg_max_it", C.c_int), ("pcg_rate", C.c_double)]


class PASEParam(C.Structure):
    """GCGE_CUDA_PASE_PARAM of the multilevel eigensolver."""
    _fields_ = [("more_nev", C.c_int), ("aux_level", C.c_int), ("max_cycles", C.c_int),
                ("smooth_steps", C.c_int), ("aux_max_it", C.c_int), ("initial_max_it", C.c_int),
                ("tol", C.c_double), ("initial_tol", C.c_double), ("aux_tol", C.c_double)]


class PASEStats(C.Structure):
    """GCGE_CUDA_PASE_STATS: cycle and iteration counts, final residual, phase times (s)."""
    _fields_ = [("cycles", C.c_int), ("initial_gcg_iterations", C.c_int),
                ("aux_gcg_iterations", C.c_int), ("smoothing_steps", C.c_int),
                ("max_residual", C.c_double), ("seconds", C.c_double),
                ("t_initial", C.c_double), ("t_smooth", C.c_double), ("t_aux_build", C.c_double),
                ("t_aux_solve", C.c_double), ("t_prolong", C.c_double), ("t_check", C.c_double)]


# GCGE_CUDA_MULTI_LINEAR_SOLVER(ctx, A, rhs, x, k, n, stream)
MultiLinearSolver = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, c_pp, c_pp, C.c_int, C.c_int,
                                C.c_void_p)


class Stats(C.Structure):
    """GCGE_CUDA_STATS."""
    _fields_ = [("num_iter", C.c_int), ("num_conv_continuous", C.c_int), ("bcg_steps", C.c_int),
                ("kernel_launches", C.c_longlong), ("seconds", C.c_double),
                ("t_x_orth", C.c_double), ("t_rr_mat", C.c_double), ("t_rr_eig", C.c_double),
                ("t_x_axpy", C.c_double), ("t_p", C.c_double), ("t_w_line", C.c_double),
                ("t_w_orth", C.c_double), ("t_conv", C.c_double), ("w_orth_passes", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> (restype, argtypes)
SIGNATURES = {
    "GCGE_CUDA_GetErrorString": (C.c_char_p, [C.c_int]),
    "GCGE_CUDA_GetLastErrorMessage": (C.c_char_p, []),
    "GCGE_CUDA_MatCreateFromCSR": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(CSRHost)]),
    "GCGE_CUDA_MatCreate": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_int]),
    "GCGE_CUDA_MatDestroy": (C.c_int, [C.POINTER(C.c_void_p)]),
    "GCGE_CUDA_MatGetSize": (C.c_int, [C.c_void_p, c_int_p, c_int_p]),
    "GCGE_CUDA_CSR_ReadFile": (C.c_int, [C.c_char_p, C.POINTER(CSRHost)]),
    "GCGE_CUDA_CSR_WriteText": (C.c_int, [C.c_char_p, C.POINTER(CSRHost)]),
    "GCGE_CUDA_CSR_WriteBinary": (C.c_int, [C.c_char_p, C.POINTER(CSRHost)]),
    "GCGE_CUDA_CSR_Free": (C.c_int, [C.POINTER(CSRHost)]),
    "GCGE_CUDA_MatCreateFromFile": (C.c_int, [C.POINTER(C.c_void_p), C.c_char_p]),
    "GCGE_CUDA_SOLVER_Create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "GCGE_CUDA_SOLVER_SetMatA": (C.c_int, [C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_SOLVER_SetMatB": (C.c_int, [C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_SOLVER_SetNumEigen": (C.c_int, [C.c_void_p, C.c_int]),
    "GCGE_CUDA_SOLVER_SetEigenvalues": (C.c_int, [C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_SOLVER_SetEigenvectors": (C.c_int, [C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_SOLVER_SetEigenvectorsDevice": (C.c_int, [C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_SOLVER_GetStream": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "GCGE_CUDA_SOLVER_SetFromCommandLine": (C.c_int, [C.c_void_p, C.c_int,
                                                      C.POINTER(C.c_char_p)]),
    "GCGE_CUDA_SOLVER_SetParamInt": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "GCGE_CUDA_SOLVER_SetParamDouble": (C.c_int, [C.c_void_p, C.c_char_p, C.c_double]),
    "GCGE_CUDA_SOLVER_Setup": (C.c_int, [C.c_void_p]),
    "GCGE_CUDA_SOLVER_Solve": (C.c_int, [C.c_void_p]),
    "GCGE_CUDA_SOLVER_GetEigenvalues": (C.c_int, [C.c_void_p, C.POINTER(c_double_p)]),
    "GCGE_CUDA_SOLVER_GetEigenvectors": (C.c_int, [C.c_void_p, C.POINTER(c_double_p)]),
    "GCGE_CUDA_SOLVER_GetResiduals": (C.c_int, [C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_SOLVER_GetStats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "GCGE_CUDA_SOLVER_Free": (C.c_int, [C.POINTER(C.c_void_p)]),
    "GCGE_CUDA_SOLVER_Free_All": (C.c_int, [C.POINTER(C.c_void_p)]),
    "GCGE_CUDA_Solver_Init": (C.c_void_p, [C.POINTER(CSRHost), C.POINTER(CSRHost), C.c_int,
                                           C.c_int, C.POINTER(C.c_char_p)]),
    "GCGE_CUDA_MatDotMultiVec": (C.c_int, [C.c_void_p, c_pp, c_pp, C.c_int]),
    "GCGE_CUDA_MatDotMultiVecAsync": (C.c_int, [C.c_void_p, c_pp, c_pp, C.c_int, C.c_void_p]),
    "GCGE_CUDA_MatDotMultiVecF32Async": (C.c_int, [C.c_void_p, c_pp, c_pp, C.c_int, C.c_void_p]),
    "GCGE_CUDA_SOLVER_SetMultiLinearSolver": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_JacobiPCG": (C.c_int, [C.c_void_p, C.c_void_p, c_pp, c_pp, C.c_int, C.c_int,
                                      C.c_void_p]),
    "GCGE_CUDA_ChebyshevPCG": (C.c_int, [C.c_void_p, C.c_void_p, c_pp, c_pp, C.c_int, C.c_int,
                                      C.c_void_p]),
    "GCGE_CUDA_AMG_DefaultParam": (None, [C.c_void_p]),
    "GCGE_CUDA_AMG_Create": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_AMG_Destroy": (C.c_int, [C.c_void_p]),
    "GCGE_CUDA_AMG_GetNumLevels": (C.c_int, [C.c_void_p, c_int_p]),
    "GCGE_CUDA_AMG_GetLevelInfo": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_int_p, c_int_p,
                                             c_double_p]),
    "GCGE_CUDA_AMG_GetLevelCSR": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_int_p, c_int_p,
                                            c_double_p]),
    "GCGE_CUDA_AMG_GetAggregates": (C.c_int, [C.c_void_p, C.c_int, c_int_p]),
    "GCGE_CUDA_AMG_Apply": (C.c_int, [C.c_void_p, c_pp, c_pp, C.c_int, C.c_void_p]),
    "GCGE_CUDA_AMGPCG": (C.c_int, [C.c_void_p, C.c_void_p, c_pp, c_pp, C.c_int, C.c_int,
                                   C.c_void_p]),
    "GCGE_CUDA_AMG_GetLastSteps": (C.c_int, [C.c_void_p, c_int_p]),
    "GCGE_CUDA_PASE_DefaultParam": (None, [C.c_void_p]),
    "GCGE_CUDA_PASE_Solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                       c_double_p, C.c_void_p, C.c_void_p]),
    "GCGE_CUDA_EigvecAdjointSolve": (C.c_int, [C.c_void_p, C.c_void_p, c_pp, c_double_p, C.c_int,
                                              c_pp, c_pp, c_double_p, C.c_int, C.c_double,
                                              c_int_p]),
    "GCGE_CUDA_EigvecAdjointSolveAMG": (C.c_int, [C.c_void_p, C.c_void_p, c_pp, c_double_p,
                                                 C.c_int, c_pp, c_pp, c_double_p, C.c_int,
                                                 C.c_double, c_int_p, C.c_void_p]),
    "GCGE_CUDA_EigGradCSR2": (C.c_int, [C.c_void_p, c_pp, c_pp, c_double_p, c_double_p, C.c_int,
                                        C.c_void_p]),
    "GCGE_CUDA_EigGradCSR": (C.c_int, [C.c_void_p, c_pp, C.c_void_p, C.c_int, C.c_void_p]),
    "GCGE_CUDA_MatDotRowsF32Async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                               C.c_void_p]),
    "GCGE_CUDA_MultiVecInnerProd": (C.c_int, [c_pp, C.c_int, c_pp, C.c_int, C.c_int, C.c_void_p,
                                              C.c_int, C.c_int]),
    "GCGE_CUDA_MultiVecInnerProdOzaki": (C.c_int, [c_pp, C.c_int, c_pp, C.c_int, C.c_int,
                                                   C.c_void_p, C.c_int, C.c_int]),
    "GCGE_CUDA_SetOps": (C.c_int, [C.c_void_p]),
    "GCGE_CUDA_MultiVecCreate": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "GCGE_CUDA_MultiVecDestroy": (C.c_int, [C.c_void_p]),
    "GCGE_CUDA_MultiVecSetFromHost": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                C.c_int]),
    "GCGE_CUDA_MultiVecGetToHost": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]),
    "GCGE_CUDA_OpsGetError": (C.c_int, []),
    "GCGE_CUDA_OpsClearError": (None, []),
    "GCGE_CUDA_PlanesBytes": (C.c_size_t, [C.c_int, C.c_int]),
    "GCGE_CUDA_PlanesGramScratchDoubles": (C.c_size_t, [C.c_int, C.c_int]),
    "GCGE_CUDA_PlanesCut": (C.c_int, [c_pp, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                      C.c_int, C.c_void_p]),
    "GCGE_CUDA_PlanesGram": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                       C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                       C.c_void_p]),
    "GCGE_CUDA_MultiVecInnerProdPlanes": (C.c_int, [c_pp, C.c_int, c_pp, C.c_int, C.c_int,
                                                    C.c_void_p, C.c_void_p, C.c_int]),
    "GCGE_CUDA_MultiVecInnerProdNoAlloc": (C.c_int, [c_pp, C.c_int, c_pp, C.c_int, C.c_int,
                                                     C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "GCGE_CUDA_MultiVecLinearComb": (C.c_int, [c_pp, C.c_int, c_pp, C.c_int, C.c_int, C.c_void_p,
                                               C.c_int, C.c_double]),
    "GCGE_CUDA_MultiVecLinearCombOzaki": (C.c_int, [c_pp, C.c_int, c_pp, C.c_int, C.c_int,
                                                    C.c_void_p, C.c_int, C.c_double]),
    "GCGE_CUDA_MultiVecAxpby": (C.c_int, [C.c_double, c_pp, C.c_double, c_pp, C.c_int, C.c_int]),
    "GCGE_CUDA_DenseMatEigenSolver": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "GCGE_CUDA_BlockCG": (C.c_int, [C.c_void_p, c_pp, c_pp, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.c_int, c_int_p]),
}

_lib = None


def load(build_if_missing: bool = False):
    """Load the CUDA library (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                "GB300 CUDA library %s is not built; run __graft_entry__.build() "
                "(no CPU fallback exists)" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class GcgeCudaError(RuntimeError):
    pass


def check(rc: int, what: str = ""):
    if rc != 0:
        lib = load()
        msg = lib.GCGE_CUDA_GetLastErrorMessage().decode(errors="replace")
        name = lib.GCGE_CUDA_GetErrorString(rc).decode()
        raise GcgeCudaError("%s: %s (%d) %s" % (what, name, rc, msg))
