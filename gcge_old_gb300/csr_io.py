"""Matrix files through the library's native readers and writers
(GCGE_CUDA_CSR_ReadFile / WriteText / WriteBinary): the reference's CSR text
format (CSR_ReadMatFile, app/csr/gcge_app_csr.c:185-236) and PETSc's binary Mat
format, detected from the first four bytes on read."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import lib as L
from .matrices import CSRMatrix


def read_csr(path: str | os.PathLike) -> CSRMatrix:
    """Reads a square matrix from a CSR text or PETSc binary file."""
    lib = L.load()
    h = L.CSRHost()
    L.check(lib.GCGE_CUDA_CSR_ReadFile(os.fsencode(path), C.byref(h)), "CSR_ReadFile")
    try:
        n, nnz = h.N_Rows, h.N_Entries
        if h.N_Columns != n:
            raise ValueError("%s: %d x %d matrix is not square" % (path, n, h.N_Columns))
        rp = np.ctypeslib.as_array(h.RowPtr, (n + 1,)).copy()
        ci = np.ctypeslib.as_array(h.KCol, (nnz,)).copy() if nnz else np.zeros(0, np.int32)
        va = np.ctypeslib.as_array(h.Entries, (nnz,)).copy() if nnz else np.zeros(0)
    finally:
        lib.GCGE_CUDA_CSR_Free(C.byref(h))
    return CSRMatrix(n, rp.astype(np.int32), ci.astype(np.int32), va.astype(np.float64))


def _host(A: CSRMatrix):
    rp = np.ascontiguousarray(A.rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(A.col, dtype=np.int32)
    va = np.ascontiguousarray(A.val, dtype=np.float64)
    h = L.CSRHost(A.n, A.n, int(rp[-1]), ci.ctypes.data_as(L.c_int_p),
                  rp.ctypes.data_as(L.c_int_p), va.ctypes.data_as(L.c_double_p))
    return h, (rp, ci, va)


def write_csr_text(path: str | os.PathLike, A: CSRMatrix) -> None:
    h, keep = _host(A)
    L.check(L.load().GCGE_CUDA_CSR_WriteText(os.fsencode(path), C.byref(h)), "CSR_WriteText")


def write_csr_binary(path: str | os.PathLike, A: CSRMatrix) -> None:
    h, keep = _host(A)
    L.check(L.load().GCGE_CUDA_CSR_WriteBinary(os.fsencode(path), C.byref(h)), "CSR_WriteBinary")
