"""ORACLE TEST INFRASTRUCTURE — not part of the product.

ctypes front end for the two CPU checkers of the GCG eigensolver path:

* the oracle port (``oracle/gcge_port.c``): a C restatement of the reference
  GCGE_Solve (src/gcge_eigsol.c:65-646) and everything below it; it builds
  anywhere gcc is present;
* the reference itself (``oracle/_ref/libgcge_ref.so``), compiled from the
  reference checkout by ``oracle/build_ref.sh`` where that checkout exists.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SRC = os.path.join(HERE, "gcge_port.c")
# where the reference checkout is read from when the checker is built (the
# reference is never needed at run time): $GCGE_REFERENCE_DIR, else the
# checkout location of the build container
REFERENCE_DIR = os.environ.get("GCGE_REFERENCE_DIR", "/root/reference")
PORT_SO = os.path.join(HERE, "_build", "libgcge_port.so")
REF_SO = os.path.join(HERE, "_ref", "libgcge_ref.so")


class PortPara(C.Structure):
    """Mirror of port_para in gcge_port.c (defaults: src/gcge_para.c:25-113)."""
    _fields_ = [("nev", C.c_int), ("block_size", C.c_int), ("ev_max_it", C.c_int),
                ("cg_max_it", C.c_int), ("max_reorth_time", C.c_int),
                ("ev_tol", C.c_double), ("cg_rate", C.c_double),
                ("orth_zero_tol", C.c_double), ("reorth_tol", C.c_double),
                ("scbgs_reorth_tol", C.c_double), ("multi_tol_for_lock", C.c_double),
                ("use_shift", C.c_int), ("if_shift", C.c_int), ("eval_sm", C.c_int),
                ("shift", C.c_double), ("mixed", C.c_int), ("conv_type", C.c_int),
                ("conv_omega_norm", C.c_double)]


def build_port(force: bool = False) -> str:
    """Compile the oracle port (OpenMP enabled) into oracle/_build/."""
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < os.path.getmtime(PORT_SRC):
        os.makedirs(os.path.dirname(PORT_SO), exist_ok=True)
        tmp = PORT_SO + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-o", tmp,
                               PORT_SRC, "-lm"])
        os.replace(tmp, PORT_SO)
    return PORT_SO


def reference_present() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_DIR, "src", "gcge_eigsol.c"))


def build_ref() -> str | None:
    """Compile the reference into oracle/_ref/ when its checkout is present."""
    script = os.path.join(HERE, "build_ref.sh")
    r = subprocess.run(["bash", script, REFERENCE_DIR], capture_output=True, text=True)
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


_port = None
_ref = None


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def port_lib():
    global _port
    if _port is None:
        _port = C.CDLL(build_port())
        _port.gcge_port_solve.restype = C.c_int
        _port.gcge_port_default_para.restype = None
        assert _port.gcge_port_para_size() == C.sizeof(PortPara)
    return _port


def default_para(nev: int, **kw) -> PortPara:
    p = PortPara()
    port_lib().gcge_port_default_para(C.byref(p), nev)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def port_solve(A, B, nev, x0, para: PortPara | None = None, max_outer: int = -1,
               threads: int | None = None):
    """Run the oracle port (threads: OpenMP threads, default 1 like the
    single-threaded reference).  Returns dict(eval, evec (nev x n rows =
    columns), res, iters, seconds, spmv)."""
    lib = port_lib()
    lib.gcge_port_set_threads(int(threads) if threads is not None else 1)
    para = para or default_para(nev)
    n = A.n
    x0 = np.ascontiguousarray(x0, dtype=np.float64).reshape(nev, n)
    ev = np.zeros(nev)
    vec = np.zeros((nev, n))
    res = np.zeros(nev)
    it = C.c_int(0)
    sec = C.c_double(0)
    nsp = C.c_longlong(0)
    ph = np.zeros(3)
    rc = lib.gcge_port_solve(
        C.c_int(n), _iptr(A.rowptr), _iptr(A.col), _dptr(A.val),
        _iptr(B.rowptr) if B is not None else None, _iptr(B.col) if B is not None else None,
        _dptr(B.val) if B is not None else None, C.byref(para), _dptr(x0), C.c_int(max_outer),
        _dptr(ev), _dptr(vec), _dptr(res), C.byref(it), C.byref(sec), C.byref(nsp), _dptr(ph))
    if rc != 0:
        raise RuntimeError("oracle port failed: %d" % rc)
    return dict(eval=ev, evec=vec, res=res, iters=it.value, seconds=sec.value, spmv=nsp.value,
                t_init=ph[0], t_loop=ph[1], loop_iters=int(ph[2]))


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("oracle/_ref/libgcge_ref.so not built")
        _ref = C.CDLL(REF_SO)
        _ref.ref_gcge_solve.restype = C.c_int
    return _ref


class _RefCSR(C.Structure):
    # CSR_MAT of app/csr/gcge_app_csr.h:27-41
    _fields_ = [("N_Rows", C.c_int), ("N_Columns", C.c_int), ("N_Entries", C.c_int),
                ("KCol", C.POINTER(C.c_int)), ("RowPtr", C.POINTER(C.c_int)),
                ("Entries", C.POINTER(C.c_double))]


def ref_read_csr(path: str):
    """The reference's own CSR_ReadMatFile (app/csr/gcge_app_csr.c:185-236) on a
    text file: returns (nrow, ncol, rowptr, col, val) as numpy arrays.  The
    reference exits the process on a missing file, so the path is checked first."""
    import numpy as np
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = ref_lib()
    lib.CSR_ReadMatFile.restype = C.POINTER(_RefCSR)
    lib.CSR_ReadMatFile.argtypes = [C.c_char_p]
    m = lib.CSR_ReadMatFile(os.fsencode(path))
    c = m.contents
    n, nnz = c.N_Rows, c.N_Entries
    out = (n, c.N_Columns, np.ctypeslib.as_array(c.RowPtr, (n + 1,)).copy(),
           np.ctypeslib.as_array(c.KCol, (nnz,)).copy(),
           np.ctypeslib.as_array(c.Entries, (nnz,)).copy())
    lib.CSR_MatFree.argtypes = [C.POINTER(C.POINTER(_RefCSR))]
    lib.CSR_MatFree(C.byref(m))
    return out


def ref_solve(A, B, nev, x0, flags: dict | None = None):
    """Run the unmodified reference through GCGE_CSR_Solver_Init / Solve with
    the initial block x0 passed as num_init_evec = nev."""
    lib = ref_lib()
    n = A.n
    fl = {"-gcge_num_init_evec": nev, "-gcge_print_para": 0, "-gcge_print_result": 0,
          "-gcge_print_final_part_time": 0, "-gcge_print_conv": 0, "-gcge_print_eval": 0}
    fl.update(flags or {})
    args = ["ref"]
    for k, v in fl.items():
        args += [k, str(v)]
    argv = (C.c_char_p * len(args))(*[a.encode() for a in args])
    x0 = np.ascontiguousarray(x0, dtype=np.float64).reshape(nev, n)
    ev = np.zeros(nev)
    vec = np.zeros((nev, n))
    res = np.zeros(nev)
    it = C.c_int(0)
    sec = C.c_double(0)
    rc = lib.ref_gcge_solve(
        C.c_int(n), _iptr(A.rowptr), _iptr(A.col), _dptr(A.val),
        _iptr(B.rowptr) if B is not None else None, _iptr(B.col) if B is not None else None,
        _dptr(B.val) if B is not None else None, C.c_int(nev), _dptr(x0), C.c_int(len(args)),
        argv, _dptr(ev), _dptr(vec), C.byref(it), C.byref(sec), _dptr(res))
    if rc != 0:
        raise RuntimeError("reference driver failed: %d" % rc)
    return dict(eval=ev, evec=vec, res=res, iters=it.value, seconds=sec.value)


def true_residuals(A, B, ev, vecs):
    """||A x - lambda B x|| / (|lambda| ||x||) per pair, in FP64 (scipy)."""
    a = A.to_scipy()
    b = B.to_scipy() if B is not None else None
    out = np.zeros(len(ev))
    for k in range(len(ev)):
        x = vecs[k]
        bx = b @ x if b is not None else x
        r = a @ x - ev[k] * bx
        out[k] = np.linalg.norm(r) / (abs(ev[k]) * np.linalg.norm(x))
    return out
