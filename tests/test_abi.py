"""CPU tests of the C ABI: the library builds, loads and exports every
function include/gcge_cuda.h declares; host-side argument checking works
without touching a GPU."""
import ctypes as C
import os
import re

import numpy as np

from conftest import ROOT


def header_functions():
    """Every GCGE_CUDA_* function declared in include/*.h (the table's
    struct fields are members, not exports: only names followed by "(" at the
    start of a declaration count)."""
    import glob
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"^[A-Za-z_][\w\s\*]*?\b(GCGE_CUDA_\w+)\s*\(", txt, flags=re.M))
    return sorted(names)


def test_library_builds_and_exports_header(tmp_path):
    from gcge_old_gb300 import build as B
    from gcge_old_gb300 import lib as L
    path = B.build()
    assert os.path.exists(path)
    lib = C.CDLL(path)
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares every exported function
    assert set(names) <= set(L.SIGNATURES), set(names) - set(L.SIGNATURES)


def test_error_strings_and_host_side_checks():
    from gcge_old_gb300 import lib as L
    lib = L.load(build_if_missing=True)
    assert lib.GCGE_CUDA_GetErrorString(0) == b"ok"
    assert lib.GCGE_CUDA_GetErrorString(1) == b"invalid argument"
    # malformed CSR is rejected before any device allocation
    rp = np.array([0, 2, 1], dtype=np.int32)
    ci = np.array([0, 1], dtype=np.int32)
    v = np.ones(2)
    h = C.c_void_p()
    p = lambda a: C.c_void_p(a.ctypes.data)
    assert lib.GCGE_CUDA_MatCreate(C.byref(h), 2, p(rp), p(ci), p(v), 0) == 1
    assert b"RowPtr" in lib.GCGE_CUDA_GetLastErrorMessage()
    rp = np.array([1, 1, 2], dtype=np.int32)
    assert lib.GCGE_CUDA_MatCreate(C.byref(h), 2, p(rp), p(ci), p(v), 0) == 1
    assert lib.GCGE_CUDA_MatCreate(C.byref(h), 0, p(rp), p(ci), p(v), 0) == 1


def test_solver_parameter_surface_without_gpu():
    from gcge_old_gb300 import lib as L
    lib = L.load(build_if_missing=True)
    s = C.c_void_p()
    assert lib.GCGE_CUDA_SOLVER_Create(C.byref(s)) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"block_size", 10) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamDouble(s, b"-gcge_ev_tol", 1e-10) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"no_such_flag", 1) == 1
    args = [b"prog", b"-gcge_nev", b"7", b"-gcge_cg_rate", b"0.05", b"-unknown", b"-gcge_precision",
            b"mixed"]
    argv = (C.c_char_p * len(args))(*args)
    assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, len(args), argv) == 0
    # shift and eval_type (GCGE_PARA use_shift / if_shift / shift / eval_type)
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"use_shift", 1) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamDouble(s, b"shift", 2.5) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"eval_type", 1) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"eval_type", 2) == 1
    for flag in ([b"-gcge_eval_type", b"sm"], [b"-gcge_use_shift", b"0"]):
        argv = (C.c_char_p * 2)(*flag)
        assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, 2, argv) == 0
    argv = (C.c_char_p * 2)(b"-gcge_eval_type", b"lm")
    assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, 2, argv) == 1
    bad = [b"-gcge_precision", b"half"]
    argv = (C.c_char_p * 2)(*bad)
    assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, 2, argv) == 1
    # Solve before Setup is a state error, not a crash
    assert lib.GCGE_CUDA_SOLVER_Solve(s) == 4
    stream = C.c_void_p()
    assert lib.GCGE_CUDA_SOLVER_GetStream(s, C.byref(stream)) == 4
    assert lib.GCGE_CUDA_SOLVER_Free(C.byref(s)) == 0
    assert not s.value


def test_new_entry_points_check_arguments_without_gpu():
    """The W-step hook, the stock PCG, the eigenvector adjoint and the file
    readers reject bad arguments before any device work."""
    from gcge_old_gb300 import lib as L
    lib = L.load(build_if_missing=True)
    s = C.c_void_p()
    assert lib.GCGE_CUDA_SOLVER_Create(C.byref(s)) == 0
    assert lib.GCGE_CUDA_SOLVER_SetMultiLinearSolver(s, C.cast(lib.GCGE_CUDA_JacobiPCG, C.c_void_p),
                                                     None) == 0
    assert lib.GCGE_CUDA_SOLVER_SetMultiLinearSolver(s, None, None) == 0
    assert lib.GCGE_CUDA_SOLVER_SetMultiLinearSolver(None, None, None) == 1
    assert lib.GCGE_CUDA_SOLVER_Free(C.byref(s)) == 0
    assert lib.GCGE_CUDA_JacobiPCG(None, None, None, None, 1, 10, None) == 1
    assert lib.GCGE_CUDA_ChebyshevPCG(None, None, None, None, 1, 10, None) == 1
    assert lib.GCGE_CUDA_AMG_Create(None, None, None) == 1
    assert lib.GCGE_CUDA_AMGPCG(None, None, None, None, 1, 10, None) == 1
    assert lib.GCGE_CUDA_AMG_Apply(None, None, None, 1, None) == 1
    prm = L.AMGParam()
    lib.GCGE_CUDA_AMG_DefaultParam(C.byref(prm))
    assert (prm.max_levels, prm.coarse_size, prm.smooth_p, prm.cheb_degree) == (10, 256, 1, 3)
    assert (prm.pcg_max_it, prm.pcg_rate) == (20, 1e-2)
    pp = L.PASEParam()
    lib.GCGE_CUDA_PASE_DefaultParam(C.byref(pp))
    assert (pp.more_nev, pp.aux_level, pp.smooth_steps, pp.aux_max_it, pp.tol) == (10, 1, 2, 3, 1e-10)
    assert lib.GCGE_CUDA_PASE_Solve(None, None, None, 4, None, None, None, None) == 1
    ev = np.array([1.0, 2.0])
    assert lib.GCGE_CUDA_EigvecAdjointSolve(None, None, None, ev.ctypes.data_as(L.c_double_p), 2,
                                            None, None, None, 10, 1e-8, None) == 1
    a = np.ones(2)
    assert lib.GCGE_CUDA_EigGradCSR2(None, None, None, a.ctypes.data_as(L.c_double_p), None, 2,
                                     None) == 1
    assert lib.GCGE_CUDA_MatGetSize(None, None, None) == 1
    assert lib.GCGE_CUDA_MatCreateFromFile(None, b"x") == 1


def _argv(*args):
    return len(args), (C.c_char_p * len(args))(*[a.encode() for a in args])


def test_command_line_rejects_what_it_does_not_honour():
    """Reference flags (src/gcge_para.c:128-407) are honoured, accepted where
    they have no effect on one GPU, accepted only at the value this solver
    implements, or rejected: none is dropped silently."""
    from gcge_old_gb300 import lib as L
    lib = L.load(build_if_missing=True)
    s = C.c_void_p()
    assert lib.GCGE_CUDA_SOLVER_Create(C.byref(s)) == 0
    ok = [("-gcge_conv_type", "O"), ("-gcge_conv_type", "A"), ("-gcge_conv_type", "R"),
          ("-gcge_conv_omega_norm", "3.5"), ("-gcge_orth_type", "B"),
          ("-gcge_w_orth_type", "multi"), ("-gcge_p_orth_type", "multi"),
          ("-gcge_x_orth_type", "bgs"), ("-gcge_if_use_bcg", "1"), ("-gcge_if_use_cg", "1"),
          ("-gcge_use_bcg_continuous", "0"), ("-gcge_if_lobgcg", "0"),
          ("-gcge_opt_rr_eig_partly", "0"), ("-gcge_opt_bcast", "1"), ("-gcge_multi_tol", "0.3"),
          ("-gcge_print_result", "0"), ("-gcge_print_final_part_time", "0"),
          ("-gcge_w_form", "correction"), ("-gcge_w_form", "reference")]
    for f, v in ok:
        assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, *_argv(f, v)) == 0, (f, v)
    bad = [("-gcge_w_orth_type", "scbgs"), ("-gcge_x_orth_type", "scbgs"), ("-gcge_orth_type", "A"),
           ("-gcge_if_use_bcg", "0"), ("-gcge_use_bcg_continuous", "1"), ("-gcge_if_lobgcg", "1"),
           ("-gcge_w_orth_block_size", "5"), ("-gcge_conv_type", "X"), ("-gcge_no_such_flag", "1"),
           ("-gcge_w_form", "other")]
    for f, v in bad:
        assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, *_argv(f, v)) == 1, (f, v)
        assert f.encode() in lib.GCGE_CUDA_GetLastErrorMessage(), f
    # a flag without its value
    assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, *_argv("prog", "-gcge_nev")) == 1
    # arguments that are not -gcge_* flags are skipped, as the reference skips them
    assert lib.GCGE_CUDA_SOLVER_SetFromCommandLine(s, *_argv("prog", "-other", "x")) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"conv_type", 1) == 0
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"conv_type", 3) == 1
    assert lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"w_form", 1) == 0
    assert lib.GCGE_CUDA_SOLVER_Free(C.byref(s)) == 0
