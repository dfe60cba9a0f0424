#!/usr/bin/env python3
"""Benchmark of the GB300 GCG eigensolver (one JSON line on stdout).

Workload (the reference's headline GPU configuration): 3D 7-point Laplacian
scaled by h on a 128^3 interior grid (n = 2,097,152, nnz = 14,581,760),
h = 1/129, B = diagonal lumped mass h^3 (1 + U(-0.1, 0.1)) from seed 0,
nev = 50 smallest pairs, relative residual ||Ax - lambda Bx|| / (|lambda| ||x||)
<= 1e-10 for every pair (the reference's "R" criterion with ev_tol = 1e-10:
all lambda > 1), seeded N(0,1) initial block.  A step is one complete solve.

value: seconds per solve of the mixed-precision form (FP32 block CG, FP64
everything else) with the matrices and the initial block resident in HBM,
timed with CUDA events on the solver's stream; fp64_s: the all-FP64 form
(FP64 block CG; tall-skinny products FP64-accurate on the tensor cores in both
forms); fp64_correction_form_s: the FP64 form with the mixed form's W step (the
block-CG correction alone as the W block), so that mixed vs it differs in the
precision of the block CG only; fp64_fma_products_s: one FP64 solve with those products on FP64 FMA
units instead; tuned_inner_solve: one solve of each form with the block size
and block-CG step cap that suit it (mixed 12 / 40, FP64 15 / 40; the
reference's defaults 10 / 20 are what value uses).
e2e: the same solve through the C ABI with HOST buffers: matrix upload,
initial block upload and eigenvector download inside the timed region.
roofline: the Gram pass of the W orthogonalisation, the solve's largest
kernel family: the digit-plane cut of W (diagonal B folded in) and the plane
Gram [X,P]^T diag(b) W at 80 x 10 columns, algorithmic bytes (80+10+1)*n*8
per pass; the per-iteration cut of the basis planes beside it.  rooflines:
the SpMM of the mixed solve's block CG (FP32 CSR SpMM on row-interleaved
blocks, k = 10, algorithmic bytes nnz*8 + 4(n+1) + 2*k*n*4 per launch) and
the FP64 and FP32 column SpMMs.
cpu_baseline: the oracle port (C restatement of the reference, OpenMP on all
host cores) on a bounded sample of the same solve: the start phase plus three
GCG iterations, extrapolated to the reference's iteration count and corrected
by the committed full solve of the port on the same host
(profiles/cpu_port_full_solve_lap3d128.json, `--calibrate-cpu`): the first
iterations cost more than the average one.

--impl reference runs that CPU path alone (rank 0), each step one bounded
sample, and prints the same metric.

--config 3 instead runs the mixed-precision configuration of the headline
once in each precision: 27-point Q1 variable-coefficient diffusion (per-cell
kappa = exp(N(0,1))) with its consistent mass on a 160^3 grid (n = 4,096,000,
nnz = 109,215,352), nev = 100, at --c3tol (default 1e-11: with a mass matrix
of size h^3 the residual bound 1e-10 leaves the eigenvalues free by more than
1e-10 relative), and reports both times, the per-pair difference of the mixed
result from the FP64 one and of each from the oracle port's solve
(tests/golden/cfg3_port_summary.json), as a JSON line of its own.

--config 4 runs the differentiation configuration: 2D anisotropic diffusion
(5-point, per-cell kappa ~ U(0.5, 2), y-edges weighted 10) on a 512 x 512
grid with diagonal mass, nev = 32, loss = sum_k w_k lambda_k
+ ||x_1 * mask||^2; it times the forward solve and the backward pass (the
eigenvalue and eigenvector adjoints), checks the gradients with respect to
kappa and to A's and B's values against central differences of the solver,
and the same on a 64 x 64 copy against adjoints from a dense generalized
eigendecomposition.

--config 5 runs the uneven-row configuration: the shifted graph Laplacian
A = L + 1e-3 I of a seeded Chung-Lu power-law graph (n = 8M, mean degree 16,
exponent 2.5, edge weights U(0.5, 1.5)) with B = D, nev = 128, in mixed
precision, capped at --c5it GCG iterations (the reference's method converges
slowly on this clustered spectrum: its oracle port leaves 23 of 128 pairs above
1e-10 after 300 iterations at n = 20,000); it reports the time per iteration,
the converged pairs, and the gradient of sum_k w_k lambda_k with respect to
the edge weights from the solve's vectors (the CSR-value adjoint kernel),
checked against the closed form per edge on 10,000 sampled edges; the
finite-difference check of the same assembly runs on a small graph in
tests/test_gpu_uneven.py.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "s to nev eigenpairs @1e-10 resid: mixed vs FP64 on GB300; SpMM HBM GB/s"
# iteration count of the reference GCGE on this workload (num_iter, counted
# as para->num_iter: the start RR check, the [X,W] step, then one per loop)
REF_ITERS_FILE = os.path.join(HERE, "tests", "golden", "cfg2_reference_summary.json")


def workload(small: bool):
    from gcge_old_gb300 import matrices as M
    m = 48 if small else 128
    A, B = M.laplace3d_mass(m, seed=0)
    nev = 50
    x0 = M.initial_block(A.n, nev, seed=0)
    return A, B, nev, x0, m


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.p = None
        self.path = os.path.join("/tmp", "gcge_clocks_%d_%d.csv" % (os.getpid(), gpu_index))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def time_solves(torch, S, L, dA, dB, nev, x0_dev, precision, warmup, steps, gemm="ozaki", **kw):
    """Solves with device-resident inputs; returns (times_s, stats, eval, evec_dev)."""
    lib = L.load()
    kw.setdefault("ev_tol", 1e-10)
    mls = kw.pop("mls", None)
    s = S.GCGESolver(dA, dB, nev, ev_max_it=1000, precision=precision, gemm=gemm, **kw)
    if mls is not None:
        s.use_amg_pcg(mls)
    evec_dev = torch.empty_like(x0_dev)
    L.check(lib.GCGE_CUDA_SOLVER_SetEigenvectorsDevice(s.handle, C.c_void_p(evec_dev.data_ptr())),
            "SetEigenvectorsDevice")
    sp = C.c_void_p()
    L.check(lib.GCGE_CUDA_SOLVER_GetStream(s.handle, C.byref(sp)), "GetStream")
    stream = torch.cuda.ExternalStream(sp.value)
    times = []
    stats = []
    for it in range(warmup + steps):
        evec_dev.copy_(x0_dev)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.check(lib.GCGE_CUDA_SOLVER_Solve(s.handle), "Solve")
        e1.record(stream)
        torch.cuda.synchronize()
        if it >= warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
            stats.append(s.stats())
    ev = s.eval.copy()
    s.close()
    return times, stats, ev, evec_dev


def spmm_roofline(torch, L, dA, A, k, launches=20):
    lib = L.load()
    n = A.n
    X = [torch.randn(n, dtype=torch.float64, device="cuda") for _ in range(k)]
    Y = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(k)]
    xp = (C.c_void_p * k)(*[C.c_void_p(t.data_ptr()) for t in X])
    yp = (C.c_void_p * k)(*[C.c_void_p(t.data_ptr()) for t in Y])
    st = torch.cuda.Stream()
    for _ in range(3):
        L.check(lib.GCGE_CUDA_MatDotMultiVecAsync(dA.handle, xp, yp, k, C.c_void_p(st.cuda_stream)), "spmm")
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(launches):
        L.check(lib.GCGE_CUDA_MatDotMultiVecAsync(dA.handle, xp, yp, k, C.c_void_p(st.cuda_stream)), "spmm")
    e1.record(st)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / launches
    # check against scipy on one column
    y0 = Y[0].cpu().numpy()
    ref = A.to_scipy() @ X[0].cpu().numpy()
    assert np.allclose(y0, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    nbytes = A.nnz * 12 + 4 * (n + 1) + 2 * k * n * 8
    # FP32 SpMM of the mixed inner solve (same k)
    X32 = [t.float() for t in X]
    Y32 = [torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(k)]
    xp32 = (C.c_void_p * k)(*[C.c_void_p(t.data_ptr()) for t in X32])
    yp32 = (C.c_void_p * k)(*[C.c_void_p(t.data_ptr()) for t in Y32])
    for _ in range(3):
        L.check(lib.GCGE_CUDA_MatDotMultiVecF32Async(dA.handle, xp32, yp32, k, C.c_void_p(st.cuda_stream)), "spmm32")
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(launches):
        L.check(lib.GCGE_CUDA_MatDotMultiVecF32Async(dA.handle, xp32, yp32, k, C.c_void_p(st.cuda_stream)), "spmm32")
    e1.record(st)
    torch.cuda.synchronize()
    t32 = e0.elapsed_time(e1) / 1e3 / launches
    nbytes32 = A.nnz * 8 + 4 * (n + 1) + 2 * k * n * 4
    # the SpMM of the mixed solve's block CG: FP32 on row-interleaved blocks
    kw = (k + 3) // 4 * 4
    XR = torch.randn(n, kw, dtype=torch.float32, device="cuda")
    YR = torch.empty(n, kw, dtype=torch.float32, device="cuda")
    for _ in range(3):
        L.check(lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(XR.data_ptr()),
                                                 C.c_void_p(YR.data_ptr()), k,
                                                 C.c_void_p(st.cuda_stream)), "spmm rows")
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(launches):
        L.check(lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(XR.data_ptr()),
                                                 C.c_void_p(YR.data_ptr()), k,
                                                 C.c_void_p(st.cuda_stream)), "spmm rows")
    e1.record(st)
    torch.cuda.synchronize()
    trows = e0.elapsed_time(e1) / 1e3 / launches
    ref = (A.to_scipy() @ XR[:, 0].double().cpu().numpy())
    assert np.allclose(YR[:, 0].double().cpu().numpy(), ref, rtol=0, atol=1e-5 * np.abs(ref).max())
    return t, nbytes, t32, nbytes32, trows


def gram_roofline(torch, L, n, k1=80, k2=10, launches=10):
    """The Gram of one block Gram-Schmidt pass of the W orthogonalisation at
    the solve's shape, G = [X, P]^T diag(b) W (k1 = 80 basis columns, k2 = 10
    W columns, a diagonal B): per pass the solver cuts W's digit planes (the
    diagonal folded in, k_cut_planes) and runs the plane Gram (k_gram_pp and
    its fixed-order reduction); the basis planes are cut once per GCG
    iteration for all of that iteration's Gram products.  Algorithmic bytes of
    the pass: (k1 + k2 + 1) n 8 (the FP64 operands and the diagonal, once)."""
    lib = L.load()
    g = torch.Generator(device="cuda").manual_seed(1)
    V = [torch.randn(n, dtype=torch.float64, device="cuda", generator=g) for _ in range(k1)]
    W = [torch.randn(n, dtype=torch.float64, device="cuda", generator=g) for _ in range(k2)]
    d = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) + 0.5
    vp = (C.c_void_p * k1)(*[C.c_void_p(t.data_ptr()) for t in V])
    wp = (C.c_void_p * k2)(*[C.c_void_p(t.data_ptr()) for t in W])
    vpl = torch.empty(int(lib.GCGE_CUDA_PlanesBytes(n, k1)), dtype=torch.uint8, device="cuda")
    wpl = torch.empty(int(lib.GCGE_CUDA_PlanesBytes(n, k2)), dtype=torch.uint8, device="cuda")
    part = torch.empty(int(lib.GCGE_CUDA_PlanesGramScratchDoubles(k1, k2)), dtype=torch.float64,
                       device="cuda")
    G = torch.empty(k2, k1, dtype=torch.float64, device="cuda")
    st = torch.cuda.Stream()
    sp = C.c_void_p(st.cuda_stream)

    def cut_v():
        L.check(lib.GCGE_CUDA_PlanesCut(vp, k1, n, None, C.c_void_p(vpl.data_ptr()), k1, 0, sp),
                "PlanesCut V")

    def one_pass():
        L.check(lib.GCGE_CUDA_PlanesCut(wp, k2, n, C.c_void_p(d.data_ptr()),
                                        C.c_void_p(wpl.data_ptr()), k2, 0, sp), "PlanesCut W")
        L.check(lib.GCGE_CUDA_PlanesGram(C.c_void_p(vpl.data_ptr()), k1, 0, k1,
                                         C.c_void_p(wpl.data_ptr()), k2, 0, k2, n,
                                         C.c_void_p(G.data_ptr()), k1, C.c_void_p(part.data_ptr()),
                                         sp), "PlanesGram")

    def timed(f, reps):
        for _ in range(2):
            f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            f()
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    t_cut_v = timed(cut_v, launches)
    t_pass = timed(one_pass, launches)
    ref = torch.stack(V) @ (torch.stack(W) * d[None, :]).T
    err = float(((G.T - ref).abs().max() / ref.abs().max()).item())
    assert err < 1e-13, err
    nbytes = (k1 + k2 + 1) * n * 8
    cut_bytes = k1 * n * 8 + int(lib.GCGE_CUDA_PlanesBytes(n, k1))
    return {"t_pass": t_pass, "bytes": nbytes, "t_cut_basis": t_cut_v, "cut_bytes": cut_bytes,
            "max_rel_err_vs_fp64_matmul": err}


def e2e_solves(torch, S, L, A, B, nev, x0, precision, warmup, steps):
    """Through the public C ABI with pinned HOST buffers: MatCreate (H2D of
    the CSR arrays), Solve reading the host initial block and writing host
    eigenvectors, eigenvalues back on the host."""
    lib = L.load()

    def pinned(a):
        t = torch.empty(a.shape, dtype={np.dtype("float64"): torch.float64,
                                        np.dtype("int32"): torch.int32}[a.dtype], pin_memory=True)
        t.numpy()[...] = a
        return t

    ha = [pinned(A.rowptr), pinned(A.col), pinned(A.val)]
    hb = [pinned(B.rowptr), pinned(B.col), pinned(B.val)]
    hx = pinned(np.ascontiguousarray(x0.reshape(nev, A.n)))
    hv = pinned(np.zeros((nev, A.n)))
    hev = np.zeros(nev)
    h2d = sum(t.numel() * t.element_size() for t in ha + hb) + hx.numel() * 8
    d2h = hv.numel() * 8 + nev * 8
    times = []
    for it in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ma, mb, s = C.c_void_p(), C.c_void_p(), C.c_void_p()
        L.check(lib.GCGE_CUDA_MatCreate(C.byref(ma), A.n, C.c_void_p(ha[0].data_ptr()),
                                        C.c_void_p(ha[1].data_ptr()), C.c_void_p(ha[2].data_ptr()), 0), "MatCreate A")
        L.check(lib.GCGE_CUDA_MatCreate(C.byref(mb), B.n, C.c_void_p(hb[0].data_ptr()),
                                        C.c_void_p(hb[1].data_ptr()), C.c_void_p(hb[2].data_ptr()), 0), "MatCreate B")
        L.check(lib.GCGE_CUDA_SOLVER_Create(C.byref(s)), "Create")
        lib.GCGE_CUDA_SOLVER_SetMatA(s, ma)
        lib.GCGE_CUDA_SOLVER_SetMatB(s, mb)
        lib.GCGE_CUDA_SOLVER_SetNumEigen(s, nev)
        lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"num_init_evec", nev)
        lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"ev_max_it", 1000)
        lib.GCGE_CUDA_SOLVER_SetParamDouble(s, b"ev_tol", 1e-10)
        lib.GCGE_CUDA_SOLVER_SetParamInt(s, b"precision", 1 if precision == "mixed" else 0)
        lib.GCGE_CUDA_SOLVER_SetEigenvalues(s, C.c_void_p(hev.ctypes.data))
        # the initial block is read from the result array (num_init_evec = nev)
        hv.copy_(hx)
        lib.GCGE_CUDA_SOLVER_SetEigenvectors(s, C.c_void_p(hv.data_ptr()))
        L.check(lib.GCGE_CUDA_SOLVER_Setup(s), "Setup")
        L.check(lib.GCGE_CUDA_SOLVER_Solve(s), "Solve")
        lib.GCGE_CUDA_SOLVER_Free(C.byref(s))
        lib.GCGE_CUDA_MatDestroy(C.byref(ma))
        lib.GCGE_CUDA_MatDestroy(C.byref(mb))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        if it >= warmup:
            times.append(t1 - t0)
    return times, h2d, d2h, hev.copy(), hv.numpy().copy()


def true_residuals_gpu(torch, A, B, ev, evec_rows):
    """FP64 post-check ||A x - lambda B x|| / (|lambda| ||x||) per pair (torch
    sparse on the GPU; checking only, outside the timed region)."""
    a = torch.sparse_csr_tensor(torch.from_numpy(A.rowptr.astype(np.int64)),
                                torch.from_numpy(A.col.astype(np.int64)),
                                torch.from_numpy(A.val), size=(A.n, A.n)).to("cuda")
    X = evec_rows.T.contiguous()  # n x nev
    AX = a @ X
    lam = torch.from_numpy(ev).to("cuda")
    if B.nnz == B.n and np.array_equal(B.col, np.arange(B.n)):
        BX = torch.from_numpy(B.val).to("cuda")[:, None] * X
    else:
        b = torch.sparse_csr_tensor(torch.from_numpy(B.rowptr.astype(np.int64)),
                                    torch.from_numpy(B.col.astype(np.int64)),
                                    torch.from_numpy(B.val), size=(B.n, B.n)).to("cuda")
        BX = b @ X
        del b
    del a
    R = AX - lam[None, :] * BX
    return (R.norm(dim=0) / (lam.abs() * X.norm(dim=0))).cpu().numpy()


GRAM_TRAFFIC_FILE = os.path.join(HERE, "profiles", "gram_traffic.json")
CFG3_PORT_FILE = os.path.join(HERE, "tests", "golden", "cfg3_port_summary.json")


def gram_traffic(n):
    """DRAM bytes per W-orthogonalisation Gram pass from the committed ncu
    capture (a smaller grid, scaled by the rows processed: the traffic of both
    kernels grows in proportion), or None."""
    if not os.path.exists(GRAM_TRAFFIC_FILE):
        return None
    d = json.load(open(GRAM_TRAFFIC_FILE))
    return d["bytes_per_pass"] * n / d["n"]


def reference_iters():
    if os.path.exists(REF_ITERS_FILE):
        return int(json.load(open(REF_ITERS_FILE))["iters"]), "reference run (tests/golden)"
    return None, None


CPU_FULL_RUN_FILE = os.path.join(HERE, "profiles", "cpu_port_full_solve_lap3d128.json")


def cpu_calibration():
    """The committed full (not sampled) solve of the oracle port on this
    workload, for the extrapolation error of the bounded sample."""
    if os.path.exists(CPU_FULL_RUN_FILE):
        return json.load(open(CPU_FULL_RUN_FILE))
    return None


def calibrated(est, full_size=True):
    """The sampled CPU estimate corrected by the committed full solve of the
    same workload on the same kind of host (the first iterations, which the
    sample times, cost more than the average one): value = est * full /
    sampled-at-calibration.  Returns (value, calibration record or None)."""
    cal = cpu_calibration() if full_size else None
    if not cal or not cal.get("sampled_estimate_s"):
        return est, None
    f = cal["full_solve_s"] / cal["sampled_estimate_s"]
    return est * f, {"full_solve_s": cal["full_solve_s"], "iters": cal["iters"],
                     "sampled_estimate_s_at_calibration": cal["sampled_estimate_s"],
                     "factor": f, "uncalibrated_estimate_s": est, "host": cal["host"],
                     "file": "profiles/cpu_port_full_solve_lap3d128.json"}


def cpu_sample(A, B, nev, x0, threads, fallback_iters, full_size=True,
               fallback_src="GPU FP64 iteration count", loop_iters=3):
    """Oracle port on the host: the start phase plus loop_iters GCG iterations
    (their mean cost per iteration), extrapolated to the full iteration count
    (the reference's own count on the full-size workload, else fallback_iters)."""
    from oracle import oracle as O
    p = O.default_para(nev, ev_tol=1e-10, ev_max_it=1000)
    r = O.port_solve(A, B, nev, x0, p, max_outer=loop_iters, threads=threads)
    iters, src = reference_iters() if full_size else (None, None)
    if iters is None:
        iters, src = fallback_iters, fallback_src
    t_iter = r["t_loop"] / max(1, r["loop_iters"])
    est = r["t_init"] + max(0, iters - 2) * t_iter
    sample = ("oracle port, %d threads: start phase (X orth, RR, [X,W] step) %.2f s + %d GCG "
              "iterations %.2f s each, extrapolated to %d iterations (%s)"
              % (threads, r["t_init"], r["loop_iters"], t_iter, iters, src))
    return est, r["t_init"] + r["t_loop"], sample


def cpu_full_run(args):
    """--calibrate-cpu: one complete oracle-port solve of the workload on all
    host threads, written to profiles/ as the calibration of the sampled CPU
    baseline (a few minutes on 16 cores)."""
    import platform
    from oracle import oracle as O
    A, B, nev, x0, m = workload(args.small)
    threads = os.cpu_count() or 1
    p = O.default_para(nev, ev_tol=1e-10, ev_max_it=1000)
    r = O.port_solve(A, B, nev, x0, p, threads=threads)
    est, _, sample = cpu_sample(A, B, nev, x0, threads, r["iters"], full_size=not args.small)
    out = {"workload": "laplace3d_7pt_%d^3_diagmass_nev50_tol1e-10" % m,
           "host": "%d threads, %s" % (threads, platform.machine()),
           "full_solve_s": r["seconds"], "iters": r["iters"],
           "sampled_estimate_s": est, "sample": sample,
           "extrapolation_error": est / r["seconds"] - 1.0,
           "command": "python bench.py --calibrate-cpu"}
    if not args.small:
        json.dump(out, open(CPU_FULL_RUN_FILE, "w"), indent=1)
    print(json.dumps(out))
    return 0


def workload_config(A, nev, m):
    return {"workload": "laplace3d_7pt_%d^3_diagmass_nev50_tol1e-10" % m, "n": A.n,
            "nnz": A.nnz, "nev": nev, "block_size": 10, "parallelism": "replicas only",
            "l2": "inputs larger than L2 (A 175 MB, basis 1.5 GB)"}


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    A, B, nev, x0, m = workload(args.small)
    threads = os.cpu_count() or 1
    vals = []
    wall = []
    sample = ""
    for it in range(args.warmup + args.steps):
        est, w, sample = cpu_sample(A, B, nev, x0, threads, 60, full_size=not args.small,
                                    fallback_src="an assumed 60 iterations")
        if it >= args.warmup:
            vals.append(est)
            wall.append(w)
    v, cal = calibrated(statistics.mean(vals), full_size=not args.small)
    out = {"metric": METRIC, "value": v, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(wall),
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded generator)",
           "config": workload_config(A, nev, m),
           "cpu_baseline": {"value": v, "unit": "s", "cores": threads, "kind": "port",
                            "sample": sample + ("; corrected by the full-solve calibration"
                                                if cal else ""), "calibration": cal},
           "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def run_config3(args):
    import torch
    import __graft_entry__ as g
    g.build()
    from gcge_old_gb300 import lib as L
    from gcge_old_gb300 import matrices as M
    from gcge_old_gb300 import solver as S
    m, nev = 160, 100
    t0 = time.time()
    A, B = M.diffusion27(m, seed=0)
    x0 = M.initial_block(A.n, nev, seed=0)
    gen_s = time.time() - t0
    dA, dB = S.DeviceMatrix(A), S.DeviceMatrix(B)
    x0_dev = torch.from_numpy(x0).to("cuda")
    res = {}
    evs = {}
    for prec in ("mixed", "fp64"):
        t, st, ev, vec = time_solves(torch, S, L, dA, dB, nev, x0_dev, prec, 0, 1,
                                     ev_tol=args.c3tol)
        r = true_residuals_gpu(torch, A, B, ev, vec)
        res[prec] = {"s": t[0], "gcg_iterations": st[0]["num_iter"], "bcg_steps": st[0]["bcg_steps"],
                     "max_residual": float(r.max()),
                     "phase_s": {k: round(v, 3) for k, v in st[0].items() if k.startswith("t_")}}
        evs[prec] = ev
        del vec
        torch.cuda.empty_cache()
    # the mixed solve with the W step by AMG-PCG (GCGE_CUDA_AMGPCG) instead of
    # the built-in block CG: hierarchy set-up timed separately
    if args.c3amg:
        torch.cuda.synchronize()
        t0 = time.time()
        amg = S.AMG(dA)
        torch.cuda.synchronize()
        t_setup = time.time() - t0
        levels = [amg.level_info(l)["n"] for l in range(amg.num_levels)]
        t, st, ev, vec = time_solves(torch, S, L, dA, dB, nev, x0_dev, "mixed", 0, 1,
                                     ev_tol=args.c3amgtol, mls=amg)
        r = true_residuals_gpu(torch, A, B, ev, vec)
        res["mixed_amg"] = {"s": t[0], "ev_tol": args.c3amgtol, "amg_setup_s": t_setup,
                            "levels": levels,
                            "gcg_iterations": st[0]["num_iter"], "max_residual": float(r.max()),
                            "phase_s": {k: round(v, 3) for k, v in st[0].items()
                                        if k.startswith("t_")}}
        evs["mixed_amg"] = ev
        del vec
        if args.c3pase:
            # the multilevel eigensolver on the same hierarchy (GCGE_CUDA_PASE_Solve)
            out_t = torch.empty((nev, A.n), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            t0 = time.time()
            ev, _, pst = S.pase_solve(dA, dB, nev, amg=amg, evec_device=out_t, tol=args.c3pasetol,
                                      max_cycles=120)
            torch.cuda.synchronize()
            t_p = time.time() - t0
            r = true_residuals_gpu(torch, A, B, ev, out_t)
            res["pase"] = {"s": t_p, "tol": args.c3pasetol, "cycles": pst["cycles"],
                           "max_residual": float(r.max()),
                           "phase_s": {k: round(v, 3) for k, v in pst.items() if k.startswith("t_")}}
            evs["pase"] = ev
            del out_t
        amg.close()
        torch.cuda.empty_cache()
    ev_m, ev_d = evs["mixed"], evs["fp64"]
    rel = np.abs(ev_m - ev_d) / np.abs(ev_d)
    out = {"metric": METRIC, "config": {"workload": "diffusion27_q1_lognormal_%d^3_consistent_mass_"
                                                    "nev100" % m, "ev_tol": args.c3tol,
                                        "n": A.n, "nnz_A": A.nnz, "nnz_B": B.nnz, "nev": nev},
           "unit": "s", **res,
           "mixed_speedup_vs_fp64": res["fp64"]["s"] / res["mixed"]["s"],
           "per_pair_eigenvalue_rel_diff_mixed_vs_fp64": {"max": float(rel.max()),
                                                          "median": float(np.median(rel))},
           "generator_s": gen_s, "data": "synthetic (seeded generator)"}
    # per pair against the oracle port's solve of the same matrices and start
    if os.path.exists(CFG3_PORT_FILE):
        ref = np.array(json.load(open(CFG3_PORT_FILE))["eval"])
        out["per_pair_eigenvalue_rel_diff_vs_oracle_port"] = {
            p: float(np.max(np.abs(evs[p] - ref) / np.abs(ref))) for p in evs}
    for key in ("mixed_amg", "pase"):
        if key in evs:
            out["per_pair_eigenvalue_rel_diff_%s_vs_fp64" % key] = float(
                np.max(np.abs(evs[key] - ev_d) / np.abs(ev_d)))
    if args.c3save:
        np.savez(args.c3save, ev_tol=args.c3tol, **evs)
    print(json.dumps(out))
    return 0


def _config4_grad(torch, M, m, nev, seed, ev_tol, adjoint_amg=None):
    """Forward + backward of the config-4 loss; returns the problem, tensors and times.
    adjoint_amg: the eigenvector adjoint's CG preconditioner (None: diag(A))."""
    from gcge_old_gb300.autograd import eigpairs_csr
    A, B, Smap, kappa = M.aniso2d(m, seed=seed)
    rng = np.random.default_rng(seed + 1)
    w = rng.uniform(0.0, 1.0, nev)
    mask = (rng.uniform(size=A.n) < 0.5).astype(np.float64)
    x0 = M.initial_block(A.n, nev, seed=seed)
    S = Smap.tocoo()
    St = torch.sparse_coo_tensor(np.vstack([S.row, S.col]), S.data, S.shape)
    kap = torch.tensor(kappa, requires_grad=True)
    b = torch.tensor(B.val, requires_grad=True)
    params = dict(ev_tol=ev_tol, ev_max_it=5000, precision="fp64")
    torch.cuda.synchronize()
    t0 = time.time()
    a = torch.sparse.mm(St, kap[:, None])[:, 0]
    a.retain_grad()
    lam, X = eigpairs_csr(a, A, nev, x0, b_val=b, B_pattern=B, adjoint_amg=adjoint_amg, **params)
    t1 = time.time()
    wt, mt = torch.from_numpy(w), torch.from_numpy(mask)
    loss_ev = (wt * lam).sum()
    loss = loss_ev + ((X[0] * mt) ** 2).sum()
    loss.backward(retain_graph=True)
    torch.cuda.synchronize()
    t2 = time.time()
    ga = a.grad.numpy().copy()
    ga_ev, gb_ev = torch.autograd.grad(loss_ev, [a, b])

    def f(av, bv, seed_x0=seed):
        """(eigenvalue part, full loss) from one solve with A values av, B values bv."""
        with torch.no_grad():
            l, Y = eigpairs_csr(torch.from_numpy(av), A, nev,
                                M.initial_block(A.n, nev, seed=seed_x0),
                                b_val=torch.from_numpy(bv), B_pattern=B, **params)
        le = float((w * l.numpy()).sum())
        return le, le + float(((Y[0].numpy() * mask) ** 2).sum())

    from gcge_old_gb300.autograd import last_adjoint
    adj = dict(last_adjoint)
    return dict(A=A, B=B, S=Smap, kappa=kappa, w=w, mask=mask, lam=lam.detach().numpy(), adj=adj,
                X=X.detach().numpy(), ga=ga, gb=b.grad.numpy(), gk=kap.grad.numpy(),
                ga_ev=ga_ev.numpy(), gb_ev=gb_ev.numpy(), f=f, t_fwd=t1 - t0, t_bwd=t2 - t1)


def run_config4(args):
    import torch
    import __graft_entry__ as g
    g.build()
    import scipy.linalg as sla
    from gcge_old_gb300 import matrices as M
    nev = 32
    r = _config4_grad(torch, M, 512, nev, 0, 1e-12)
    # the same forward + backward with the adjoint's CG preconditioned by an AMG
    # V-cycle of A (hierarchy set-up inside the backward time)
    ra = _config4_grad(torch, M, 512, nev, 0, 1e-12, adjoint_amg=True)
    amg_arm = {"cg_steps": ra["adj"]["steps"], "backward_s": ra["t_bwd"],
               "forward_s": ra["t_fwd"],
               "gradA_rel_diff_vs_jacobi": float(np.abs(ra["ga"] - r["ga"]).max()
                                                 / np.abs(r["ga"]).max()),
               "gradB_rel_diff_vs_jacobi": float(np.abs(ra["gb"] - r["gb"]).max()
                                                 / np.abs(r["gb"]).max())}
    kappa, Bv, Av, Smap = r["kappa"], r["B"].val, r["A"].val, r["S"]
    rng = np.random.default_rng(3)
    # the same solve from another initial block: the spread of the two losses is
    # the noise floor of a finite difference (FP64 rounding of the Rayleigh
    # quotients for the eigenvalue part; the eigenvector term carries
    # ||x_1||^2 ~ 1/h^2 times an eigenvector error bounded by the residual floor)
    l0, l1 = r["f"](Av, Bv), r["f"](Av, Bv, seed_x0=7)
    noise = {"eigenvalue_loss": abs(l0[0] - l1[0]), "full_loss": abs(l0[1] - l1[1])}
    # directional derivatives along seeded random directions: kappa (through
    # A = S kappa), A's values (symmetric perturbation of the stored pattern), B's values
    Asp = r["A"].to_scipy()
    R = Asp.copy()
    R.data = rng.standard_normal(R.nnz)
    R = (R + R.T).tocsr()
    R.sort_indices()
    assert R.nnz == len(Av) and (R.indptr == Asp.indptr).all() and (R.indices == Asp.indices).all()
    dA = R.data * np.abs(Av)
    # edge-wise direction: random relative change of each off-diagonal pair with
    # the diagonal moved so that row sums stay as they are (a conductance change)
    coo = Asp.tocoo()
    off = coo.row != coo.col
    E = Asp.copy()
    E.data = np.where(off, R.data * np.abs(Av), 0.0)
    dE = E.data - np.where(~off, np.asarray(E.sum(axis=1)).ravel()[coo.row], 0.0)
    dk = rng.standard_normal(len(kappa)) * kappa
    dB = rng.standard_normal(len(Bv)) * Bv
    dirs = [("kappa", Smap @ dk, np.zeros_like(Bv), float(r["gk"] @ dk),
             float(r["ga_ev"] @ (Smap @ dk))),
            ("A_values", dA, np.zeros_like(Bv), float(r["ga"] @ dA), float(r["ga_ev"] @ dA)),
            ("A_edges", dE, np.zeros_like(Bv), float(r["ga"] @ dE), float(r["ga_ev"] @ dE)),
            ("B_values", np.zeros_like(Av), dB, float(r["gb"] @ dB), float(r["gb_ev"] @ dB))]
    checks = {"eigenvalue_loss": [], "full_loss": []}
    for name, da, db, adj_full, adj_ev in dirs:
        for eps in ((1e-6, 1e-5, 1e-4) if name.startswith("A_") else (1e-4, 1e-3)):
            fp, fm = r["f"](Av + eps * da, Bv + eps * db), r["f"](Av - eps * da, Bv - eps * db)
            for i, key, adj in ((0, "eigenvalue_loss", adj_ev), (1, "full_loss", adj_full)):
                v = (fp[i] - fm[i]) / (2 * eps)
                checks[key].append({"direction": name, "eps": eps, "fd": v, "adjoint": adj,
                                    "rel": abs(v - adj) / abs(adj)})
    # 64 x 64 copy against dense generalized-eigendecomposition adjoints
    s = _config4_grad(torch, M, 64, nev, 0, 1e-12)
    A, B = s["A"], s["B"]
    ev, V = sla.eigh(A.to_scipy().toarray(), B.to_scipy().toarray())
    V = V.T.copy()
    idx = np.abs(V[:nev]).argmax(axis=1)
    V[:nev] *= np.sign(V[np.arange(nev), idx])[:, None]
    g0 = 2 * s["mask"] ** 2 * V[0]
    d = ev - ev[0]
    d[0] = np.inf
    mu0 = ((V @ g0) / d) @ V
    Asp, Bsp = A.to_scipy().tocoo(), B.to_scipy().tocoo()
    w = s["w"]
    gA = sum(w[k] * V[k][Asp.row] * V[k][Asp.col] for k in range(nev)) - mu0[Asp.row] * V[0][Asp.col]
    gB = (sum(-w[k] * ev[k] * V[k][Bsp.row] * V[k][Bsp.col] for k in range(nev))
          + ev[0] * mu0[Bsp.row] * V[0][Bsp.col] - 0.5 * (g0 @ V[0]) * V[0][Bsp.row] * V[0][Bsp.col])
    dense = {"n": A.n, "eigenvalue_rel_max": float(np.max(np.abs(s["lam"] - ev[:nev]) / ev[:nev])),
             "gradA_rel_max": float(np.abs(s["ga"] - gA).max() / np.abs(gA).max()),
             "gradB_rel_max": float(np.abs(s["gb"] - gB).max() / np.abs(gB).max()),
             "gradKappa_rel_max": float(np.abs(s["gk"] - s["S"].T @ gA).max()
                                        / np.abs(s["S"].T @ gA).max())}
    out = {"metric": "eigenvalue + eigenvector loss gradient (adjoint) vs finite differences",
           "config": {"workload": "aniso2d_5pt_512x512_kappa_U(0.5,2)_ratio10_diag_mass_nev32",
                      "n": int(r["A"].n), "nnz_A": int(r["A"].nnz), "nev": nev,
                      "loss": "sum w_k lambda_k + ||x_1 * mask||^2"},
           "forward_s": r["t_fwd"], "backward_s": r["t_bwd"],
           "eigenvector_adjoint": {"columns": r["adj"]["columns"], "cg_steps": r["adj"]["steps"],
                                   "tol": 1e-10, "preconditioner": "jacobi"},
           "eigenvector_adjoint_amg": amg_arm,
           "fd_checks": checks,
           "fd_rel_best_eigenvalue_loss": {d: min(c["rel"] for c in checks["eigenvalue_loss"]
                                                  if c["direction"] == d)
                                           for d in ("kappa", "A_values", "A_edges", "B_values")},
           "fd_rel_best_full_loss": {d: min(c["rel"] for c in checks["full_loss"]
                                            if c["direction"] == d)
                                     for d in ("kappa", "A_values", "A_edges", "B_values")},
           "fd_noise_floor": noise,
           "dense_64x64": dense, "data": "synthetic (seeded generator)"}
    print(json.dumps(out))
    return 0


def run_config5(args):
    import torch
    import __graft_entry__ as g
    g.build()
    from gcge_old_gb300 import matrices as M
    from gcge_old_gb300 import solver as S
    n, nev = args.c5n, 128
    t0 = time.time()
    A, B, (ei, ej, ew, pos) = M.chung_lu(n, seed=0)
    gen_s = time.time() - t0
    rows = np.diff(A.rowptr)
    x0 = M.initial_block(n, nev, seed=0)
    params = dict(ev_tol=1e-10, ev_max_it=args.c5it, precision="mixed")
    s = S.GCGESolver(A, B, nev, **params)
    try:
        ev, vec = s.solve(x0)
        st = s.stats()
    finally:
        s.close()
    vec_d = torch.from_numpy(vec).to("cuda")
    tr = true_residuals_gpu(torch, A, B, ev, vec_d)
    del vec_d
    torch.cuda.empty_cache()
    crit = tr * np.abs(ev) / np.maximum(1.0, np.abs(ev))
    nconv = int(np.argmax(crit >= 1e-10)) if (crit >= 1e-10).any() else nev
    # gradient of sum_k w_k lambda_k (all nev pairs) with respect to the edge
    # weights from this solve's vectors: the adjoint kernel on A's and B's patterns
    from gcge_old_gb300.autograd import _adjoint
    wl = np.random.default_rng(1).uniform(0.0, 1.0, nev)
    torch.cuda.synchronize()
    t1 = time.time()
    ga = _adjoint(A, vec, wl).cpu().numpy()
    gb = _adjoint(B, vec, -wl * ev).cpu().numpy()
    torch.cuda.synchronize()
    t2 = time.time()
    p_ij, p_ji, p_ii, p_jj, bi, bj = pos
    gw = -ga[p_ij] - ga[p_ji] + ga[p_ii] + ga[p_jj] + gb[bi] + gb[bj]
    # the same from the closed form (x_i - x_j)^2 - lambda (x_i^2 + x_j^2) per edge
    sample = np.random.default_rng(3).choice(len(ew), 10000, replace=False)
    xi, xj = vec[:, ei[sample]], vec[:, ej[sample]]
    closed = (wl[:, None] * ((xi - xj) ** 2 - ev[:, None] * (xi ** 2 + xj ** 2))).sum(axis=0)
    grad_check = float(np.abs(gw[sample] - closed).max() / np.abs(closed).max())
    del vec
    out = {"metric": "s per GCG iteration and pairs converged @1e-10 (uneven rows, mixed) "
                     "+ edge-weight gradient",
           "config": {"workload": "chung_lu_n%d_deg16_gamma2.5_shift1e-3_B=D_nev%d" % (n, nev),
                      "n": n, "nnz_A": int(A.nnz), "max_row": int(rows.max()),
                      "rows_over_64": int((rows > 64).sum()),
                      "entries_in_rows_over_64": float(rows[rows > 64].sum() / A.nnz),
                      "ev_max_it": args.c5it},
           "solve_s": st["seconds"], "gcg_iterations": st["num_iter"],
           "s_per_iteration": st["seconds"] / max(1, st["num_iter"]),
           "bcg_steps": st["bcg_steps"],
           "phase_s": {k: round(v, 3) for k, v in st.items() if k.startswith("t_")},
           "pairs_converged_leading": nconv,
           "pairs_converged_total": int((crit < 1e-10).sum()),
           "reference_criterion_max": float(crit.max()),
           "eigenvalues_first_last": [float(ev[0]), float(ev[-1])],
           "gradient": {"loss": "sum_k w_k lambda_k", "adjoint_s": t2 - t1,
                        "max_rel_diff_vs_closed_form_10k_edges": grad_check},
           "generator_s": gen_s, "data": "synthetic (seeded generator)"}
    print(json.dumps(out))
    return 0


def max_over_ranks(values, device):
    """Element-wise maximum of per-rank values over the process group (the
    replicas' times: the job takes as long as its slowest replica)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="48^3 grid (quick check)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--calibrate-cpu", action="store_true",
                    help="run one full oracle-port solve and record it in profiles/")
    ap.add_argument("--c5n", type=int, default=8_000_000, help="graph size of --config 5")
    ap.add_argument("--c5it", type=int, default=100, help="GCG iteration cap of --config 5")
    ap.add_argument("--c3tol", type=float, default=1e-11, help="ev_tol of --config 3")
    ap.add_argument("--c3amg", action="store_true", help="--config 3: also solve with the AMG-PCG "
                                                         "W step")
    ap.add_argument("--c3pase", action="store_true", help="--config 3 (with --c3amg): also solve "
                                                          "with the multilevel eigensolver")
    ap.add_argument("--c3amgtol", type=float, default=3e-12,
                    help="ev_tol of --config 3's AMG-PCG solve (other iterates than the "
                         "reference's: a tighter bound keeps every eigenvalue within 1e-10)")
    ap.add_argument("--c3pasetol", type=float, default=1e-11,
                    help="residual tolerance of --config 3's multilevel solve")
    ap.add_argument("--c3save", default="", help="--config 3: write both precisions' eigenvalues "
                                                "to this .npz")
    ap.add_argument("--config", type=int, default=2, choices=[2, 3, 4, 5],
                    help="3: the 160^3 27-point mixed-precision configuration (one solve each); "
                         "4: the 512^2 differentiation configuration (gradient checks)")
    args = ap.parse_args()
    if args.calibrate_cpu:
        return cpu_full_run(args)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.config == 3:
        return run_config3(args)
    if args.config == 4:
        return run_config4(args)
    if args.config == 5:
        return run_config5(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as g
    if rank == 0:
        g.build()
    if world > 1:
        dist.barrier()
    from gcge_old_gb300 import lib as L
    from gcge_old_gb300 import solver as S
    L.load()

    A, B, nev, x0, m = workload(args.small)
    dA, dB = S.DeviceMatrix(A), S.DeviceMatrix(B)
    x0_dev = torch.from_numpy(np.ascontiguousarray(x0)).to("cuda")

    sampler = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    t_mixed, st_mixed, ev_mixed, vec_mixed = time_solves(torch, S, L, dA, dB, nev, x0_dev, "mixed",
                                                         args.warmup, args.steps)
    t_fp64, st_fp64, ev_fp64, vec_fp64 = time_solves(torch, S, L, dA, dB, nev, x0_dev, "fp64",
                                                     max(1, args.warmup // 3), max(1, args.steps // 2))
    # the FP64 solve with the mixed form's W step (the correction e alone as the
    # W block): mixed vs this is the ratio that only the precision changes
    t_fcor, st_fcor, _, vec_fcor = time_solves(torch, S, L, dA, dB, nev, x0_dev, "fp64", 0, 1,
                                               w_form="correction")
    del vec_fcor
    # the same FP64 solve with the tall-skinny products on FP64 FMA units instead of
    # the FP64-accurate tensor-core products (one solve: what the tensor cores buy)
    t_fma, st_fma, _, vec_fma = time_solves(torch, S, L, dA, dB, nev, x0_dev, "fp64", 0, 1,
                                            gemm="fp64")
    del vec_fma
    # the mixed solve with the W step by AMG-PCG (hierarchy set-up timed apart)
    torch.cuda.synchronize()
    t0 = time.time()
    amg = S.AMG(dA)
    torch.cuda.synchronize()
    amg_setup = time.time() - t0
    amg_levels = [amg.level_info(l)["n"] for l in range(amg.num_levels)]
    t_amg, st_amg, ev_amg, vec_amg = time_solves(torch, S, L, dA, dB, nev, x0_dev, "mixed", 1, 2,
                                                 mls=amg)
    res_amg = true_residuals_gpu(torch, A, B, ev_amg, vec_amg)
    del vec_amg
    # the multilevel eigensolver (GCGE_CUDA_PASE_Solve) on the same hierarchy
    out_p = torch.empty((nev, A.n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.time()
    ev_pase, _, pst = S.pase_solve(dA, dB, nev, amg=amg, evec_device=out_p, tol=1e-10)
    torch.cuda.synchronize()
    t_pase = time.time() - t0
    res_pase = true_residuals_gpu(torch, A, B, ev_pase, out_p)
    del out_p
    amg.close()
    # each form with the block size and inner block-CG step cap that suit it
    # (found by a sweep; the reference's defaults are 10 and 20): more inner
    # steps buy fewer outer iterations, and the FP32 ones are cheap
    tuned = {}
    for prec, bs, cap in (("mixed", 12, 40), ("fp64", 15, 40)):
        tt, stt, _, vt = time_solves(torch, S, L, dA, dB, nev, x0_dev, prec, 0, 1, cg_max_it=cap,
                                     block_size=bs)
        tuned[prec] = {"s": tt[0], "block_size": bs, "cg_max_it": cap,
                       "gcg_iterations": stt[0]["num_iter"], "bcg_steps": stt[0]["bcg_steps"]}
        del vt
    torch.cuda.synchronize()
    clocks = sampler.stop()
    v_mixed = statistics.mean(t_mixed)
    v_fp64 = statistics.mean(t_fp64)
    if world > 1:
        v_mixed, v_fp64 = max_over_ranks([v_mixed, v_fp64], "cuda")

    # correctness of the timed solves (outside the timed region)
    res_m = true_residuals_gpu(torch, A, B, ev_mixed, vec_mixed)
    res_d = true_residuals_gpu(torch, A, B, ev_fp64, vec_fp64)
    ev_rel = float(np.max(np.abs(ev_mixed - ev_fp64) / np.abs(ev_fp64)))

    t_spmm, b_spmm, t_spmm32, b_spmm32, t_rows = spmm_roofline(torch, L, dA, A, 10)
    peak, peak_src = peaks()
    # algorithmic bytes of the k = 10 FP32 SpMM: A once, x and y once each
    # (the 2 padding floats of a 12-float row count as waste, not as work)
    ach = b_spmm32 / t_rows / 1e9
    gr = gram_roofline(torch, L, A.n)
    ach_g = gr["bytes"] / gr["t_pass"] / 1e9

    e2e_t, h2d, d2h, _, _ = e2e_solves(torch, S, L, A, B, nev, x0, "mixed", 1, max(1, args.steps // 2))
    e2e_v = statistics.mean(e2e_t)
    if world > 1:
        e2e_v = max_over_ranks([e2e_v], "cuda")[0]

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        est, wall, sample = cpu_sample(A, B, nev, x0, threads, st_fp64[-1]["num_iter"],
                                       full_size=not args.small)
        est, cal = calibrated(est, full_size=not args.small)
        cpu = {"value": est, "unit": "s", "cores": threads, "kind": "port",
               "sample": sample + ("; corrected by the full-solve calibration" if cal else ""),
               "calibration": cal}

    traffic = None
    tf = os.path.join(HERE, "profiles", "spmm_traffic.json")
    if os.path.exists(tf) and not args.small:
        traffic = json.load(open(tf)).get("bytes_per_launch")

    launches = int(statistics.mean([s["kernel_launches"] for s in st_mixed]))
    out = {
        "metric": METRIC, "value": v_mixed, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * v_mixed, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic (seeded generator)",
        "config": workload_config(A, nev, m),
        "fp64_s": v_fp64, "mixed_s": v_mixed, "mixed_speedup_vs_fp64": v_fp64 / v_mixed,
        "fp64_correction_form_s": t_fcor[0],
        "mixed_speedup_vs_fp64_same_w_form": t_fcor[0] / v_mixed,
        "mixed_speedup_vs_best_fp64": min(v_fp64, t_fcor[0]) / v_mixed,
        "fp64_fma_products_s": t_fma[0],
        "mixed_amg_pcg": {"s": statistics.mean(t_amg), "setup_s": amg_setup, "levels": amg_levels,
                          "gcg_iterations": st_amg[-1]["num_iter"],
                          "max_residual": float(res_amg.max()),
                          "eigenvalue_rel_diff_vs_fp64": float(np.max(np.abs(ev_amg - ev_fp64)
                                                                      / np.abs(ev_fp64))),
                          "speedup_vs_mixed": v_mixed / statistics.mean(t_amg)},
        "pase": {"s": t_pase, "cycles": pst["cycles"], "max_residual": float(res_pase.max()),
                 "eigenvalue_rel_diff_vs_fp64": float(np.max(np.abs(ev_pase - ev_fp64)
                                                             / np.abs(ev_fp64))),
                 "phase_s": {k: round(v, 3) for k, v in pst.items() if k.startswith("t_")}},
        "tuned_inner_solve": dict(tuned, mixed_speedup_vs_fp64=tuned["fp64"]["s"] / tuned["mixed"]["s"]),
        "gcg_iterations": {"mixed": st_mixed[-1]["num_iter"], "fp64": st_fp64[-1]["num_iter"],
                           "fp64_correction_form": st_fcor[0]["num_iter"]},
        "max_residual": {"mixed": float(res_m.max()), "fp64": float(res_d.max())},
        "eigenvalue_rel_diff_mixed_vs_fp64": ev_rel,
        "phase_s_mixed": {k: round(v, 4) for k, v in st_mixed[-1].items() if k.startswith("t_")},
        "w_orth_passes": {"mixed": st_mixed[-1]["w_orth_passes"],
                          "fp64": st_fp64[-1]["w_orth_passes"]},
        "roofline": {"kernel": "W-orthogonalisation Gram pass: k_cut_planes (W with the "
                               "diagonal of B) + k_gram_pp + reduction, [X,P]^T diag(b) W, "
                               "80 x 10 columns", "bound": "hbm",
                     "achieved": ach_g, "peak": peak, "unit": "GB/s", "frac": ach_g / peak,
                     "peak_source": peak_src, "traffic": gram_traffic(A.n),
                     "algorithmic_bytes": gr["bytes"], "us_per_launch": gr["t_pass"] * 1e6,
                     "basis_plane_cut": {"us": gr["t_cut_basis"] * 1e6, "bytes": gr["cut_bytes"],
                                         "gbs": gr["cut_bytes"] / gr["t_cut_basis"] / 1e9,
                                         "per": "GCG iteration (80 columns)"},
                     "max_rel_err_vs_fp64_matmul": gr["max_rel_err_vs_fp64_matmul"]},
        "rooflines": [
            {"kernel": "k_rows_spmm<12> (FP32 CSR SpMM of the block CG, k=10, row-interleaved)",
             "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
             "traffic": traffic, "algorithmic_bytes": b_spmm32, "us_per_launch": t_rows * 1e6},
            {"kernel": "k_spmm<double> (FP64 CSR SpMM, k=10, columns)", "bound": "fp64 fma",
             "achieved": b_spmm / t_spmm / 1e9, "unit": "GB/s",
             "note": "bound by GB300's FP64 FMA rate (~1 TFLOP/s), not by HBM"},
            {"kernel": "FP32 CSR SpMM, k=10, columns", "bound": "hbm",
             "achieved": b_spmm32 / t_spmm32 / 1e9, "unit": "GB/s",
             "frac": b_spmm32 / t_spmm32 / 1e9 / peak}],
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
