"""Profiling driver: one GCG solve of the 3D 7-point Laplacian with diagonal
mass (the benchmark's generator) on an m^3 grid for a fixed number of GCG
iterations, so a profiler sees a bounded, repeatable launch sequence.

    python profile_solve.py --grid 96 --iters 6 --precision mixed

With --spmm K it only runs K-column CSR SpMMs of the same matrix (five FP64
launches, five FP32 column launches, five FP32 row-interleaved launches), for
traffic counters of those kernels:

    python profile_solve.py --grid 96 --spmm 10

--graph N solves the shifted Laplacian of an N-node Chung-Lu graph with B = D
instead (uneven rows); --aniso M --adjoint K solves the 2D anisotropic problem
on an M x M grid and then runs K steps of the eigenvector adjoint's projected
CG for the first eigenvector (a bounded launch sequence: the adjoint stops
there whether or not it converged):

    python profile_solve.py --graph 1000000 --nev 128 --iters 3
    python profile_solve.py --aniso 512 --nev 32 --adjoint 200

--gram P runs only P Gram passes of the W orthogonalisation (80 x 10 columns
on grid^3 rows, the planes of the basis cut once):

    python profile_solve.py --grid 96 --gram 3

--diff27 M solves the 27-point variable-coefficient diffusion problem on an
M^3 grid instead; --amg gives the W step to AMG-PCG on the AMG hierarchy of A
(GCGE_CUDA_AMGPCG); --pase runs the multilevel eigensolver for --iters cycles:

    python profile_solve.py --diff27 96 --nev 100 --iters 4 --amg
    python profile_solve.py --diff27 96 --nev 100 --iters 3 --pase
"""
import argparse

from gcge_old_gb300 import matrices as M
from gcge_old_gb300 import solver as S


def spmm_only(A, k):
    import ctypes as C

    import torch

    from gcge_old_gb300 import lib as L
    lib = L.load()
    dA = S.DeviceMatrix(A)
    X = [torch.randn(A.n, dtype=torch.float64, device="cuda") for _ in range(k)]
    Y = [torch.empty(A.n, dtype=torch.float64, device="cuda") for _ in range(k)]
    X32 = [t.float() for t in X]
    Y32 = [torch.empty(A.n, dtype=torch.float32, device="cuda") for _ in range(k)]
    ptrs = lambda ts: (C.c_void_p * k)(*[C.c_void_p(t.data_ptr()) for t in ts])
    xp, yp, xp32, yp32 = ptrs(X), ptrs(Y), ptrs(X32), ptrs(Y32)
    for _ in range(5):
        L.check(lib.GCGE_CUDA_MatDotMultiVecAsync(dA.handle, xp, yp, k, None), "spmm")
    for _ in range(5):
        L.check(lib.GCGE_CUDA_MatDotMultiVecF32Async(dA.handle, xp32, yp32, k, None), "spmm32")
    if k <= 16:  # the block CG's row-interleaved FP32 operator
        kw = (k + 3) // 4 * 4
        XR = torch.randn(A.n, kw, dtype=torch.float32, device="cuda")
        YR = torch.empty(A.n, kw, dtype=torch.float32, device="cuda")
        for _ in range(5):
            L.check(lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(XR.data_ptr()),
                                                     C.c_void_p(YR.data_ptr()), k, None), "rows")
    torch.cuda.synchronize()
    print("spmm n=%d nnz=%d k=%d done" % (A.n, A.nnz, k))


def gram_passes(n, passes, k1=80, k2=10):
    """The W-orthogonalisation's Gram pass at the solve's shape: the basis
    planes cut once (80 columns), then `passes` times the cut of W's planes
    (10 columns, a diagonal folded in) and the plane Gram [X,P]^T diag(b) W."""
    import ctypes as C

    import torch

    from gcge_old_gb300 import lib as L
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
    L.check(lib.GCGE_CUDA_PlanesCut(vp, k1, n, None, C.c_void_p(vpl.data_ptr()), k1, 0, None),
            "PlanesCut V")
    for _ in range(passes):
        L.check(lib.GCGE_CUDA_PlanesCut(wp, k2, n, C.c_void_p(d.data_ptr()),
                                        C.c_void_p(wpl.data_ptr()), k2, 0, None), "PlanesCut W")
        L.check(lib.GCGE_CUDA_PlanesGram(C.c_void_p(vpl.data_ptr()), k1, 0, k1,
                                         C.c_void_p(wpl.data_ptr()), k2, 0, k2, n,
                                         C.c_void_p(G.data_ptr()), k1, C.c_void_p(part.data_ptr()),
                                         None), "PlanesGram")
    torch.cuda.synchronize()
    print("gram passes n=%d k1=%d k2=%d passes=%d done" % (n, k1, k2, passes))


def adjoint_steps(A, B, nev, steps):
    import ctypes as C

    import numpy as np
    import torch

    from gcge_old_gb300 import lib as L
    lib = L.load()
    x0 = M.initial_block(A.n, nev, seed=0)
    ev, vec, _ = S.solve(A, B, nev, x0, ev_tol=1e-12, ev_max_it=2000, precision="fp64")
    X = torch.from_numpy(vec).cuda()
    G = torch.zeros_like(X)
    G[0] = torch.randn(A.n, dtype=torch.float64, device="cuda")
    MU = torch.zeros_like(X)
    cols = lambda t, on: (C.c_void_p * nev)(*[C.c_void_p(t[j].data_ptr()) if on(j) else None
                                              for j in range(nev)])
    dA, dB = S.DeviceMatrix(A), S.DeviceMatrix(B)
    it = C.c_int(0)
    rc = lib.GCGE_CUDA_EigvecAdjointSolve(dA.handle, dB.handle, cols(X, lambda j: True),
                                          ev.ctypes.data_as(L.c_double_p), nev,
                                          cols(G, lambda j: j == 0), cols(MU, lambda j: j == 0),
                                          None, steps, 1e-10, C.byref(it))
    torch.cuda.synchronize()
    print("adjoint n=%d nev=%d steps=%d rc=%d" % (A.n, nev, it.value, rc))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=96)
    ap.add_argument("--iters", type=int, default=6)
    ap.add_argument("--nev", type=int, default=50)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--gemm", default="ozaki", choices=["ozaki", "fp64"])
    ap.add_argument("--spmm", type=int, default=0, help="only K-column SpMMs")
    ap.add_argument("--graph", type=int, default=0, help="Chung-Lu graph with this many nodes")
    ap.add_argument("--aniso", type=int, default=0, help="2D anisotropic grid size")
    ap.add_argument("--adjoint", type=int, default=0, help="eigenvector-adjoint CG steps")
    ap.add_argument("--diff27", type=int, default=0, help="27-point diffusion grid size")
    ap.add_argument("--amg", action="store_true", help="W step by AMG-PCG")
    ap.add_argument("--pase", action="store_true", help="the multilevel eigensolver")
    ap.add_argument("--tol", type=float, default=1e-10, help="stopping residual of --pase")
    ap.add_argument("--gram", type=int, default=0,
                    help="only W-orthogonalisation Gram passes (80 x 10) at grid^3 rows")
    a = ap.parse_args()
    if a.gram:
        gram_passes(a.grid ** 3, a.gram)
        return
    if a.graph:
        A, B, _ = M.chung_lu(a.graph, seed=0)
    elif a.aniso:
        A, B, _, _ = M.aniso2d(a.aniso, seed=0)
    elif a.diff27:
        A, B = M.diffusion27(a.diff27, seed=0)
    else:
        A, B = M.laplace3d_mass(a.grid, seed=0)
    if a.adjoint:
        adjoint_steps(A, B, a.nev, a.adjoint)
        return
    if a.spmm:
        spmm_only(A, a.spmm)
        return
    if a.pase:
        from gcge_old_gb300 import lib as L
        try:
            ev, vec, st = S.pase_solve(A, B, a.nev, tol=a.tol, max_cycles=a.iters)
            print(st)
        except L.GcgeCudaError as e:  # the cycle cap ends the run before convergence
            print("pase stopped at the cycle cap:", e)
        return
    x0 = M.initial_block(A.n, a.nev, seed=0)
    s = S.GCGESolver(A, B, a.nev, ev_tol=1e-10, ev_max_it=a.iters, precision=a.precision,
                     gemm=a.gemm)
    if a.amg:
        s.use_amg_pcg()
    s.solve(x0)
    print(s.stats())
    s.close()


if __name__ == "__main__":
    main()
