"""Profiling driver: one GCG solve of the 3D 7-point Laplacian with diagonal
mass (the benchmark's generator) on an m^3 grid for a fixed number of GCG
iterations, so a profiler sees a bounded, repeatable launch sequence.

    python -m gcge_old_gb300.profile_solve --grid 96 --iters 6 --precision mixed

With --spmm K it only runs K-column CSR SpMMs of the same matrix (five FP64
launches, five FP32 column launches, five FP32 row-interleaved launches), for
traffic counters of those kernels:

    python -m gcge_old_gb300.profile_solve --grid 96 --spmm 10
"""
import argparse

from . import matrices as M
from . import solver as S


def spmm_only(A, k):
    import ctypes as C

    import torch

    from . import lib as L
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=96)
    ap.add_argument("--iters", type=int, default=6)
    ap.add_argument("--nev", type=int, default=50)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--gemm", default="ozaki", choices=["ozaki", "fp64"])
    ap.add_argument("--spmm", type=int, default=0, help="only K-column SpMMs")
    a = ap.parse_args()
    A, B = M.laplace3d_mass(a.grid, seed=0)
    if a.spmm:
        spmm_only(A, a.spmm)
        return
    x0 = M.initial_block(A.n, a.nev, seed=0)
    ev, vec, st = S.solve(A, B, a.nev, x0, ev_tol=1e-10, ev_max_it=a.iters, precision=a.precision,
                          gemm=a.gemm)
    print(st)


if __name__ == "__main__":
    main()
