"""Profiling driver: one GCG solve of the 3D 7-point Laplacian with diagonal
mass (the benchmark's generator) on an m^3 grid for a fixed number of GCG
iterations, so a profiler sees a bounded, repeatable launch sequence.

    python -m gcge_old_gb300.profile_solve --grid 96 --iters 6 --precision mixed
"""
import argparse

from . import matrices as M
from . import solver as S


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=96)
    ap.add_argument("--iters", type=int, default=6)
    ap.add_argument("--nev", type=int, default=50)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--gemm", default="ozaki", choices=["ozaki", "fp64"])
    a = ap.parse_args()
    A, B = M.laplace3d_mass(a.grid, seed=0)
    x0 = M.initial_block(A.n, a.nev, seed=0)
    ev, vec, st = S.solve(A, B, a.nev, x0, ev_tol=1e-10, ev_max_it=a.iters, precision=a.precision,
                          gemm=a.gemm)
    print(st)


if __name__ == "__main__":
    main()
