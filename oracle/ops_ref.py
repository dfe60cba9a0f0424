"""ORACLE TEST INFRASTRUCTURE — not part of the product.

numpy restatements of the reference's multivector operations and block CG,
used as checkers for the CUDA kernels of the same operations (each op runs
on the GPU through the C ABI in tests/test_gpu_kernels.py and is compared
with the function here on the same seeded inputs).  Sizes are small.
"""
from __future__ import annotations

import numpy as np


def mat_dot_multivec(A, X):
    """CSR_MatDotVec column by column (app/csr/gcge_app_csr.c:297-323);
    X: (k, n) rows are the columns of the multivector."""
    a = A.to_scipy()
    return np.stack([a @ x for x in X]) if len(X) else np.zeros((0, A.n))


def multivec_inner_prod(V, W, sym: bool):
    """GCGE_Default_MultiVecInnerProd (src/gcge_ops.c:226-309): a(i,j) =
    V_i . W_j; "sym" forms the upper triangle (i <= j) then mirrors it."""
    k1, k2 = len(V), len(W)
    a = np.zeros((k1, k2))
    for j in range(k2):
        for i in range(k1):
            if sym and i > j:
                continue
            a[i, j] = float(np.dot(V[i], W[j]))
    if sym:
        for j in range(k2):
            for i in range(j + 1, k1):
                a[i, j] = a[j, i]
    return a


def multivec_linear_comb(X, C, Y=None, beta=0.0):
    """GCGE_Default_MultiVecLinearComb (src/gcge_ops.c:190-221):
    y_j = sum_i x_i C[i, j] + beta y_j."""
    out = (C.T @ X)
    if beta != 0.0 and Y is not None:
        out = out + beta * Y
    return out


def block_cg(A, RHS, X, max_it, rate):
    """GCGE_BCG (src/gcge_cg.c:302-501) in float64, including its scalar
    indexing (beta by column index, alpha and the rho update by compacted
    index).  Returns (X, R, niter)."""
    a = A.to_scipy()
    R = RHS.copy()
    X = X.copy()
    k = len(R)
    P = np.zeros_like(R)
    Wv = np.zeros_like(R)
    rho1 = np.zeros(k)
    rho2 = np.zeros(k)
    ptw = np.zeros(k)
    lerr = np.zeros(k)
    for idx in range(k):
        R[idx] = R[idx] - a @ X[idx]
        rho2[idx] = R[idx] @ R[idx]
    err = np.sqrt(rho2)
    lerr[:] = err
    unl = [i for i in range(k) if err[i] >= 1e-15]
    niter = 1
    while unl and niter < max_it:
        for id_, idx in enumerate(unl):
            if niter == 1:
                P[idx] = R[idx]
            else:
                P[idx] = R[idx] + (rho2[idx] / rho1[idx]) * P[idx]
            Wv[idx] = a @ P[idx]
            ptw[id_] = P[idx] @ Wv[idx]
        for id_, idx in enumerate(unl):
            alpha = rho2[id_] / ptw[id_]
            X[idx] = X[idx] + alpha * P[idx]
            R[idx] = R[idx] - alpha * Wv[idx]
            rho1[id_] = rho2[id_]
            rho2[id_] = R[idx] @ R[idx]
        for id_, idx in enumerate(unl):
            lerr[idx] = np.sqrt(abs(rho2[id_]))
        unl = [idx for idx in unl if lerr[idx] >= rate * err[idx] and lerr[idx] >= 1e-15]
        niter += 1
    return X, R, niter
