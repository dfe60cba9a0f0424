"""GPU parity of each kernel through the C ABI against the oracle's
restatement of the same reference operation (oracle/ops_ref.py)."""
import ctypes as C

import numpy as np
import pytest

from gcge_old_gb300 import matrices as M
from gcge_old_gb300.solver import DeviceMatrix
from gpu_util import dev_cols, host
from oracle import ops_ref as R

pytestmark = pytest.mark.gpu


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("gen,k", [(lambda: M.laplace2d(40), 1), (lambda: M.laplace2d(40), 13),
                                   (lambda: M.laplace3d_mass(14, seed=1)[0], 10),
                                   (lambda: M.diffusion27(9, seed=3)[0], 20)])
def test_spmm_matches_csr_matdotvec(cuda_lib, gen, k):
    A = gen()
    rng = np.random.default_rng(k)
    X = rng.standard_normal((k, A.n))
    xs, xp = dev_cols(X)
    ys, yp = dev_cols(np.zeros((k, A.n)))
    dA = DeviceMatrix(A)
    assert cuda_lib.GCGE_CUDA_MatDotMultiVec(dA.handle, xp, yp, k) == 0
    ref = R.mat_dot_multivec(A, X)
    np.testing.assert_allclose(host(ys), ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())


@pytest.mark.parametrize("k", [1, 4, 10, 13, 16, 20, 32])
def test_rows_spmm_matches_column_spmm(cuda_lib, k):
    """The row-interleaved FP32 operator of the mixed block CG equals A x
    column by column (FP32 sums of the same products in the same order)."""
    import torch
    A = M.laplace3d_mass(14, seed=1)[0]
    kw = (k + 3) // 4 * 4
    rng = np.random.default_rng(k)
    X = rng.standard_normal((A.n, kw)).astype(np.float32)
    X[:, k:] = 0.0
    x = torch.from_numpy(X).cuda()
    y = torch.full((A.n, kw), np.nan, dtype=torch.float32, device="cuda")
    dA = DeviceMatrix(A)
    assert cuda_lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(x.data_ptr()),
                                                 C.c_void_p(y.data_ptr()), k, None) == 0
    torch.cuda.synchronize()
    got = y.cpu().numpy()[:, :k]
    ref = (A.to_scipy().astype(np.float64) @ X[:, :k].astype(np.float64))
    # FP32 products summed in FP32 over <= 7 entries per row
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-5 * np.abs(ref).max())
    # bad arguments: more than 32 columns, misaligned rows
    assert cuda_lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(x.data_ptr()),
                                                 C.c_void_p(y.data_ptr()), 33, None) == 1
    assert cuda_lib.GCGE_CUDA_MatDotRowsF32Async(dA.handle, C.c_void_p(x.data_ptr() + 4),
                                                 C.c_void_p(y.data_ptr()), k, None) == 1


@pytest.mark.parametrize("k1,k2,sym,n", [(7, 3, 0, 1000), (90, 10, 0, 50000), (20, 20, 1, 30001),
                                         (130, 70, 0, 4099), (64, 64, 1, 777), (1, 1, 1, 5)])
def test_gram_matches_inner_prod(cuda_lib, k1, k2, sym, n):
    rng = np.random.default_rng(k1 * 7 + k2)
    V = rng.standard_normal((k1, n))
    W = V[:k2].copy() if sym else rng.standard_normal((k2, n))
    vs, vp = dev_cols(V)
    ws, wp = dev_cols(W)
    a = np.zeros((k1 + 3) * k2)
    assert cuda_lib.GCGE_CUDA_MultiVecInnerProd(vp, k1, wp, k2, n, _ptr(a), k1 + 3, sym) == 0
    got = a.reshape(k2, k1 + 3).T[:k1]
    ref = R.multivec_inner_prod(V, W, bool(sym))
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.sqrt(n))
    if sym:
        assert np.array_equal(got, got.T)


@pytest.mark.parametrize("k1,k2,beta,n", [(90, 70, 0.0, 20000), (5, 33, 1.0, 999),
                                          (200, 45, 0.5, 3000), (1, 1, 0.0, 7)])
def test_lincomb_matches_linear_comb(cuda_lib, k1, k2, beta, n):
    rng = np.random.default_rng(k1 + k2)
    X = rng.standard_normal((k1, n))
    Y0 = rng.standard_normal((k2, n))
    Cm = rng.standard_normal((k1, k2))
    lda = k1 + 2
    a = np.zeros((k2, lda))
    a[:, :k1] = Cm.T
    xs, xp = dev_cols(X)
    ys, yp = dev_cols(Y0)
    assert cuda_lib.GCGE_CUDA_MultiVecLinearComb(xp, k1, yp, k2, n, _ptr(a), lda, beta) == 0
    ref = R.multivec_linear_comb(X, Cm, Y0, beta)
    np.testing.assert_allclose(host(ys), ref, rtol=1e-12, atol=1e-12 * np.sqrt(k1))


def test_axpby(cuda_lib):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((4, 1001))
    Y = rng.standard_normal((4, 1001))
    xs, xp = dev_cols(X)
    ys, yp = dev_cols(Y)
    assert cuda_lib.GCGE_CUDA_MultiVecAxpby(2.0, xp, -0.5, yp, 4, 1001) == 0
    np.testing.assert_allclose(host(ys), 2.0 * X - 0.5 * Y, rtol=1e-15, atol=1e-15)


@pytest.mark.parametrize("m,il,iu", [(12, 1, 12), (80, 1, 40), (91, 3, 70), (150, 1, 150),
                                     (2, 1, 2), (1, 1, 1), (198, 1, 148), (256, 5, 256)])
def test_dense_eigensolver(cuda_lib, m, il, iu):
    rng = np.random.default_rng(m)
    Q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    w = np.sort(rng.uniform(1e-3, 1e3, m))
    if m > 10:
        w[5] = w[4]  # an exact double eigenvalue
    a = (Q * w) @ Q.T
    a = 0.5 * (a + a.T)
    lda = m + 1
    ah = np.zeros((m, lda))
    ah[:, :m] = a  # column-major with lda (symmetric)
    ev = np.zeros(iu - il + 1)
    vec = np.zeros((iu - il + 1, m + 2))
    rc = cuda_lib.GCGE_CUDA_DenseMatEigenSolver(_ptr(ah), lda, m, _ptr(ev), _ptr(vec), m + 2, il, iu)
    assert rc == 0
    ref = np.linalg.eigvalsh(a)[il - 1:iu]
    np.testing.assert_allclose(ev, ref, rtol=1e-12, atol=1e-12 * w.max())
    Z = vec[:, :m]
    for j in range(len(ev)):
        r = a @ Z[j] - ev[j] * Z[j]
        assert np.linalg.norm(r) < 1e-11 * w.max()
    np.testing.assert_allclose(Z @ Z.T, np.eye(len(ev)), atol=1e-12)


@pytest.mark.parametrize("fp32", [0, 1])
def test_block_cg_matches_reference_bcg(cuda_lib, fp32):
    A = M.laplace2d(30)
    k = 6
    rng = np.random.default_rng(5)
    rhs = rng.standard_normal((k, A.n))
    x0 = rng.standard_normal((k, A.n)) * 0.1
    rs, rp = dev_cols(rhs)
    xs, xp = dev_cols(x0)
    dA = DeviceMatrix(A)
    steps = C.c_int(0)
    assert cuda_lib.GCGE_CUDA_BlockCG(dA.handle, rp, xp, k, A.n, 20, 1e-2, fp32, C.byref(steps)) == 0
    X, Rr, niter = R.block_cg(A, rhs, x0, 20, 1e-2)
    got = host(xs)
    if not fp32:
        assert steps.value == niter
        np.testing.assert_allclose(got, X, rtol=1e-9, atol=1e-10 * np.abs(X).max())
    else:
        # single precision: same stopping rule, solution to FP32 accuracy
        assert abs(steps.value - niter) <= 2
        np.testing.assert_allclose(got, X, rtol=0, atol=1e-4 * np.abs(X).max())
    # every column reached the rate (or the step cap)
    a = A.to_scipy()
    for j in range(k):
        r0 = np.linalg.norm(rhs[j] - a @ x0[j])
        assert np.linalg.norm(rhs[j] - a @ got[j]) <= 1e-2 * r0 * (1.05 if fp32 else 1.0001) or steps.value == 20


def test_matcreate_rejects_bad_csr(cuda_lib):
    rp = np.array([0, 1, 3], dtype=np.int32)
    ci = np.array([0, 2, 1], dtype=np.int32)
    v = np.ones(3)
    h = C.c_void_p()
    rc = cuda_lib.GCGE_CUDA_MatCreate(C.byref(h), 2, _ptr(rp), _ptr(ci), _ptr(v), 0)
    assert rc == 1


@pytest.mark.parametrize("k1,k2,beta,n", [(90, 50, 0.0, 20001), (130, 70, 0.0, 3000),
                                          (200, 45, 0.5, 4097), (1, 1, 0.0, 7), (33, 8, 1.0, 64),
                                          (256, 130, 0.0, 1000)])
def test_ozaki_lincomb_is_fp64_accurate(cuda_lib, k1, k2, beta, n):
    """Tensor-core (error-free split) linear combination against an
    extended-precision reference: error below ~k1 * 2^-53 of sum |x||c|."""
    rng = np.random.default_rng(k1 * 3 + k2)
    X = rng.standard_normal((k1, n)) * np.exp(rng.uniform(-3, 3, size=(1, n)))
    Y0 = rng.standard_normal((k2, n))
    Cm = rng.standard_normal((k1, k2)) * np.exp(rng.uniform(-2, 2, size=(1, k2)))
    lda = k1 + 1
    a = np.zeros((k2, lda))
    a[:, :k1] = Cm.T
    xs, xp = dev_cols(X)
    ys, yp = dev_cols(Y0)
    assert cuda_lib.GCGE_CUDA_MultiVecLinearCombOzaki(xp, k1, yp, k2, n, _ptr(a), lda, beta) == 0
    got = host(ys)
    ref = (Cm.T.astype(np.longdouble) @ X.astype(np.longdouble)) + beta * Y0.astype(np.longdouble)
    bound = (np.abs(Cm.T) @ np.abs(X)) + abs(beta) * np.abs(Y0)
    err = np.abs(got - ref.astype(np.float64))
    assert np.max(err / bound) < 4 * 2.0 ** -52 * max(1, np.sqrt(k1)), np.max(err / bound)


def test_ozaki_lincomb_special_rows(cuda_lib):
    """Zero rows stay zero, a non-finite entry makes its row NaN, huge and
    tiny magnitudes keep their relative accuracy."""
    k1, k2, n = 20, 9, 300
    rng = np.random.default_rng(9)
    X = rng.standard_normal((k1, n))
    X[:, 5] = 0.0
    X[3, 17] = np.nan
    X[:, 40] *= 1e250
    X[:, 41] *= 1e-250
    Cm = rng.standard_normal((k1, k2))
    a = np.ascontiguousarray(Cm.T)
    xs, xp = dev_cols(X)
    ys, yp = dev_cols(np.zeros((k2, n)))
    assert cuda_lib.GCGE_CUDA_MultiVecLinearCombOzaki(xp, k1, yp, k2, n, _ptr(a), k1, 0.0) == 0
    got = host(ys)
    assert np.all(got[:, 5] == 0.0)
    assert np.all(np.isnan(got[:, 17]))
    ok = [c for c in range(n) if c != 17]
    Xf = np.nan_to_num(X)
    ref = (Cm.T.astype(np.longdouble) @ Xf.astype(np.longdouble)).astype(np.float64)
    bound = np.abs(Cm.T) @ np.abs(Xf)
    ok = [c for c in ok if c != 5]  # the zero row (bound 0) is checked above
    # one row 1e250 times larger sets every column's balancing exponent, and
    # the spread of that row's exponents (a few bits) comes off the
    # precision of C's slices: about 2^-48 of the bound here, 2^-52 for
    # balanced data
    assert np.max(np.abs(got[:, ok] - ref[:, ok]) / bound[:, ok]) < 64 * 2.0 ** -52


@pytest.mark.parametrize("k1,k2,sym,n", [(80, 10, 0, 100003), (20, 20, 1, 30001), (130, 70, 0, 4099),
                                         (50, 50, 1, 5000), (1, 1, 1, 5), (200, 25, 0, 777)])
def test_ozaki_gram_is_fp64_accurate(cuda_lib, k1, k2, sym, n):
    rng = np.random.default_rng(k1 * 5 + k2 + sym)
    V = rng.standard_normal((k1, n)) * np.exp(rng.uniform(-4, 4, size=(k1, 1)))
    V[:, : n // 3] *= 1e-3  # rows of very different size inside a column
    W = V[:k2].copy() if sym else rng.standard_normal((k2, n))
    vs, vp = dev_cols(V)
    ws, wp = dev_cols(W)
    a = np.zeros((k2, k1 + 2))
    assert cuda_lib.GCGE_CUDA_MultiVecInnerProdOzaki(vp, k1, wp, k2, n, _ptr(a), k1 + 2, sym) == 0
    got = a[:, :k1].T
    ref = (V.astype(np.longdouble) @ W.T.astype(np.longdouble)).astype(np.float64)
    bound = np.abs(V) @ np.abs(W).T
    # each 32-row chunk is scaled by its column maxima, so an entry much
    # smaller than its chunk's largest keeps fewer relative bits; the error
    # stays within a few units of 2^-53 of sum |v||w| (an FP64 dot product
    # of this length is bounded by n * 2^-53)
    assert np.max(np.abs(got - ref) / bound) < 16 * 2.0 ** -52, np.max(np.abs(got - ref) / bound)
    if sym:
        assert np.array_equal(got, got.T)


@pytest.mark.parametrize("k1,k2,n,diag", [(80, 10, 100003, True), (90, 10, 65536, False),
                                          (130, 20, 4099, True), (1, 1, 5, False),
                                          (96, 16, 64 * 37 + 1, True), (200, 33, 777, False)])
def test_plane_gram_is_fp64_accurate(cuda_lib, k1, k2, n, diag):
    """The Gram from digit planes of V (cut once) against exact products:
    columns of very different size, a chunk whose largest value sits just
    below a power of two (its top digit would be 128: cut with one more
    exponent bit), a zero column and ragged row counts; with and without a
    diagonal weight (the B-inner product of a diagonal B)."""
    import torch
    rng = np.random.default_rng(k1 * 7 + k2 + n)
    V = rng.standard_normal((k1, n)) * np.exp(rng.uniform(-4, 4, size=(k1, 1)))
    V[:, : n // 3] *= 1e-3
    if k1 > 2:
        V[1] = 0.0
        V[2, : min(n, 64)] = rng.uniform(-0.5, 0.5, min(n, 64))
        V[2, 0] = np.nextafter(1.0, 0.0)  # m = 2^55 - 4 at E = 0: needs E = 1
    W = rng.standard_normal((k2, n))
    d = rng.uniform(0.5, 2.0, n) if diag else np.ones(n)
    vs, vp = dev_cols(V)
    ws, wp = dev_cols(W)
    dt = torch.from_numpy(d).to("cuda") if diag else None
    a = np.zeros((k2, k1 + 3))
    assert cuda_lib.GCGE_CUDA_MultiVecInnerProdPlanes(
        vp, k1, wp, k2, n, C.c_void_p(dt.data_ptr()) if diag else None, _ptr(a), k1 + 3) == 0
    got = a[:, :k1].T
    Wd = W * d[None, :]
    ref = (V.astype(np.longdouble) @ Wd.T.astype(np.longdouble)).astype(np.float64)
    bound = np.abs(V) @ np.abs(Wd).T
    ok = bound > 0
    assert np.all(got[~ok] == 0.0)
    # each 64-row chunk is cut at its own column scales: the truncation error
    # of a chunk is a few units of 2^-55 of (rows x largest |v| x largest |w d|)
    # there, which on long columns is a few units of 2^-53 of sum |v| |w d|
    nc = (n + 63) // 64
    pad = nc * 64 - n
    vm = np.abs(np.pad(V, ((0, 0), (0, pad)))).reshape(k1, nc, 64).max(axis=2)
    wm = np.abs(np.pad(Wd, ((0, 0), (0, pad)))).reshape(k2, nc, 64).max(axis=2)
    cbound = 64 * vm @ wm.T
    assert np.max(np.abs(got[ok] - ref[ok]) / cbound[ok]) < 4 * 2.0 ** -53
    if n > 10_000:
        assert np.max(np.abs(got[ok] - ref[ok]) / bound[ok]) < 16 * 2.0 ** -52
    # the same products through the per-call digit path
    b = np.zeros((k2, k1))
    if not diag:
        assert cuda_lib.GCGE_CUDA_MultiVecInnerProdOzaki(vp, k1, wp, k2, n, _ptr(b), k1, 0) == 0
        assert np.max(np.abs(got - b.T)[ok] / cbound[ok]) < 8 * 2.0 ** -53


def test_plane_gram_non_finite_column(cuda_lib):
    """A NaN in a column of V turns that column's products into NaN only."""
    n, k1, k2 = 5000, 12, 3
    rng = np.random.default_rng(3)
    V = rng.standard_normal((k1, n))
    V[4, 777] = np.nan
    W = rng.standard_normal((k2, n))
    vs, vp = dev_cols(V)
    ws, wp = dev_cols(W)
    a = np.zeros((k2, k1))
    assert cuda_lib.GCGE_CUDA_MultiVecInnerProdPlanes(vp, k1, wp, k2, n, None, _ptr(a), k1) == 0
    got = a.T
    assert np.all(np.isnan(got[4]))
    rest = np.delete(np.arange(k1), 4)
    np.testing.assert_allclose(got[rest], V[rest] @ W.T, rtol=1e-13, atol=1e-12)


def test_ozaki_lincomb_unbalanced_columns(cuda_lib):
    """W R^{-1} of a CholQR step near convergence: the columns of W span
    eight orders of magnitude and R^{-1} undoes it; the balanced tensor-core
    product must stay at FP64 accuracy."""
    n, k = 4096, 10
    rng = np.random.default_rng(17)
    W = rng.standard_normal((n, k)) * np.logspace(-4, -12, k)[None, :]
    W[:, 9] += 1e-3 * W[:, 8]
    R = np.linalg.cholesky(W.T @ W).T
    T = np.linalg.inv(R)
    xs, xp = dev_cols(np.ascontiguousarray(W.T))
    ys, yp = dev_cols(np.zeros((k, n)))
    a = np.ascontiguousarray(T.T)  # column-major T
    assert cuda_lib.GCGE_CUDA_MultiVecLinearCombOzaki(xp, k, yp, k, n, _ptr(a), k, 0.0) == 0
    got = host(ys).T
    ref = (W.astype(np.longdouble) @ T.astype(np.longdouble)).astype(np.float64)
    assert np.abs(got - ref).max() < 1e-15 * np.abs(ref).max() * 10


@pytest.mark.parametrize("m,kind", [(60, "near"), (90, "many"), (120, "graded"), (30, "near"),
                                    (198, "many"), (256, "near")])
def test_dense_eigensolver_clusters(cuda_lib, m, kind):
    """Near-degenerate and graded spectra (the FP32 stage cannot separate
    them; the refinement and the clustered-pair Jacobi must)."""
    rng = np.random.default_rng(m + len(kind))
    Q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    if kind == "near":
        w = np.sort(rng.uniform(1, 10, m))
        w[3] = w[2] * (1 + 1e-9)
        w[7] = w[6] * (1 + 1e-12)
    elif kind == "many":
        w = np.sort(np.concatenate([30 + 1e-6 * rng.standard_normal(40), rng.uniform(1e3, 1e5, m - 40)]))
    else:
        w = np.sort(np.logspace(-2, 5, m))
    a = (Q * w) @ Q.T
    a = 0.5 * (a + a.T)
    il, iu = 1, min(m, 70)
    ev = np.zeros(iu - il + 1)
    vec = np.zeros((iu - il + 1, m))
    ah = np.ascontiguousarray(a)
    assert cuda_lib.GCGE_CUDA_DenseMatEigenSolver(_ptr(ah), m, m, _ptr(ev), _ptr(vec), m, il, iu) == 0
    ref = np.linalg.eigvalsh(a)[il - 1:iu]
    scale = np.abs(w).max()
    np.testing.assert_allclose(ev, ref, rtol=0, atol=1e-13 * scale)
    for j in range(len(ev)):
        assert np.linalg.norm(a @ vec[j] - ev[j] * vec[j]) < 1e-12 * scale
    np.testing.assert_allclose(vec @ vec.T, np.eye(len(ev)), atol=1e-13)
