// Multivector operations of include/gcge_cuda.h in the shape of the GCGE_OPS
// callbacks (src/gcge_ops.h:76-137), each a synchronous call over device
// columns.  They share the kernels of the solver.  Scratch (reduction
// partials, dense staging) is a per-process device buffer grown on demand;
// concurrent calls from several host threads are not supported.
#include <mutex>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "gcge_cuda_bcg.cuh"
#include "gcge_cuda_common.cuh"
#include "gcge_cuda_dense.cuh"


int gcge_record_error(int code, const char* msg);

namespace {

std::mutex g_mu;
double* g_scratch = nullptr;
size_t g_scratch_len = 0;

int scratch(size_t len, double** out) {
  if (len > g_scratch_len) {
    if (g_scratch) cudaFree(g_scratch);
    g_scratch = nullptr;
    g_scratch_len = 0;
    if (cudaMalloc(&g_scratch, sizeof(double) * len) != cudaSuccess) return GCGE_CUDA_ERR_ALLOC;
    g_scratch_len = len;
  }
  *out = g_scratch;
  return GCGE_CUDA_OK;
}

int finish() {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? GCGE_CUDA_OK : GCGE_CUDA_ERR_CUDA;
}

ColList<double> mk(double* const* p, int k) {
  ColList<double> c;
  for (int i = 0; i < k; i++) c.p[i] = p[i];
  return c;
}

}  // namespace

extern "C" int GCGE_CUDA_MatDotMultiVec(const GCGE_CUDA_MAT* A, double* const* x,
                                        double* const* y, int k) {
  if (!A || !x || !y || k < 0 || k > GCGE_MAXCOLS) return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  gcge::spmm_f64(A->m, mk(x, k), mk(y, k), k, 0);
  return finish();
}

extern "C" int GCGE_CUDA_MatDotMultiVecAsync(const GCGE_CUDA_MAT* A, double* const* x,
                                             double* const* y, int k, void* stream) {
  if (!A || !x || !y || k < 0 || k > GCGE_MAXCOLS) return GCGE_CUDA_ERR_ARG;
  gcge::spmm_f64(A->m, mk(x, k), mk(y, k), k, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? GCGE_CUDA_OK : GCGE_CUDA_ERR_CUDA;
}

namespace {
__global__ void k_val_to_f32(const double* __restrict__ a, float* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
}  // namespace

extern "C" int GCGE_CUDA_MatDotMultiVecF32Async(GCGE_CUDA_MAT* A, float* const* x,
                                                float* const* y, int k, void* stream) {
  if (!A || !x || !y || k < 0 || k > GCGE_MAXCOLS) return GCGE_CUDA_ERR_ARG;
  if (!A->m.v32) {
    if (cudaMalloc(&A->m.v32, sizeof(float) * (A->m.nnz > 0 ? A->m.nnz : 1)) != cudaSuccess)
      return GCGE_CUDA_ERR_ALLOC;
    if (A->m.nnz > 0)
      k_val_to_f32<<<(A->m.nnz + 255) / 256, 256, 0, (cudaStream_t)stream>>>(A->m.v, A->m.v32,
                                                                             A->m.nnz);
  }
  ColList<float> X, Y;
  for (int i = 0; i < k; i++) {
    X.p[i] = x[i];
    Y.p[i] = y[i];
  }
  gcge::spmm_f32(A->m, X, Y, k, (cudaStream_t)stream);
  return cudaGetLastError() == cudaSuccess ? GCGE_CUDA_OK : GCGE_CUDA_ERR_CUDA;
}

namespace {
// grad[e] = sum_j c_j x_j[row(e)] x_j[col(e)] over the stored entries e of M
__global__ void k_eiggrad(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                          ColList<double> X, DblList c, int k, double* __restrict__ grad) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int e = __ldg(rp + r); e < __ldg(rp + r + 1); e++) {
    const int col = __ldg(ci + e);
    double s = 0.0;
    for (int j = 0; j < k; j++) s = fma(c.v[j] * X.p[j][r], X.p[j][col], s);
    grad[e] = s;
  }
}
}  // namespace

extern "C" int GCGE_CUDA_EigGradCSR(const GCGE_CUDA_MAT* M, double* const* x, const double* coef,
                                    int k, double* grad) {
  if (!M || !x || !coef || !grad || k <= 0 || k > GCGE_MAXCOLS) return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  DblList c;
  for (int j = 0; j < k; j++) c.v[j] = coef[j];
  if (M->m.n > 0)
    k_eiggrad<<<(M->m.n + 255) / 256, 256>>>(M->m.n, M->m.rp, M->m.ci, mk(x, k), c, k, grad);
  return finish();
}

namespace {
constexpr int kPcgBlocks = 304;

__global__ void k_inv_diag(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ v, double* __restrict__ dinv) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 0.0;
  for (int e = rp[r]; e < rp[r + 1]; e++)
    if (ci[e] == r) d += v[e];
  dinv[r] = (d != 0.0) ? 1.0 / d : 1.0;
}

// partial[c * gridDim.x + b] = sum over this block's rows of X_c . Y_c
__global__ void k_coldot(ColList<double> X, ColList<double> Y, int k, int n,
                         double* __restrict__ partial) {
  __shared__ double sh[256];
  const int c = blockIdx.y;
  double s = 0.0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    s = fma(X.p[c][r], Y.p[c][r], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)c * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(const double* __restrict__ partial, int nblk, int k,
                               double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= k) return;
  double s = 0.0;
  for (int b = 0; b < nblk; b++) s += partial[(size_t)c * nblk + b];
  out[c] = s;
}

// r = rhs - w (in place in rhs); z = D^-1 r; p = z
__global__ void k_pcg_start(ColList<double> R, ColList<double> W, ColList<double> Z,
                            ColList<double> P, const double* __restrict__ dinv, int n) {
  const int c = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double r = R.p[c][i] - W.p[c][i];
    R.p[c][i] = r;
    const double z = dinv[i] * r;
    Z.p[c][i] = z;
    P.p[c][i] = z;
  }
}

// x += alpha p, r -= alpha w
__global__ void k_pcg_update(ColList<double> X, ColList<double> R, ColList<double> P,
                             ColList<double> W, DblList alpha, int n) {
  const int c = blockIdx.y;
  const double a = alpha.v[c];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    X.p[c][i] = fma(a, P.p[c][i], X.p[c][i]);
    R.p[c][i] = fma(-a, W.p[c][i], R.p[c][i]);
  }
}

// z = D^-1 r
__global__ void k_pcg_prec(ColList<double> R, ColList<double> Z, const double* __restrict__ dinv,
                           int n) {
  const int c = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    Z.p[c][i] = dinv[i] * R.p[c][i];
}

// p = z + beta p
__global__ void k_pcg_dir(ColList<double> Z, ColList<double> P, DblList beta, int n) {
  const int c = blockIdx.y;
  const double b = beta.v[c];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    P.p[c][i] = fma(b, P.p[c][i], Z.p[c][i]);
}

// per-column dots X_c . Y_c (c < k) -> host array out
int coldots(const ColList<double>& X, const ColList<double>& Y, int k, int n, double* partial,
            double* dout, double* out, cudaStream_t st) {
  k_coldot<<<dim3(kPcgBlocks, k), 256, 0, st>>>(X, Y, k, n, partial);
  k_sum_partials<<<(k + 63) / 64, 64, 0, st>>>(partial, kPcgBlocks, k, dout);
  if (cudaMemcpyAsync(out, dout, sizeof(double) * k, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  return cudaStreamSynchronize(st) == cudaSuccess ? GCGE_CUDA_OK : GCGE_CUDA_ERR_CUDA;
}

ColList<double> pick(const ColList<double>& X, const std::vector<int>& idx) {
  ColList<double> c;
  for (size_t j = 0; j < idx.size(); j++) c.p[j] = X.p[idx[j]];
  return c;
}
}  // namespace

extern "C" int GCGE_CUDA_JacobiPCG(void* ctx, const GCGE_CUDA_MAT* A, double* const* rhs,
                                   double* const* x, int k, int n, void* stream) {
  if (!A || !rhs || !x || k <= 0 || k > GCGE_MAXCOLS || n != A->m.n) return GCGE_CUDA_ERR_ARG;
  const GCGE_CUDA_PCG_PARAM* prm = static_cast<const GCGE_CUDA_PCG_PARAM*>(ctx);
  const int max_it = prm ? prm->max_it : 20;
  const double rate = prm ? prm->rate : 1e-2;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_mu);
  const size_t ld = ((size_t)n + 31) / 32 * 32;
  const size_t need = 3 * (size_t)k * ld + ld + (size_t)kPcgBlocks * k + GCGE_MAXCOLS;
  double* buf;
  if (scratch(need, &buf)) return GCGE_CUDA_ERR_ALLOC;
  ColList<double> R = mk(rhs, k), X = mk(x, k), Z, P, W;
  for (int j = 0; j < k; j++) {
    Z.p[j] = buf + (size_t)j * ld;
    P.p[j] = buf + (size_t)(k + j) * ld;
    W.p[j] = buf + (size_t)(2 * k + j) * ld;
  }
  double* dinv = buf + 3 * (size_t)k * ld;
  double* partial = dinv + ld;
  double* dout = partial + (size_t)kPcgBlocks * k;
  const GcgeDevCsr& M = A->m;
  k_inv_diag<<<(n + 255) / 256, 256, 0, st>>>(n, M.rp, M.ci, M.v, dinv);
  gcge::spmm_f64(M, X, W, k, st);
  k_pcg_start<<<dim3(kPcgBlocks, k), 256, 0, st>>>(R, W, Z, P, dinv, n);
  std::vector<double> rz(k), r0(k), tmp(k);
  int rc = coldots(R, R, k, n, partial, dout, r0.data(), st);
  if (!rc) rc = coldots(R, Z, k, n, partial, dout, rz.data(), st);
  if (rc) return rc;
  std::vector<int> act;
  for (int j = 0; j < k; j++) {
    r0[j] = sqrt(r0[j]);
    if (r0[j] > 0.0) act.push_back(j);
  }
  for (int it = 0; it < max_it && !act.empty(); it++) {
    const int m = (int)act.size();
    ColList<double> Ra = pick(R, act), Xa = pick(X, act), Za = pick(Z, act), Pa = pick(P, act),
                    Wa = pick(W, act);
    gcge::spmm_f64(M, Pa, Wa, m, st);
    if ((rc = coldots(Pa, Wa, m, n, partial, dout, tmp.data(), st))) return rc;
    DblList alpha;
    for (int a = 0; a < m; a++) alpha.v[a] = tmp[a] != 0.0 ? rz[act[a]] / tmp[a] : 0.0;
    k_pcg_update<<<dim3(kPcgBlocks, m), 256, 0, st>>>(Xa, Ra, Pa, Wa, alpha, n);
    if ((rc = coldots(Ra, Ra, m, n, partial, dout, tmp.data(), st))) return rc;
    std::vector<int> next;
    for (int a = 0; a < m; a++)
      if (sqrt(tmp[a]) >= rate * r0[act[a]]) next.push_back(act[a]);
    if (next.empty() || it + 1 == max_it) break;
    const int m2 = (int)next.size();
    ColList<double> Rn = pick(R, next), Zn = pick(Z, next), Pn = pick(P, next);
    k_pcg_prec<<<dim3(kPcgBlocks, m2), 256, 0, st>>>(Rn, Zn, dinv, n);
    if ((rc = coldots(Rn, Zn, m2, n, partial, dout, tmp.data(), st))) return rc;
    DblList beta;
    for (int a = 0; a < m2; a++) {
      beta.v[a] = rz[next[a]] != 0.0 ? tmp[a] / rz[next[a]] : 0.0;
      rz[next[a]] = tmp[a];
    }
    k_pcg_dir<<<dim3(kPcgBlocks, m2), 256, 0, st>>>(Zn, Pn, beta, n);
    act = next;
  }
  return cudaStreamSynchronize(st) == cudaSuccess && cudaGetLastError() == cudaSuccess
             ? GCGE_CUDA_OK
             : GCGE_CUDA_ERR_CUDA;
}

extern "C" int GCGE_CUDA_MatDotRowsF32Async(GCGE_CUDA_MAT* A, const float* x, float* y, int k,
                                            void* stream) {
  if (!A || !x || !y || k <= 0 || k > 32 || ((uintptr_t)x & 15) || ((uintptr_t)y & 15))
    return GCGE_CUDA_ERR_ARG;
  if (!A->m.v32) {
    if (cudaMalloc(&A->m.v32, sizeof(float) * (A->m.nnz > 0 ? A->m.nnz : 1)) != cudaSuccess)
      return GCGE_CUDA_ERR_ALLOC;
    if (A->m.nnz > 0)
      k_val_to_f32<<<(A->m.nnz + 255) / 256, 256, 0, (cudaStream_t)stream>>>(A->m.v, A->m.v32,
                                                                             A->m.nnz);
  }
  gcge::spmm_rows_f32(A->m.rp, A->m.ci, A->m.v32, A->m.n, x, y, k, (cudaStream_t)stream, &A->m);
  return cudaGetLastError() == cudaSuccess ? GCGE_CUDA_OK : GCGE_CUDA_ERR_CUDA;
}

extern "C" int GCGE_CUDA_MultiVecInnerProd(double* const* V, int k1, double* const* W, int k2,
                                           int n, double* a, int lda, int sym) {
  if (!V || !W || !a || k1 < 0 || k2 < 0 || k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || n <= 0 ||
      lda < k1 || (sym && k1 != k2))
    return GCGE_CUDA_ERR_ARG;
  if (k1 == 0 || k2 == 0) return GCGE_CUDA_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  const int tiles = ((k1 + 63) / 64) * ((k2 + 63) / 64);
  double* buf;
  const size_t part = (size_t)gcge::kRowBlocks * tiles * 64 * 64;
  if (scratch(part + (size_t)k1 * k2, &buf)) return GCGE_CUDA_ERR_ALLOC;
  double* G = buf + part;
  gcge::gram_f64(mk(V, k1), k1, mk(W, k2), k2, n, G, k1, sym != 0, buf, 0);
  std::vector<double> h((size_t)k1 * k2);
  if (cudaMemcpy(h.data(), G, sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) a[i + (size_t)j * lda] = h[i + (size_t)j * k1];
  return finish();
}

extern "C" int GCGE_CUDA_MultiVecInnerProdOzaki(double* const* V, int k1, double* const* W,
                                                int k2, int n, double* a, int lda, int sym) {
  if (!V || !W || !a || k1 < 0 || k2 < 0 || k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || n <= 0 ||
      lda < k1 || (sym && k1 != k2))
    return GCGE_CUDA_ERR_ARG;
  if (k1 == 0 || k2 == 0) return GCGE_CUDA_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  const size_t part = gcge::gram_oz_partial_doubles(k1, k2);
  double* buf;
  if (scratch(part + (size_t)k1 * k2, &buf)) return GCGE_CUDA_ERR_ALLOC;
  double* G = buf + part;
  gcge::gram_oz(mk(V, k1), k1, mk(W, k2), k2, n, G, k1, sym != 0, buf, 0);
  std::vector<double> h((size_t)k1 * k2);
  if (cudaMemcpy(h.data(), G, sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) a[i + (size_t)j * lda] = h[i + (size_t)j * k1];
  return finish();
}

extern "C" int GCGE_CUDA_MultiVecInnerProdPlanes(double* const* V, int k1, double* const* W,
                                                 int k2, int n, const double* wdiag, double* a,
                                                 int lda) {
  if (!V || !W || !a || k1 < 0 || k2 < 0 || k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || n <= 0 ||
      lda < k1)
    return GCGE_CUDA_ERR_ARG;
  if (k1 == 0 || k2 == 0) return GCGE_CUDA_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  const size_t part = gcge::gram_oz_partial_doubles(k1, k2);
  const size_t pl_doubles = (gcge::planes_bytes(n, k1) + gcge::planes_bytes(n, k2) + 7) / 8 + 4;
  double* buf;
  if (scratch(part + (size_t)k1 * k2 + pl_doubles, &buf)) return GCGE_CUDA_ERR_ALLOC;
  double* G = buf + part;
  uint8_t* planes = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(G + (size_t)k1 * k2) + 15) & ~(uintptr_t)15);
  uint8_t* wplanes = planes + (gcge::planes_bytes(n, k1) + 15) / 16 * 16;
  gcge::cut_planes(mk(V, k1), k1, n, planes, k1, 0, 0);
  gcge::cut_planes(mk(W, k2), k2, n, wplanes, k2, 0, 0, wdiag);
  gcge::gram_oz_planes(planes, k1, 0, k1, wplanes, k2, 0, k2, n, G, k1, buf, 0);
  std::vector<double> h((size_t)k1 * k2);
  if (cudaMemcpy(h.data(), G, sizeof(double) * h.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) a[i + (size_t)j * lda] = h[i + (size_t)j * k1];
  return finish();
}

extern "C" size_t GCGE_CUDA_PlanesBytes(int n, int ldp) {
  return (n > 0 && ldp > 0) ? gcge::planes_bytes(n, ldp) : 0;
}

extern "C" size_t GCGE_CUDA_PlanesGramScratchDoubles(int k1, int k2) {
  return (k1 > 0 && k2 > 0) ? gcge::gram_oz_partial_doubles(k1, k2) : 0;
}

extern "C" int GCGE_CUDA_PlanesCut(double* const* X, int k, int n, const double* wdiag,
                                   void* planes, int ldp, int c0, void* stream) {
  if (!X || !planes || k < 0 || k > GCGE_MAXCOLS || n <= 0 || c0 < 0 || c0 + k > ldp ||
      ((uintptr_t)planes & 15) != 0)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "PlanesCut: bad arguments");
  gcge::cut_planes(mk(X, k), k, n, static_cast<uint8_t*>(planes), ldp, c0, (cudaStream_t)stream,
                   wdiag);
  return cudaPeekAtLastError() == cudaSuccess
             ? GCGE_CUDA_OK
             : gcge_record_error(GCGE_CUDA_ERR_CUDA, "PlanesCut: launch failed");
}

extern "C" int GCGE_CUDA_PlanesGram(const void* vplanes, int ldv, int voff, int k1,
                                    const void* wplanes, int ldw, int woff, int k2, int n,
                                    double* a, int lda, double* partial, void* stream) {
  if (!vplanes || !wplanes || !a || !partial || k1 <= 0 || k2 <= 0 || k1 > GCGE_MAXCOLS ||
      k2 > GCGE_MAXCOLS || n <= 0 || voff < 0 || woff < 0 || voff + k1 > ldv ||
      woff + k2 > ldw || lda < k1 || ((uintptr_t)vplanes & 15) != 0 ||
      ((uintptr_t)wplanes & 15) != 0)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "PlanesGram: bad arguments");
  gcge::gram_oz_planes(static_cast<const uint8_t*>(vplanes), ldv, voff, k1,
                       static_cast<const uint8_t*>(wplanes), ldw, woff, k2, n, a, lda, partial,
                       (cudaStream_t)stream);
  return cudaPeekAtLastError() == cudaSuccess
             ? GCGE_CUDA_OK
             : gcge_record_error(GCGE_CUDA_ERR_CUDA, "PlanesGram: launch failed");
}

extern "C" int GCGE_CUDA_MultiVecLinearComb(double* const* x, int k1, double* const* y, int k2,
                                            int n, const double* a, int lda, double beta) {
  if (!x || !y || !a || k1 < 0 || k2 < 0 || k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || n <= 0 ||
      lda < k1)
    return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  double* C;
  if (scratch((size_t)(k1 > 0 ? k1 : 1) * (k2 > 0 ? k2 : 1), &C)) return GCGE_CUDA_ERR_ALLOC;
  std::vector<double> h((size_t)k1 * k2);
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) h[i + (size_t)j * k1] = a[i + (size_t)j * lda];
  if (!h.empty() &&
      cudaMemcpy(C, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  gcge::lincomb_f64(mk(x, k1), k1, C, k1, mk(y, k2), k2, beta, n, 0);
  return finish();
}

extern "C" int GCGE_CUDA_MultiVecLinearCombOzaki(double* const* x, int k1, double* const* y,
                                                  int k2, int n, const double* a, int lda,
                                                  double beta) {
  if (!x || !y || !a || k1 < 0 || k2 < 0 || k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || n <= 0 ||
      lda < k1)
    return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  const size_t cb = (size_t)(k1 > 0 ? k1 : 1) * (k2 > 0 ? k2 : 1);
  const size_t sb = (gcge::lincomb_oz_scratch_bytes(k1, k2) + 15) / 8 + 2;
  double* buf;
  if (scratch(cb + sb, &buf)) return GCGE_CUDA_ERR_ALLOC;
  double* C = buf;
  void* sc = reinterpret_cast<void*>(((uintptr_t)(buf + cb) + 15) & ~(uintptr_t)15);
  std::vector<double> h(cb, 0.0);
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) h[i + (size_t)j * k1] = a[i + (size_t)j * lda];
  if (cudaMemcpy(C, h.data(), sizeof(double) * cb, cudaMemcpyHostToDevice) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  gcge::lincomb_oz(mk(x, k1), k1, C, k1 > 0 ? k1 : 1, mk(y, k2), k2, beta, n, sc, 0, true);
  return finish();
}

extern "C" int GCGE_CUDA_MultiVecAxpby(double alpha, double* const* x, double beta,
                                       double* const* y, int k, int n) {
  if (!x || !y || k < 0 || k > GCGE_MAXCOLS || n <= 0) return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  gcge::axpby_f64(alpha, mk(x, k), beta, mk(y, k), k, n, 0);
  return finish();
}

extern "C" int GCGE_CUDA_DenseMatEigenSolver(const double* a, int lda, int nrows, double* eval,
                                             double* evec, int lde, int il, int iu) {
  if (!a || !eval || !evec || nrows <= 0 || nrows > 256 || lda < nrows || lde < nrows || il < 1 ||
      iu < il || iu > nrows)
    return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  const int m = iu - il + 1;
  const size_t need = (size_t)nrows * nrows + (size_t)nrows * m + m +
                      gcge::jacobi_work_doubles(nrows) + 1;
  double* buf;
  if (scratch(need, &buf)) return GCGE_CUDA_ERR_ALLOC;
  double* dA = buf;
  double* dV = dA + (size_t)nrows * nrows;
  double* dE = dV + (size_t)nrows * m;
  double* work = dE + m;
  int* status = reinterpret_cast<int*>(work + gcge::jacobi_work_doubles(nrows));
  if (cudaMemcpy2D(dA, sizeof(double) * nrows, a, sizeof(double) * lda, sizeof(double) * nrows,
                   nrows, cudaMemcpyHostToDevice) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  gcge::jacobi_eig(nrows, dA, nrows, dE, dV, nrows, il, iu, work, status, 0);
  int st = 0;
  if (cudaMemcpy(&st, status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  if (cudaMemcpy(eval, dE, sizeof(double) * m, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  if (cudaMemcpy2D(evec, sizeof(double) * lde, dV, sizeof(double) * nrows, sizeof(double) * nrows,
                   m, cudaMemcpyDeviceToHost) != cudaSuccess)
    return GCGE_CUDA_ERR_CUDA;
  if (st < 0) return GCGE_CUDA_ERR_NUMERIC;
  return finish();
}

namespace {
__global__ void k_cvt_d2f(const double* __restrict__ a, float* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
__global__ void k_cvt_f2d(const float* __restrict__ a, double* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}
}  // namespace

extern "C" int GCGE_CUDA_BlockCG(const GCGE_CUDA_MAT* A, double* const* rhs, double* const* x,
                                 int k, int n, int max_it, double rate, int fp32, int* steps) {
  if (!A || !rhs || !x || k <= 0 || k > GCGE_MAXCOLS || n != A->m.n) return GCGE_CUDA_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  const int nb = gcge::kRowBlocks;
  const size_t ld = ((size_t)n + 31) / 32 * 32;
  // scalars: 6 arrays of k doubles, partial k*nb, vectors (P, W, and for FP32
  // also RHS, X copies) in the precision of the solve
  const size_t nvec = fp32 ? 4 : 2;
  const size_t vec_doubles = fp32 ? (nvec * k * ld + 1) / 2 + 1 : nvec * k * ld;
  double* buf;
  if (scratch(6 * (size_t)GCGE_MAXCOLS + (size_t)k * nb + vec_doubles + GCGE_MAXCOLS, &buf))
    return GCGE_CUDA_ERR_ALLOC;
  int* ints = nullptr;
  int* pinned = nullptr;
  if (cudaMalloc(&ints, sizeof(int) * (GCGE_MAXCOLS + 1)) != cudaSuccess) return GCGE_CUDA_ERR_ALLOC;
  if (cudaHostAlloc(&pinned, sizeof(int) * 4, cudaHostAllocMapped) != cudaSuccess) {
    cudaFree(ints);
    return GCGE_CUDA_ERR_ALLOC;
  }
  gcge::BcgScalars s;
  s.rho1 = buf;
  s.rho2 = buf + GCGE_MAXCOLS;
  s.err = buf + 2 * GCGE_MAXCOLS;
  s.lerr = buf + 3 * GCGE_MAXCOLS;
  s.ptw = buf + 4 * GCGE_MAXCOLS;
  s.rnew = buf + 5 * GCGE_MAXCOLS;
  s.unl = ints;
  s.nu = ints + GCGE_MAXCOLS;
  s.nu_host = pinned;
  s.acol = nullptr;  // column path only
  s.mask = nullptr;
  s.bcol = nullptr;
  s.acolf = nullptr;
  double* partial = buf + 6 * GCGE_MAXCOLS;
  double* vecs = partial + (size_t)k * nb;
  int it = -1;
  GcgeDevCsr M = A->m;
  if (!fp32) {
    ColList<double> R = mk(rhs, k), X = mk(x, k), P, W;
    for (int j = 0; j < k; j++) {
      P.p[j] = vecs + (size_t)j * ld;
      W.p[j] = vecs + (size_t)(k + j) * ld;
    }
    it = gcge::bcg_run<double>(M.rp, M.ci, M.v, n, R, X, P, W, k, max_it, rate, s, partial, 0,
                               nullptr, &M);
  } else {
    float* f = reinterpret_cast<float*>(vecs);
    float* v32 = nullptr;
    if (cudaMalloc(&v32, sizeof(float) * (M.nnz > 0 ? M.nnz : 1)) != cudaSuccess) {
      cudaFree(ints);
      cudaFreeHost(pinned);
      return GCGE_CUDA_ERR_ALLOC;
    }
    if (M.nnz > 0) k_cvt_d2f<<<(M.nnz + 255) / 256, 256>>>(M.v, v32, M.nnz);
    ColList<float> R, X, P, W;
    for (int j = 0; j < k; j++) {
      R.p[j] = f + (size_t)j * ld;
      X.p[j] = f + (size_t)(k + j) * ld;
      P.p[j] = f + (size_t)(2 * k + j) * ld;
      W.p[j] = f + (size_t)(3 * k + j) * ld;
      k_cvt_d2f<<<(n + 255) / 256, 256>>>(rhs[j], R.p[j], n);
      k_cvt_d2f<<<(n + 255) / 256, 256>>>(x[j], X.p[j], n);
    }
    it = gcge::bcg_run<float>(M.rp, M.ci, v32, n, R, X, P, W, k, max_it, rate, s, partial, 0,
                              nullptr, &M);
    for (int j = 0; j < k; j++) {
      k_cvt_f2d<<<(n + 255) / 256, 256>>>(X.p[j], x[j], n);
      k_cvt_f2d<<<(n + 255) / 256, 256>>>(R.p[j], rhs[j], n);
    }
    cudaDeviceSynchronize();
    cudaFree(v32);
  }
  const int rc = finish();
  cudaFree(ints);
  cudaFreeHost(pinned);
  if (steps) *steps = it;
  if (it < 0) return GCGE_CUDA_ERR_CUDA;
  return rc;
}
