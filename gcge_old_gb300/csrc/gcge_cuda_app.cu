// The GCGE_OPS table of the CUDA app (include/gcge_cuda_ops.h): the callbacks
// through which the reference core (src/gcge_*.c) works on device vectors.
//
// Vector handle: CudaVec (n, one device column).  Multivector handle: CudaMv,
// an opaque block of k CudaVec columns (like the SLEPc app's BV handle,
// app/slepc/gcge_app_slepc.c:174-392); the core never indexes a multivector
// itself, it asks GetVecFromMultiVec for a column.  MultiVecSwap exchanges
// the column buffers of two handles (what the default array-of-pointers
// multivector does, src/gcge_ops.c).  All work runs on the
// legacy default stream; the callbacks that hand a value to the host (inner
// products) synchronise.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gcge_cuda.h"
#include "../../include/gcge_cuda_ops.h"
#include "gcge_cuda_common.cuh"
#include "gcge_cuda_dense.cuh"

int gcge_record_error(int code, const char* msg);

namespace {

struct CudaVec {
  int n = 0;
  double* d = nullptr;
  bool owned = false;
};

// Each column is its own device buffer, owned by whichever handle holds it:
// MultiVecSwap moves buffers between handles and MultiVecDestroy frees the
// ones a handle holds at that time (the ownership rule of the default
// array-of-vectors multivector).
struct CudaMv {
  int n = 0, k = 0;
  std::vector<CudaVec> col;
};

std::mutex g_ops_mu;
int g_ops_err = GCGE_CUDA_OK;
double* g_ops_scratch = nullptr;   // device scratch of the block callbacks
size_t g_ops_scratch_len = 0;

bool failed() { return g_ops_err != GCGE_CUDA_OK; }

void fail(int code, const char* msg) {
  if (g_ops_err == GCGE_CUDA_OK) g_ops_err = code;
  gcge_record_error(code, msg);
}

bool cuda_ok(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return true;
  char m[256];
  snprintf(m, sizeof(m), "%s: %s", where, cudaGetErrorString(e));
  fail(GCGE_CUDA_ERR_CUDA, m);
  return false;
}

bool launched(const char* where) { return cuda_ok(cudaGetLastError(), where); }

double* ops_scratch(size_t len) {
  if (len > g_ops_scratch_len) {
    if (g_ops_scratch) cudaFree(g_ops_scratch);
    g_ops_scratch = nullptr;
    g_ops_scratch_len = 0;
    if (cudaMalloc(&g_ops_scratch, sizeof(double) * len) != cudaSuccess) {
      fail(GCGE_CUDA_ERR_ALLOC, "GCGE_CUDA ops: scratch allocation failed");
      return nullptr;
    }
    g_ops_scratch_len = len;
  }
  return g_ops_scratch;
}

CudaVec* V_(void* v) { return static_cast<CudaVec*>(v); }
CudaMv* MV_(void** v) { return reinterpret_cast<CudaMv*>(v); }
const GcgeDevCsr& M_(void* m) { return static_cast<GCGE_CUDA_MAT*>(m)->m; }

bool range_ok(const CudaMv* mv, int s, int e, const char* where) {
  if (mv && s >= 0 && e >= s && e <= mv->k) return true;
  char m[200];
  snprintf(m, sizeof(m), "%s: columns %d..%d outside the multivector (%d)", where, s, e,
           mv ? mv->k : -1);
  fail(GCGE_CUDA_ERR_ARG, m);
  return false;
}

ColList<double> cols_of(const CudaMv* mv, int s, int k) {
  ColList<double> c;
  for (int i = 0; i < k; i++) c.p[i] = mv->col[s + i].d;
  return c;
}

// U[0, 1) pseudo-random values (the reference CSR app fills rand()/(RAND_MAX+1),
// app/csr/gcge_app_csr.c:284-294); splitmix64 of (row, call counter)
__global__ void k_ops_random(double* __restrict__ x, int n, unsigned long long seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long z = (unsigned long long)i + 0x9E3779B97F4A7C15ull * (seed + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    x[i] = (double)(z >> 11) * 0x1.0p-53;
  }
}
unsigned long long g_random_calls = 0;

void fill_random(double* d, int n) {
  const int g = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  k_ops_random<<<g > 0 ? g : 1, 256>>>(d, n, ++g_random_calls);
  launched("VecSetRandomValue");
}

double* col_alloc(int n) {
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * (n > 0 ? n : 1)) != cudaSuccess) {
    fail(GCGE_CUDA_ERR_ALLOC, "GCGE_CUDA ops: device allocation failed");
    return nullptr;
  }
  if (!cuda_ok(cudaMemset(d, 0, sizeof(double) * (n > 0 ? n : 1)), "vector create")) {
    cudaFree(d);
    return nullptr;
  }
  return d;
}

void mv_destroy(CudaMv* mv) {
  if (!mv) return;
  for (auto& c : mv->col) cudaFree(c.d);
  delete mv;
}

CudaMv* mv_create(int n_vec, int n) {
  CudaMv* mv = new CudaMv();
  mv->n = n;
  mv->k = n_vec > 0 ? n_vec : 0;
  mv->col.resize(mv->k);
  for (int j = 0; j < mv->k; j++) {
    mv->col[j].n = n;
    mv->col[j].d = col_alloc(n);
    if (!mv->col[j].d) {
      mv_destroy(mv);
      return nullptr;
    }
  }
  return mv;
}

}  // namespace

// ---------------------------------------------------------------- callbacks
// The argument meanings are those of struct GCGE_OPS (src/gcge_ops.h:29-150)
// and of the reference's default multivector operations (src/gcge_ops.c).
namespace {

void cb_VecSetRandomValue(void* vec, GCGE_CUDA_OPS*) {
  if (failed() || !vec) return;
  fill_random(V_(vec)->d, V_(vec)->n);
}

void cb_MatDotVec(void* mat, void* x, void* r, GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!mat || !x || !r) return fail(GCGE_CUDA_ERR_ARG, "MatDotVec: null handle");
  ColList<double> X, Y;
  X.p[0] = V_(x)->d;
  Y.p[0] = V_(r)->d;
  gcge::spmm_f64(M_(mat), X, Y, 1, 0);
  launched("MatDotVec");
}

// y = a x + b y (src/gcge_ops.h:41); b == 0 overwrites y without reading it
void cb_VecAxpby(double a, void* x, double b, void* y, GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!x || !y) return fail(GCGE_CUDA_ERR_ARG, "VecAxpby: null handle");
  ColList<double> X, Y;
  X.p[0] = V_(x)->d;
  Y.p[0] = V_(y)->d;
  if (b == 0.0 && V_(x)->d != V_(y)->d)
    cuda_ok(cudaMemsetAsync(V_(y)->d, 0, sizeof(double) * V_(y)->n, 0), "VecAxpby");
  gcge::axpby_f64(a, X, b, Y, 1, V_(y)->n, 0);
  launched("VecAxpby");
}

void cb_VecInnerProd(void* x, void* y, double* v, GCGE_CUDA_OPS*) {
  if (!v) return;
  *v = 0.0;
  if (failed()) return;
  if (!x || !y) return fail(GCGE_CUDA_ERR_ARG, "VecInnerProd: null handle");
  double* buf = ops_scratch((size_t)gcge::kRowBlocks + 1);
  if (!buf) return;
  ColList<double> X, Y;
  X.p[0] = V_(x)->d;
  Y.p[0] = V_(y)->d;
  gcge::gram_f64(X, 1, Y, 1, V_(x)->n, buf + gcge::kRowBlocks, 1, false, buf, 0);
  if (launched("VecInnerProd"))
    cuda_ok(cudaMemcpy(v, buf + gcge::kRowBlocks, sizeof(double), cudaMemcpyDeviceToHost),
            "VecInnerProd");
}

void cb_VecCreateByMat(void** vec, void* mat, GCGE_CUDA_OPS*) {
  if (!vec) return;
  *vec = nullptr;
  if (failed()) return;
  if (!mat) return fail(GCGE_CUDA_ERR_ARG, "VecCreateByMat: null matrix");
  CudaVec* v = new CudaVec();
  v->n = M_(mat).n;
  v->d = col_alloc(v->n);
  v->owned = true;
  if (!v->d) {
    delete v;
    return;
  }
  *vec = v;
}

void cb_VecCreateByVec(void** des, void* src, GCGE_CUDA_OPS*) {
  if (!des) return;
  *des = nullptr;
  if (failed()) return;
  if (!src) return fail(GCGE_CUDA_ERR_ARG, "VecCreateByVec: null vector");
  CudaVec* v = new CudaVec();
  v->n = V_(src)->n;
  v->d = col_alloc(v->n);
  v->owned = true;
  if (!v->d) {
    delete v;
    return;
  }
  *des = v;
}

void cb_VecDestroy(void** vec, GCGE_CUDA_OPS*) {
  if (!vec || !*vec) return;
  CudaVec* v = V_(*vec);
  if (v->owned) {
    cudaFree(v->d);
    delete v;
  }
  *vec = nullptr;
}

void cb_GetVecFromMultiVec(void** V, int j, void** x, GCGE_CUDA_OPS*) {
  if (!x) return;
  CudaMv* mv = MV_(V);
  if (!mv || j < 0 || j >= mv->k) {
    *x = nullptr;
    return fail(GCGE_CUDA_ERR_ARG, "GetVecFromMultiVec: column outside the multivector");
  }
  *x = &mv->col[j];
}

void cb_RestoreVecForMultiVec(void**, int, void** x, GCGE_CUDA_OPS*) {
  if (x) *x = nullptr;
}

void cb_MultiVecCreateByMat(void*** mv, int n_vec, void* mat, GCGE_CUDA_OPS*) {
  if (!mv) return;
  *mv = nullptr;
  if (failed()) return;
  if (!mat) return fail(GCGE_CUDA_ERR_ARG, "MultiVecCreateByMat: null matrix");
  *mv = reinterpret_cast<void**>(mv_create(n_vec, M_(mat).n));
}

void cb_MultiVecCreateByVec(void*** mv, int n_vec, void* vec, GCGE_CUDA_OPS*) {
  if (!mv) return;
  *mv = nullptr;
  if (failed()) return;
  if (!vec) return fail(GCGE_CUDA_ERR_ARG, "MultiVecCreateByVec: null vector");
  *mv = reinterpret_cast<void**>(mv_create(n_vec, V_(vec)->n));
}

void cb_MultiVecCreateByMultiVec(void*** mv, int n_vec, void** init, GCGE_CUDA_OPS*) {
  if (!mv) return;
  *mv = nullptr;
  if (failed()) return;
  if (!init) return fail(GCGE_CUDA_ERR_ARG, "MultiVecCreateByMultiVec: null multivector");
  *mv = reinterpret_cast<void**>(mv_create(n_vec, MV_(init)->n));
}

void cb_MultiVecDestroy(void*** mv, int, GCGE_CUDA_OPS*) {
  if (!mv || !*mv) return;
  mv_destroy(MV_(*mv));
  *mv = nullptr;
}

void cb_MultiVecSetRandomValue(void** V, int start, int n_vec, GCGE_CUDA_OPS*) {
  if (failed()) return;
  CudaMv* mv = MV_(V);
  if (!range_ok(mv, start, start + n_vec, "MultiVecSetRandomValue")) return;
  for (int j = start; j < start + n_vec; j++) fill_random(mv->col[j].d, mv->n);
}

// y(:, start[1] : start[1] + k) = mat x(:, start[0] : end[0])
void cb_MatDotMultiVec(void* mat, void** x, void** y, int* start, int* end, GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!mat || !start || !end) return fail(GCGE_CUDA_ERR_ARG, "MatDotMultiVec: null argument");
  CudaMv *X = MV_(x), *Y = MV_(y);
  const int k = end[0] - start[0];
  if (!range_ok(X, start[0], end[0], "MatDotMultiVec") ||
      !range_ok(Y, start[1], start[1] + k, "MatDotMultiVec"))
    return;
  for (int c = 0; c < k; c += GCGE_MAXCOLS) {
    const int kk = k - c < GCGE_MAXCOLS ? k - c : GCGE_MAXCOLS;
    gcge::spmm_f64(M_(mat), cols_of(X, start[0] + c, kk), cols_of(Y, start[1] + c, kk), kk, 0);
  }
  launched("MatDotMultiVec");
}

// y(:, start[1] + j) = a x(:, start[0] + j) + b y(:, start[1] + j), j < end[0] - start[0]
void cb_MultiVecAxpby(double a, void** x, double b, void** y, int* start, int* end,
                      GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!start || !end) return fail(GCGE_CUDA_ERR_ARG, "MultiVecAxpby: null range");
  CudaMv *X = MV_(x), *Y = MV_(y);
  const int k = end[0] - start[0];
  if (!range_ok(X, start[0], end[0], "MultiVecAxpby") ||
      !range_ok(Y, start[1], start[1] + k, "MultiVecAxpby"))
    return;
  for (int j = 0; j < k; j++)
    if (b == 0.0 && X->col[start[0] + j].d != Y->col[start[1] + j].d)
      cuda_ok(cudaMemsetAsync(Y->col[start[1] + j].d, 0, sizeof(double) * Y->n, 0), "MultiVecAxpby");
  for (int c = 0; c < k; c += GCGE_MAXCOLS) {
    const int kk = k - c < GCGE_MAXCOLS ? k - c : GCGE_MAXCOLS;
    gcge::axpby_f64(a, cols_of(X, start[0] + c, kk), b, cols_of(Y, start[1] + c, kk), kk, Y->n, 0);
  }
  launched("MultiVecAxpby");
}

void cb_MultiVecAxpbyColumn(double a, void** x, int col_x, double b, void** y, int col_y,
                            GCGE_CUDA_OPS* ops) {
  int s[2] = {col_x, col_y}, e[2] = {col_x + 1, col_y + 1};
  cb_MultiVecAxpby(a, x, b, y, s, e, ops);
}

void cb_MultiVecSwap(void** V1, void** V2, int* start, int* end, GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!start || !end) return fail(GCGE_CUDA_ERR_ARG, "MultiVecSwap: null range");
  CudaMv *A = MV_(V1), *B = MV_(V2);
  const int k = end[0] - start[0];
  if (!range_ok(A, start[0], end[0], "MultiVecSwap") ||
      !range_ok(B, start[1], start[1] + k, "MultiVecSwap"))
    return;
  for (int j = 0; j < k; j++) std::swap(A->col[start[0] + j].d, B->col[start[1] + j].d);
}

}  // namespace

namespace {

// y(:, start[1] + j) = alpha sum_i x(:, start[0] + i) a[j lda + i] + beta y(:, start[1] + j)
// (src/gcge_ops.h:109-111); if_Vec: y[0] is one vector handle (the SLEPc app's
// reading, app/slepc/gcge_app_slepc.c:215-251)
void cb_MultiVecLinearComb(void** x, void** y, int* start, int* end, double* a, int lda,
                           int if_Vec, double alpha, double beta, GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!x || !y || !start || !end || !a) return fail(GCGE_CUDA_ERR_ARG, "MultiVecLinearComb: null argument");
  CudaMv* X = MV_(x);
  const int k1 = end[0] - start[0];
  const int k2 = if_Vec ? 1 : end[1] - start[1];
  if (!range_ok(X, start[0], end[0], "MultiVecLinearComb")) return;
  ColList<double> Yc;
  if (if_Vec) {
    if (!y[0]) return fail(GCGE_CUDA_ERR_ARG, "MultiVecLinearComb: null vector");
    Yc.p[0] = V_(y[0])->d;
  } else {
    if (!range_ok(MV_(y), start[1], end[1], "MultiVecLinearComb")) return;
    Yc = cols_of(MV_(y), start[1], k2);
  }
  if (k2 <= 0) return;
  if (k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || lda < k1)
    return fail(GCGE_CUDA_ERR_ARG, "MultiVecLinearComb: block wider than 256 columns");
  const int n = X->n;
  std::lock_guard<std::mutex> lk(g_ops_mu);
  // coefficients (alpha folded in) and, when y shares a buffer with x, a
  // temporary block for the result
  bool alias = false;
  for (int j = 0; j < k2 && !alias; j++)
    for (int i = 0; i < k1; i++)
      if (X->col[start[0] + i].d == Yc.p[j]) alias = true;
  const size_t need = (size_t)k1 * k2 + (alias ? (size_t)k2 * n : 0) + 1;
  double* buf = ops_scratch(need);
  if (!buf) return;
  std::vector<double> h((size_t)(k1 > 0 ? k1 : 1) * k2);
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) h[i + (size_t)j * k1] = alpha * a[i + (size_t)j * lda];
  if (k1 > 0 && !cuda_ok(cudaMemcpy(buf, h.data(), sizeof(double) * k1 * k2, cudaMemcpyHostToDevice),
                         "MultiVecLinearComb"))
    return;
  ColList<double> Out = Yc;
  if (alias)
    for (int j = 0; j < k2; j++) Out.p[j] = buf + (size_t)k1 * k2 + (size_t)j * n;
  if (beta == 0.0 || alias)
    for (int j = 0; j < k2; j++)
      if (!cuda_ok(cudaMemsetAsync(Out.p[j], 0, sizeof(double) * n, 0), "MultiVecLinearComb")) return;
  gcge::lincomb_f64(cols_of(X, start[0], k1), k1, buf, k1, Out, k2, alias ? 0.0 : beta, n, 0);
  if (!launched("MultiVecLinearComb")) return;
  if (alias) {  // y = out + beta y
    gcge::axpby_f64(beta, Yc, 0.0, Yc, k2, n, 0);
    gcge::axpby_f64(1.0, Out, 1.0, Yc, k2, n, 0);
    launched("MultiVecLinearComb");
  }
}

// a[(w - start[1]) lda + (v - start[0])] = V(:, v) . W(:, w); "sym" keeps the
// upper triangle (v - start[0] <= w - start[1]) and mirrors it into the lower
// (src/gcge_ops.c:226-309); if_Vec: W[0] is one vector handle
void cb_MultiVecInnerProd(void** V, void** W, double* a, char* is_sym, int* start, int* end,
                          int lda, int if_Vec, GCGE_CUDA_OPS*) {
  if (failed()) return;
  if (!V || !W || !a || !start || !end) return fail(GCGE_CUDA_ERR_ARG, "MultiVecInnerProd: null argument");
  CudaMv* Vm = MV_(V);
  const int k1 = end[0] - start[0];
  const int k2 = if_Vec ? 1 : end[1] - start[1];
  if (!range_ok(Vm, start[0], end[0], "MultiVecInnerProd")) return;
  ColList<double> Wc;
  if (if_Vec) {
    if (!W[0]) return fail(GCGE_CUDA_ERR_ARG, "MultiVecInnerProd: null vector");
    Wc.p[0] = V_(W[0])->d;
  } else {
    if (!range_ok(MV_(W), start[1], end[1], "MultiVecInnerProd")) return;
    Wc = cols_of(MV_(W), start[1], k2);
  }
  if (k1 <= 0 || k2 <= 0) return;
  if (k1 > GCGE_MAXCOLS || k2 > GCGE_MAXCOLS || lda < k1)
    return fail(GCGE_CUDA_ERR_ARG, "MultiVecInnerProd: block wider than 256 columns");
  std::lock_guard<std::mutex> lk(g_ops_mu);
  const int tiles = ((k1 + 63) / 64) * ((k2 + 63) / 64);
  const size_t part = (size_t)gcge::kRowBlocks * tiles * 64 * 64;
  double* buf = ops_scratch(part + (size_t)k1 * k2);
  if (!buf) return;
  gcge::gram_f64(cols_of(Vm, start[0], k1), k1, Wc, k2, Vm->n, buf + part, k1, false, buf, 0);
  if (!launched("MultiVecInnerProd")) return;
  std::vector<double> h((size_t)k1 * k2);
  if (!cuda_ok(cudaMemcpy(h.data(), buf + part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost),
               "MultiVecInnerProd"))
    return;
  const bool sym = is_sym && strcmp(is_sym, "sym") == 0;
  for (int j = 0; j < k2; j++)
    for (int i = 0; i < k1; i++) {
      const bool upper = i <= j;
      a[i + (size_t)j * lda] = (!sym || upper) ? h[i + (size_t)j * k1] : h[j + (size_t)i * k1];
    }
}

// Eigenpairs il..iu (1-based) of the upper triangle of a, on the device
// (DenseMatEigenSolver, src/gcge_ops.h:134-137; the default is LAPACK dsyevx,
// or dsyev for the full range, src/gcge_ops.c:401-553).  For the full range
// the default copies dsyev's eigenvectors from a (leading dimension lda) with
// one memcpy of nrows * nrows values; the same values land in a and evec here.
void cb_DenseMatEigenSolver(double* a, int lda, int nrows, double* eval, double* evec, int lde,
                            int il, int iu, int*, double*) {
  if (failed()) return;
  const bool full = (il == 1 && iu == nrows);
  const int m = iu - il + 1;
  std::vector<double> vec((size_t)nrows * (m > 0 ? m : 1));
  const int rc = GCGE_CUDA_DenseMatEigenSolver(a, lda, nrows, eval, vec.data(), nrows, il, iu);
  if (rc != GCGE_CUDA_OK) return fail(rc, "DenseMatEigenSolver: the device eigensolver failed");
  if (full) {
    for (int j = 0; j < nrows; j++)
      for (int i = 0; i < nrows; i++) a[i + (size_t)j * lda] = vec[i + (size_t)j * nrows];
    memcpy(evec, a, sizeof(double) * nrows * nrows);
  } else {
    for (int j = 0; j < m; j++)
      for (int i = 0; i < nrows; i++) evec[i + (size_t)j * lde] = vec[i + (size_t)j * nrows];
  }
}

void cb_MultiVecPrint(void** x, int n, GCGE_CUDA_OPS*) {
  CudaMv* mv = MV_(x);
  if (!mv) return;
  std::vector<double> h(mv->n);
  for (int j = 0; j < n && j < mv->k; j++) {
    if (!cuda_ok(cudaMemcpy(h.data(), mv->col[j].d, sizeof(double) * mv->n, cudaMemcpyDeviceToHost),
                 "MultiVecPrint"))
      return;
    for (int i = 0; i < mv->n; i++) printf("%e\n", h[i]);
  }
}

}  // namespace

extern "C" int GCGE_CUDA_SetOps(void* ops_) {
  if (!ops_) return gcge_record_error(GCGE_CUDA_ERR_ARG, "GCGE_CUDA_SetOps: null table");
  GCGE_CUDA_OPS* ops = static_cast<GCGE_CUDA_OPS*>(ops_);
  ops->VecCreateByVec = cb_VecCreateByVec;
  ops->VecCreateByMat = cb_VecCreateByMat;
  ops->VecDestroy = cb_VecDestroy;
  ops->VecSetRandomValue = cb_VecSetRandomValue;
  ops->MatDotVec = cb_MatDotVec;
  ops->VecAxpby = cb_VecAxpby;
  ops->VecInnerProd = cb_VecInnerProd;
  ops->VecLocalInnerProd = cb_VecInnerProd;  // one GPU: local = global
  ops->GetVecFromMultiVec = cb_GetVecFromMultiVec;
  ops->RestoreVecForMultiVec = cb_RestoreVecForMultiVec;
  ops->MultiVecCreateByVec = cb_MultiVecCreateByVec;
  ops->MultiVecCreateByMat = cb_MultiVecCreateByMat;
  ops->MultiVecCreateByMultiVec = cb_MultiVecCreateByMultiVec;
  ops->MultiVecDestroy = cb_MultiVecDestroy;
  ops->MultiVecSetRandomValue = cb_MultiVecSetRandomValue;
  ops->MatDotMultiVec = cb_MatDotMultiVec;
  ops->MultiVecAxpby = cb_MultiVecAxpby;
  ops->MultiVecAxpbyColumn = cb_MultiVecAxpbyColumn;
  ops->MultiVecLinearComb = cb_MultiVecLinearComb;
  ops->MultiVecInnerProd = cb_MultiVecInnerProd;
  ops->MultiVecInnerProdLocal = cb_MultiVecInnerProd;
  ops->MultiVecSwap = cb_MultiVecSwap;
  ops->MultiVecPrint = cb_MultiVecPrint;
  ops->DenseMatEigenSolver = cb_DenseMatEigenSolver;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MultiVecCreate(void*** multi_vec, int n_vec, const GCGE_CUDA_MAT* A) {
  if (!multi_vec || !A || n_vec < 0)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "MultiVecCreate: bad arguments");
  const int before = g_ops_err;
  CudaMv* mv = mv_create(n_vec, A->m.n);
  *multi_vec = reinterpret_cast<void**>(mv);
  if (!mv) {
    const int code = g_ops_err;
    g_ops_err = before;
    return code != GCGE_CUDA_OK ? code : GCGE_CUDA_ERR_ALLOC;
  }
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MultiVecDestroy(void*** multi_vec) {
  if (!multi_vec) return gcge_record_error(GCGE_CUDA_ERR_ARG, "MultiVecDestroy: null");
  mv_destroy(MV_(*multi_vec));
  *multi_vec = nullptr;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MultiVecSetFromHost(void** multi_vec, int start, int k, const double* h,
                                             int ldh) {
  CudaMv* mv = MV_(multi_vec);
  if (!mv || !h || start < 0 || k < 0 || start + k > mv->k || ldh < mv->n)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "MultiVecSetFromHost: bad arguments");
  for (int j = 0; j < k; j++)
    if (cudaMemcpy(mv->col[start + j].d, h + (size_t)j * ldh, sizeof(double) * mv->n,
                   cudaMemcpyHostToDevice) != cudaSuccess)
      return gcge_record_error(GCGE_CUDA_ERR_CUDA, "MultiVecSetFromHost: copy failed");
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MultiVecGetToHost(void** multi_vec, int start, int k, double* h, int ldh) {
  CudaMv* mv = MV_(multi_vec);
  if (!mv || !h || start < 0 || k < 0 || start + k > mv->k || ldh < mv->n)
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "MultiVecGetToHost: bad arguments");
  for (int j = 0; j < k; j++)
    if (cudaMemcpy(h + (size_t)j * ldh, mv->col[start + j].d, sizeof(double) * mv->n,
                   cudaMemcpyDeviceToHost) != cudaSuccess)
      return gcge_record_error(GCGE_CUDA_ERR_CUDA, "MultiVecGetToHost: copy failed");
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_OpsGetError(void) { return g_ops_err; }
extern "C" void GCGE_CUDA_OpsClearError(void) { g_ops_err = GCGE_CUDA_OK; }
