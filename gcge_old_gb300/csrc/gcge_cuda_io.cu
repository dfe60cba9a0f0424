// CSR matrix files on the host: the reference's text format and PETSc's binary
// Mat format, read into and written from GCGE_CUDA_CSR_HOST.
//
// Text (CSR_ReadMatFile, app/csr/gcge_app_csr.c:185-236): whitespace-separated
// nrow, ncol, nnz, then rowptr[nrow+1], col[nnz], val[nnz], 0-based.  The
// reader takes the whole file into memory and parses it on all host threads:
// the body is cut into byte ranges at whitespace, each thread counts its
// tokens, a prefix sum gives every token its global index, and each thread then
// converts its tokens straight into rowptr / col / val.  Values go through
// strtod (correctly rounded), so a file written with 17 significant digits
// reads back bit-exact.
//
// Binary (PETSc MatLoad / MatView format, the reference's PETSc app reads
// test/data/*.petsc.bin with it): big-endian int32 classid 1211216, rows,
// columns, nnz, row lengths[rows], col[nnz], then big-endian float64 val[nnz].
// 32-bit indices only.  Byte order is handled byte by byte, independent of the
// host's own.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gcge_cuda.h"

int gcge_record_error(int code, const char* msg);

namespace {

constexpr int32_t kPetscMatClassId = 1211216;

int io_err(const char* path, const char* what) {
  std::string m = std::string(path ? path : "(null)") + ": " + what;
  return gcge_record_error(GCGE_CUDA_ERR_IO, m.c_str());
}

// The whole file plus a terminating NUL (strtod stops there): one allocation of
// the file's size, one read.
struct FileBuf {
  char* p = nullptr;
  size_t size = 0;
  ~FileBuf() { free(p); }
};

bool read_all(const char* path, FileBuf* out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  bool ok = fseek(f, 0, SEEK_END) == 0;
  const long len = ok ? ftell(f) : -1;
  ok = ok && len >= 0 && fseek(f, 0, SEEK_SET) == 0;
  if (ok) {
    out->p = (char*)malloc((size_t)len + 1);
    ok = out->p && fread(out->p, 1, (size_t)len, f) == (size_t)len;
    if (ok) {
      out->p[len] = '\0';
      out->size = (size_t)len;
    }
  }
  fclose(f);
  return ok;
}

inline bool is_ws(char c) {
  return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f';
}

int host_threads(size_t bytes) {
  const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
  const size_t by_size = std::max<size_t>(1, bytes >> 20);  // about 1 MiB a thread at least
  return (int)std::min<size_t>({(size_t)hc, by_size, (size_t)64});
}

// Parses one int32 token [p, e); false on anything else.
bool parse_int(const char* p, const char* e, int* v) {
  bool neg = false;
  if (p < e && (*p == '+' || *p == '-')) neg = (*p++ == '-');
  if (p == e) return false;
  int64_t x = 0;
  for (; p < e; p++) {
    if (*p < '0' || *p > '9') return false;
    x = x * 10 + (*p - '0');
    if (x > (int64_t)INT32_MAX + 1) return false;
  }
  x = neg ? -x : x;
  if (x > INT32_MAX || x < INT32_MIN) return false;
  *v = (int)x;
  return true;
}

bool parse_double(const char* p, const char* e, double* v) {
  char* end = nullptr;
  errno = 0;
  const double x = strtod(p, &end);
  if (end != e) return false;
  if (errno == ERANGE && (x == HUGE_VAL || x == -HUGE_VAL)) return false;
  *v = x;
  return true;
}

// Next token at or after *p (before e): sets [*b, *t) and moves *p past it.
bool next_token(const char** p, const char* e, const char** b, const char** t) {
  const char* q = *p;
  while (q < e && is_ws(*q)) q++;
  if (q == e) return false;
  const char* s = q;
  while (q < e && !is_ws(*q)) q++;
  *b = s;
  *t = q;
  *p = q;
  return true;
}

bool alloc_csr(GCGE_CUDA_CSR_HOST* c, int nrow, int ncol, int nnz) {
  c->N_Rows = nrow;
  c->N_Columns = ncol;
  c->N_Entries = nnz;
  c->RowPtr = (int*)malloc(sizeof(int) * ((size_t)nrow + 1));
  c->KCol = (int*)malloc(sizeof(int) * std::max<size_t>(1, (size_t)nnz));
  c->Entries = (double*)malloc(sizeof(double) * std::max<size_t>(1, (size_t)nnz));
  if (c->RowPtr && c->KCol && c->Entries) return true;
  GCGE_CUDA_CSR_Free(c);
  return false;
}

// Row pointers from 0 to nnz without decrease, columns in [0, ncol).
const char* check_csr(const GCGE_CUDA_CSR_HOST* c) {
  if (c->RowPtr[0] != 0) return "row pointers must start at 0";
  for (int i = 0; i < c->N_Rows; i++)
    if (c->RowPtr[i + 1] < c->RowPtr[i]) return "row pointers decrease";
  if (c->RowPtr[c->N_Rows] != c->N_Entries) return "last row pointer differs from nnz";
  for (int e = 0; e < c->N_Entries; e++)
    if (c->KCol[e] < 0 || c->KCol[e] >= c->N_Columns) return "column index out of range";
  return nullptr;
}

int read_text(const char* path, const FileBuf& d, GCGE_CUDA_CSR_HOST* out) {
  const char* p = d.p;
  const char* end = d.p + d.size;
  int hdr[3];
  for (int i = 0; i < 3; i++) {
    const char *b, *t;
    if (!next_token(&p, end, &b, &t) || !parse_int(b, t, &hdr[i]) || hdr[i] < 0)
      return io_err(path, "bad header (expected nrow, ncol, nnz)");
  }
  const int nrow = hdr[0], ncol = hdr[1], nnz = hdr[2];
  const size_t n_rp = (size_t)nrow + 1, total = n_rp + 2 * (size_t)nnz;
  GCGE_CUDA_CSR_HOST c{};
  if (!alloc_csr(&c, nrow, ncol, nnz))
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "host allocation for the CSR file failed");

  // byte ranges cut at whitespace, so no token straddles two ranges
  const size_t body = (size_t)(end - p);
  const int nt = host_threads(body);
  std::vector<const char*> cut(nt + 1);
  cut[0] = p;
  cut[nt] = end;
  for (int i = 1; i < nt; i++) {
    const char* q = p + body * i / nt;
    q = std::max(q, cut[i - 1]);
    while (q < end && !is_ws(*q)) q++;
    cut[i] = q;
  }
  std::vector<size_t> count(nt + 1, 0);
  auto run = [&](auto fn) {
    std::vector<std::thread> th;
    for (int i = 1; i < nt; i++) th.emplace_back(fn, i);
    fn(0);
    for (auto& t : th) t.join();
  };
  run([&](int i) {
    const char* q = cut[i];
    const char *b, *t;
    size_t k = 0;
    while (next_token(&q, cut[i + 1], &b, &t)) k++;
    count[i + 1] = k;
  });
  for (int i = 0; i < nt; i++) count[i + 1] += count[i];
  if (count[nt] < total) {
    GCGE_CUDA_CSR_Free(&c);
    return io_err(path, "file ends before rowptr, col and val are complete");
  }
  // tokens past the last value are ignored, as fscanf-based readers ignore them
  std::vector<size_t> bad(nt, SIZE_MAX);
  run([&](int i) {
    const char* q = cut[i];
    const char *b, *t;
    for (size_t g = count[i]; g < std::min(count[i + 1], total); g++) {
      next_token(&q, cut[i + 1], &b, &t);
      bool ok;
      if (g < n_rp) {
        ok = parse_int(b, t, &c.RowPtr[g]);
      } else if (g < n_rp + (size_t)nnz) {
        ok = parse_int(b, t, &c.KCol[g - n_rp]);
      } else {
        ok = parse_double(b, t, &c.Entries[g - n_rp - nnz]);
      }
      if (!ok) {
        bad[i] = g;
        return;
      }
    }
  });
  for (int i = 0; i < nt; i++)
    if (bad[i] != SIZE_MAX) {
      GCGE_CUDA_CSR_Free(&c);
      const size_t g = bad[i];
      const char* sec = g < n_rp ? "rowptr" : (g < n_rp + (size_t)nnz ? "col" : "val");
      std::string m = std::string("malformed number in ") + sec + " (token " +
                      std::to_string(g + 3) + ")";
      return io_err(path, m.c_str());
    }
  if (const char* why = check_csr(&c)) {
    GCGE_CUDA_CSR_Free(&c);
    return io_err(path, why);
  }
  *out = c;
  return GCGE_CUDA_OK;
}

inline uint32_t be32(const unsigned char* b) {
  return ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
}
inline uint64_t be64(const unsigned char* b) {
  return ((uint64_t)be32(b) << 32) | (uint64_t)be32(b + 4);
}
inline void put32(unsigned char* b, uint32_t v) {
  b[0] = (unsigned char)(v >> 24);
  b[1] = (unsigned char)(v >> 16);
  b[2] = (unsigned char)(v >> 8);
  b[3] = (unsigned char)v;
}
inline void put64(unsigned char* b, uint64_t v) {
  put32(b, (uint32_t)(v >> 32));
  put32(b + 4, (uint32_t)v);
}

int read_petsc(const char* path, const FileBuf& d, GCGE_CUDA_CSR_HOST* out) {
  const size_t size = d.size;
  const unsigned char* u = reinterpret_cast<const unsigned char*>(d.p);
  if (size < 16) return io_err(path, "binary header truncated");
  const int32_t m = (int32_t)be32(u + 4), n = (int32_t)be32(u + 8), nz = (int32_t)be32(u + 12);
  if (m < 0 || n < 0 || nz < 0) return io_err(path, "negative size in the binary header");
  const size_t need = 16 + 4 * (size_t)m + 12 * (size_t)nz;
  if (size < need) return io_err(path, "binary file ends before row lengths, col and val");
  GCGE_CUDA_CSR_HOST c{};
  if (!alloc_csr(&c, m, n, nz))
    return gcge_record_error(GCGE_CUDA_ERR_ALLOC, "host allocation for the CSR file failed");
  const unsigned char* rl = u + 16;
  const unsigned char* ci = rl + 4 * (size_t)m;
  const unsigned char* va = ci + 4 * (size_t)nz;
  int64_t acc = 0;
  c.RowPtr[0] = 0;
  for (int i = 0; i < m; i++) {
    const int32_t len = (int32_t)be32(rl + 4 * (size_t)i);
    acc += len;
    if (len < 0 || acc > nz) {
      GCGE_CUDA_CSR_Free(&c);
      return io_err(path, "row lengths do not sum to nnz");
    }
    c.RowPtr[i + 1] = (int)acc;
  }
  const int nt = host_threads(12 * (size_t)nz);
  std::vector<std::thread> th;
  auto body = [&](int t) {
    const size_t lo = (size_t)nz * t / nt, hi = (size_t)nz * (t + 1) / nt;
    for (size_t e = lo; e < hi; e++) {
      c.KCol[e] = (int32_t)be32(ci + 4 * e);
      const uint64_t bits = be64(va + 8 * e);
      memcpy(&c.Entries[e], &bits, 8);
    }
  };
  for (int t = 1; t < nt; t++) th.emplace_back(body, t);
  body(0);
  for (auto& t : th) t.join();
  if (const char* why = check_csr(&c)) {
    GCGE_CUDA_CSR_Free(&c);
    return io_err(path, why);
  }
  *out = c;
  return GCGE_CUDA_OK;
}

bool csr_arg_ok(const GCGE_CUDA_CSR_HOST* c) {
  return c && c->N_Rows >= 0 && c->N_Columns >= 0 && c->N_Entries >= 0 && c->RowPtr &&
         (c->N_Entries == 0 || (c->KCol && c->Entries));
}

bool write_all(FILE* f, const std::string& s) { return fwrite(s.data(), 1, s.size(), f) == s.size(); }

}  // namespace

extern "C" int GCGE_CUDA_CSR_ReadFile(const char* path, GCGE_CUDA_CSR_HOST* csr) {
  if (!path || !csr) return gcge_record_error(GCGE_CUDA_ERR_ARG, "CSR_ReadFile: null argument");
  FileBuf d;
  if (!read_all(path, &d)) return io_err(path, "cannot open or read");
  const size_t size = d.size;
  const unsigned char* u = reinterpret_cast<const unsigned char*>(d.p);
  if (size >= 4 && (int32_t)be32(u) == kPetscMatClassId) return read_petsc(path, d, csr);
  return read_text(path, d, csr);
}

extern "C" int GCGE_CUDA_CSR_WriteText(const char* path, const GCGE_CUDA_CSR_HOST* c) {
  if (!path || !csr_arg_ok(c))
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "CSR_WriteText: bad argument");
  if (const char* why = check_csr(c)) return gcge_record_error(GCGE_CUDA_ERR_ARG, why);
  FILE* f = fopen(path, "wb");
  if (!f) return io_err(path, "cannot open for writing");
  const int nrow = c->N_Rows, nnz = c->N_Entries;
  // the three sections formatted in parallel ranges, written in order
  const size_t total = (size_t)nrow + 1 + 2 * (size_t)nnz;
  const int nt = host_threads(total * 12);
  std::vector<std::string> part(nt);
  std::vector<std::thread> th;
  auto body = [&](int t) {
    const size_t lo = total * t / nt, hi = total * (t + 1) / nt;
    std::string& s = part[t];
    s.reserve((hi - lo) * 14);
    char buf[40];
    for (size_t g = lo; g < hi; g++) {
      int len;
      if (g < (size_t)nrow + 1)
        len = snprintf(buf, sizeof(buf), "%d\n", c->RowPtr[g]);
      else if (g < (size_t)nrow + 1 + nnz)
        len = snprintf(buf, sizeof(buf), "%d\n", c->KCol[g - nrow - 1]);
      else
        len = snprintf(buf, sizeof(buf), "%.17g\n", c->Entries[g - nrow - 1 - nnz]);
      s.append(buf, (size_t)len);
    }
  };
  for (int t = 1; t < nt; t++) th.emplace_back(body, t);
  body(0);
  for (auto& t : th) t.join();
  char hdr[64];
  snprintf(hdr, sizeof(hdr), "%d\n%d\n%d\n", nrow, c->N_Columns, nnz);
  bool ok = write_all(f, hdr);
  for (int t = 0; t < nt && ok; t++) ok = write_all(f, part[t]);
  ok = (fclose(f) == 0) && ok;
  return ok ? GCGE_CUDA_OK : io_err(path, "write failed");
}

extern "C" int GCGE_CUDA_CSR_WriteBinary(const char* path, const GCGE_CUDA_CSR_HOST* c) {
  if (!path || !csr_arg_ok(c))
    return gcge_record_error(GCGE_CUDA_ERR_ARG, "CSR_WriteBinary: bad argument");
  if (const char* why = check_csr(c)) return gcge_record_error(GCGE_CUDA_ERR_ARG, why);
  const int m = c->N_Rows, nz = c->N_Entries;
  std::vector<unsigned char> b(16 + 4 * (size_t)m + 12 * (size_t)nz);
  put32(&b[0], (uint32_t)kPetscMatClassId);
  put32(&b[4], (uint32_t)m);
  put32(&b[8], (uint32_t)c->N_Columns);
  put32(&b[12], (uint32_t)nz);
  unsigned char* rl = b.data() + 16;
  unsigned char* ci = rl + 4 * (size_t)m;
  unsigned char* va = ci + 4 * (size_t)nz;
  for (int i = 0; i < m; i++) put32(rl + 4 * (size_t)i, (uint32_t)(c->RowPtr[i + 1] - c->RowPtr[i]));
  for (size_t e = 0; e < (size_t)nz; e++) {
    put32(ci + 4 * e, (uint32_t)c->KCol[e]);
    uint64_t bits;
    memcpy(&bits, &c->Entries[e], 8);
    put64(va + 8 * e, bits);
  }
  FILE* f = fopen(path, "wb");
  if (!f) return io_err(path, "cannot open for writing");
  bool ok = fwrite(b.data(), 1, b.size(), f) == b.size();
  ok = (fclose(f) == 0) && ok;
  return ok ? GCGE_CUDA_OK : io_err(path, "write failed");
}

extern "C" int GCGE_CUDA_CSR_Free(GCGE_CUDA_CSR_HOST* c) {
  if (!c) return GCGE_CUDA_ERR_ARG;
  free(c->RowPtr);
  free(c->KCol);
  free(c->Entries);
  c->RowPtr = nullptr;
  c->KCol = nullptr;
  c->Entries = nullptr;
  c->N_Rows = c->N_Columns = c->N_Entries = 0;
  return GCGE_CUDA_OK;
}

extern "C" int GCGE_CUDA_MatCreateFromFile(GCGE_CUDA_MAT** mat, const char* path) {
  if (!mat) return gcge_record_error(GCGE_CUDA_ERR_ARG, "MatCreateFromFile: null argument");
  GCGE_CUDA_CSR_HOST c{};
  int rc = GCGE_CUDA_CSR_ReadFile(path, &c);
  if (rc) return rc;
  rc = GCGE_CUDA_MatCreateFromCSR(mat, &c);
  GCGE_CUDA_CSR_Free(&c);
  return rc;
}
