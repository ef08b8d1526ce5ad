// petscbin.cu -- PETSc binary files (host code): the format VecView / MatView
// write to a binary viewer and VecLoad / MatLoad read (c/ch12/obstacle.c:138-144
// dumps u and the obstacle this way; c/ch2/loadsolve.c loads A and b), so that
// solutions of this library can be compared with dumps of the reference.
//
// Format (big-endian throughout): a Vec is int32 classid 1211214, int32 n,
// n float64; an AIJ Mat is int32 classid 1211216, int32 M, N, nz, M int32
// row lengths, nz int32 column indices, nz float64 values.  Objects follow
// one another in a file.  Vectors of a DMDA are written in natural ordering,
// which for one process is the x-fastest order used here.
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "../../include/fishgpu.h"

namespace {

constexpr int32_t VEC_CLASSID = 1211214;
constexpr int32_t MAT_CLASSID = 1211216;

void put32(unsigned char *p, uint32_t v) {
  p[0] = (unsigned char)(v >> 24);
  p[1] = (unsigned char)(v >> 16);
  p[2] = (unsigned char)(v >> 8);
  p[3] = (unsigned char)v;
}

uint32_t get32(const unsigned char *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

void put64(unsigned char *p, double d) {
  uint64_t v;
  memcpy(&v, &d, 8);
  for (int k = 0; k < 8; k++) p[k] = (unsigned char)(v >> (56 - 8 * k));
}

double get64(const unsigned char *p) {
  uint64_t v = 0;
  for (int k = 0; k < 8; k++) v = (v << 8) | p[k];
  double d;
  memcpy(&d, &v, 8);
  return d;
}

bool write_ints(FILE *f, const int32_t *a, long long n) {
  std::vector<unsigned char> buf(4 * 4096);
  for (long long k = 0; k < n;) {
    const long long c = n - k < 4096 ? n - k : 4096;
    for (long long q = 0; q < c; q++) put32(&buf[4 * q], (uint32_t)a[k + q]);
    if (fwrite(buf.data(), 4, (size_t)c, f) != (size_t)c) return false;
    k += c;
  }
  return true;
}

bool write_doubles(FILE *f, const double *a, long long n) {
  std::vector<unsigned char> buf(8 * 4096);
  for (long long k = 0; k < n;) {
    const long long c = n - k < 4096 ? n - k : 4096;
    for (long long q = 0; q < c; q++) put64(&buf[8 * q], a[k + q]);
    if (fwrite(buf.data(), 8, (size_t)c, f) != (size_t)c) return false;
    k += c;
  }
  return true;
}

bool read_ints(FILE *f, int32_t *a, long long n) {
  std::vector<unsigned char> buf(4 * 4096);
  for (long long k = 0; k < n;) {
    const long long c = n - k < 4096 ? n - k : 4096;
    if (fread(buf.data(), 4, (size_t)c, f) != (size_t)c) return false;
    for (long long q = 0; q < c; q++) a[k + q] = (int32_t)get32(&buf[4 * q]);
    k += c;
  }
  return true;
}

bool read_doubles(FILE *f, double *a, long long n) {
  std::vector<unsigned char> buf(8 * 4096);
  for (long long k = 0; k < n;) {
    const long long c = n - k < 4096 ? n - k : 4096;
    if (fread(buf.data(), 8, (size_t)c, f) != (size_t)c) return false;
    for (long long q = 0; q < c; q++) a[k + q] = get64(&buf[8 * q]);
    k += c;
  }
  return true;
}

bool skip(FILE *f, long long bytes) { return fseek(f, (long)bytes, SEEK_CUR) == 0; }

// Advances past one object (Vec or AIJ Mat); *cls receives its classid.
bool skip_object(FILE *f, int32_t *cls) {
  int32_t h[1];
  if (!read_ints(f, h, 1)) return false;
  *cls = h[0];
  if (h[0] == VEC_CLASSID) {
    int32_t n;
    return read_ints(f, &n, 1) && n >= 0 && skip(f, 8LL * n);
  }
  if (h[0] == MAT_CLASSID) {
    int32_t d[3];
    return read_ints(f, d, 3) && d[0] >= 0 && d[2] >= 0 && skip(f, 4LL * d[0] + 12LL * d[2]);
  }
  return false;
}

}  // namespace

extern "C" int fishgpu_petsc_vec_write(const char *path, int append, const double *x, long long n) {
  if (!path || n < 0 || n > 0x7fffffffLL || (n > 0 && !x)) return FISHGPU_ERR_ARG;
  FILE *f = fopen(path, append ? "ab" : "wb");
  if (!f) return FISHGPU_ERR_ARG;
  const int32_t h[2] = {VEC_CLASSID, (int32_t)n};
  const bool ok = write_ints(f, h, 2) && write_doubles(f, x, n);
  return (fclose(f) == 0 && ok) ? FISHGPU_OK : FISHGPU_ERR_ARG;
}

// Reads the `index`-th object of the file, which must be a Vec; *n receives its
// length; at most `cap` values are stored (x may be NULL to query the length).
extern "C" int fishgpu_petsc_vec_read(const char *path, int index, double *x, long long cap, long long *n) {
  if (!path || index < 0 || !n) return FISHGPU_ERR_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return FISHGPU_ERR_ARG;
  int rc = FISHGPU_OK;
  int32_t cls = 0;
  for (int k = 0; k < index && rc == FISHGPU_OK; k++)
    if (!skip_object(f, &cls)) rc = FISHGPU_ERR_ARG;
  int32_t h[2];
  if (rc == FISHGPU_OK && (!read_ints(f, h, 2) || h[0] != VEC_CLASSID || h[1] < 0)) rc = FISHGPU_ERR_ARG;
  if (rc == FISHGPU_OK) {
    *n = h[1];
    if (x) {
      if (cap < h[1]) rc = FISHGPU_ERR_ARG;
      else if (!read_doubles(f, x, h[1])) rc = FISHGPU_ERR_ARG;
    }
  }
  fclose(f);
  return rc;
}

extern "C" int fishgpu_petsc_mat_write_aij(const char *path, int append, int M, int N, const long long *rowptr,
                                           const int *col, const double *val) {
  if (!path || M < 0 || N < 0 || !rowptr) return FISHGPU_ERR_ARG;
  const long long nz = rowptr[M] - rowptr[0];
  if (nz < 0 || nz > 0x7fffffffLL || (nz > 0 && (!col || !val))) return FISHGPU_ERR_ARG;
  std::vector<int32_t> len((size_t)M);
  for (int r = 0; r < M; r++) {
    const long long l = rowptr[r + 1] - rowptr[r];
    if (l < 0) return FISHGPU_ERR_ARG;
    len[r] = (int32_t)l;
  }
  for (long long k = 0; k < nz; k++)
    if (col[rowptr[0] + k] < 0 || col[rowptr[0] + k] >= N) return FISHGPU_ERR_ARG;
  FILE *f = fopen(path, append ? "ab" : "wb");
  if (!f) return FISHGPU_ERR_ARG;
  const int32_t h[4] = {MAT_CLASSID, M, N, (int32_t)nz};
  bool ok = write_ints(f, h, 4) && write_ints(f, len.data(), M);
  ok = ok && write_ints(f, (const int32_t *)(col + rowptr[0]), nz) && write_doubles(f, val + rowptr[0], nz);
  return (fclose(f) == 0 && ok) ? FISHGPU_OK : FISHGPU_ERR_ARG;
}

// Reads the `index`-th object, which must be an AIJ Mat: first call with
// col/val NULL to get M, N, nz; then with rowptr (M+1), col (nz), val (nz).
extern "C" int fishgpu_petsc_mat_read_aij(const char *path, int index, int *M, int *N, long long *nz,
                                          long long *rowptr, int *col, double *val) {
  if (!path || index < 0 || !M || !N || !nz) return FISHGPU_ERR_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return FISHGPU_ERR_ARG;
  int rc = FISHGPU_OK;
  int32_t cls = 0;
  for (int k = 0; k < index && rc == FISHGPU_OK; k++)
    if (!skip_object(f, &cls)) rc = FISHGPU_ERR_ARG;
  int32_t h[4];
  if (rc == FISHGPU_OK && (!read_ints(f, h, 4) || h[0] != MAT_CLASSID || h[1] < 0 || h[2] < 0 || h[3] < 0))
    rc = FISHGPU_ERR_ARG;
  if (rc == FISHGPU_OK) {
    *M = h[1];
    *N = h[2];
    *nz = h[3];
    if (rowptr && col && val) {
      std::vector<int32_t> len((size_t)h[1]);
      if (!read_ints(f, len.data(), h[1])) rc = FISHGPU_ERR_ARG;
      rowptr[0] = 0;
      for (int r = 0; r < h[1] && rc == FISHGPU_OK; r++) rowptr[r + 1] = rowptr[r] + len[r];
      if (rc == FISHGPU_OK && rowptr[h[1]] != h[3]) rc = FISHGPU_ERR_ARG;
      if (rc == FISHGPU_OK && (!read_ints(f, (int32_t *)col, h[3]) || !read_doubles(f, val, h[3])))
        rc = FISHGPU_ERR_ARG;
    }
  }
  fclose(f);
  return rc;
}
