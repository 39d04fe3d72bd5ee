// Restart files of the power-iteration block: reference SavePsiFile and
// ReadPsiFile (src/Restart.f90:759-793 and :614-731).  Host code; the file is what the
// reference's Fortran writes with FORM='UNFORMATTED' (sequential access):
// each WRITE is one record framed by its byte length as a 4-byte
// little-endian integer before and after the data (gfortran's default).
// Records, in order:
//   isavi, nev (int32 each) | bounds(2) (f64) | eigv(nev) | delta(nev) |
//   then per vector: ndof, nrk (int32) | nbas(ndof) (int32) | coef(nrk) |
//   base(nD, nrk) (f64, term by term -- the block layout of this library).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/mlcp_gb300.h"
#include "common.cuh"

namespace mlcp {

int finish_status(int status);

namespace {

// Largest record written with one pair of markers; gfortran splits longer
// records into sub-records, which this library neither writes nor reads.
constexpr size_t kMaxRecord = 0x7fffffffu;

bool put_record(FILE* f, const void* data, size_t bytes) {
  if (bytes > kMaxRecord) return false;
  const int32_t m = (int32_t)bytes;
  return fwrite(&m, 4, 1, f) == 1 && (bytes == 0 || fwrite(data, bytes, 1, f) == 1) && fwrite(&m, 4, 1, f) == 1;
}

// Reads the first `bytes` bytes of the next record into dst.  As a Fortran
// READ with an input list, a record longer than the list is accepted and its
// remainder skipped; a shorter one is an error.
bool get_record(FILE* f, void* dst, size_t bytes) {
  int32_t head = 0, tail = 0;
  if (fread(&head, 4, 1, f) != 1 || head < 0 || (size_t)head < bytes) return false;
  if (bytes && fread(dst, bytes, 1, f) != 1) return false;
  if ((size_t)head > bytes && fseek(f, (long)((size_t)head - bytes), SEEK_CUR) != 0) return false;
  return fread(&tail, 4, 1, f) == 1 && tail == head;
}

}  // namespace

int save_psi(const char* path, int isavi, const double* bounds, int nev, const double* eigv, const double* delta,
             int ndof, const int* nbas, const int* ranks, const double* coef, const double* base) {
  if (!path || nev < 0 || ndof < 1) {
    set_error("mlcp_save_psi: bad arguments (nev=%d ndof=%d)", nev, ndof);
    return kBadArgument;
  }
  int nD = 0;
  for (int d = 0; d < ndof; ++d) nD += nbas[d];
  FILE* f = fopen(path, "wb");
  if (!f) {
    set_error("mlcp_save_psi: cannot open %s for writing", path);
    return kBadArgument;
  }
  const int32_t head[2] = {isavi, nev};
  bool ok = put_record(f, head, 8) && put_record(f, bounds, 16) &&
            put_record(f, eigv, 8 * (size_t)nev) && put_record(f, delta, 8 * (size_t)nev);
  size_t t = 0;
  for (int i = 0; ok && i < nev; ++i) {
    const int32_t dims[2] = {ndof, ranks[i]};
    std::vector<int32_t> nb(nbas, nbas + ndof);
    ok = put_record(f, dims, 8) && put_record(f, nb.data(), 4 * (size_t)ndof) &&
         put_record(f, coef + t, 8 * (size_t)ranks[i]) &&
         put_record(f, base + t * nD, 8 * (size_t)ranks[i] * nD);
    t += (size_t)ranks[i];
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) {
    set_error("mlcp_save_psi: write to %s failed", path);
    return kBadArgument;
  }
  return kOk;
}

// As ReadPsiFile: reads everything into temporaries, checks nev and every
// vector's ndof and nbas against the caller's, and only then replaces the
// caller's data.  *success = 0 (and nothing changed) when the file is
// missing, truncated or does not match.
int read_psi(const char* path, int* isavi, double* bounds, int nev, double* eigv, double* delta, int ndof,
             const int* nbas, int max_terms, int* ranks, double* coef, double* base, int* success) {
  *success = 0;
  if (!path || nev < 0 || ndof < 1 || max_terms < 0) {
    set_error("mlcp_read_psi: bad arguments (nev=%d ndof=%d)", nev, ndof);
    return kBadArgument;
  }
  int nD = 0;
  for (int d = 0; d < ndof; ++d) nD += nbas[d];
  FILE* f = fopen(path, "rb");
  if (!f) return kOk;  // not found: success stays 0, as the reference
  int32_t head[2];
  double bt[2];
  std::vector<double> et(nev), dt(nev), ct, bs;
  std::vector<int> rk(nev);
  bool ok = get_record(f, head, 8) && head[1] == nev && get_record(f, bt, 16) &&
            get_record(f, et.data(), 8 * (size_t)nev) && get_record(f, dt.data(), 8 * (size_t)nev);
  size_t terms = 0;
  for (int i = 0; ok && i < nev; ++i) {
    int32_t dims[2];
    ok = get_record(f, dims, 8) && dims[0] == ndof && dims[1] >= 1;
    if (!ok) break;
    std::vector<int32_t> nb(ndof);
    ok = get_record(f, nb.data(), 4 * (size_t)ndof);
    for (int d = 0; ok && d < ndof; ++d) ok = nb[d] == nbas[d];
    if (!ok || terms + (size_t)dims[1] > (size_t)max_terms) {
      ok = false;
      break;
    }
    rk[i] = dims[1];
    ct.resize(terms + dims[1]);
    bs.resize((terms + dims[1]) * nD);
    ok = get_record(f, ct.data() + terms, 8 * (size_t)dims[1]) &&
         get_record(f, bs.data() + terms * nD, 8 * (size_t)dims[1] * nD);
    terms += (size_t)dims[1];
  }
  fclose(f);
  if (!ok) return kOk;
  *isavi = head[0];
  bounds[0] = bt[0];
  bounds[1] = bt[1];
  std::memcpy(eigv, et.data(), sizeof(double) * nev);
  std::memcpy(delta, dt.data(), sizeof(double) * nev);
  std::memcpy(ranks, rk.data(), sizeof(int) * nev);
  std::memcpy(coef, ct.data(), sizeof(double) * terms);
  std::memcpy(base, bs.data(), sizeof(double) * terms * nD);
  *success = 1;
  return kOk;
}

}  // namespace mlcp

extern "C" int mlcp_save_psi(const char* path, int isavi, const double* bounds, int nev, const double* eigv,
                             const double* delta, int ndof, const int* nbas, const int* ranks, const double* coef,
                             const double* base) {
  return mlcp::finish_status(mlcp::save_psi(path, isavi, bounds, nev, eigv, delta, ndof, nbas, ranks, coef, base));
}

extern "C" int mlcp_read_psi(const char* path, int* isavi, double* bounds, int nev, double* eigv, double* delta,
                             int ndof, const int* nbas, int max_terms, int* ranks, double* coef, double* base,
                             int* success) {
  return mlcp::finish_status(
      mlcp::read_psi(path, isavi, bounds, nev, eigv, delta, ndof, nbas, max_terms, ranks, coef, base, success));
}
