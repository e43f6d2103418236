// Restart files: the state writeResult saves and lastConditions reads back
// (subWriteOutput.f90:62-72, subLastConditions.f90:2-42): u, v, w, p over the
// whole padded grid and the counters totime, ita, ita1.
//
// Binary form (this library's own): a 64-byte little-endian header
//   char magic[8] = "IB3DRST1"; int64 nx, ny, nz; double totime; int64 ita, ita1;
//   int64 nfields (= 4)
// followed by u, v, w, p as (nx+2)(ny+2)(nz+2) doubles each in the Fortran layout
// (i fastest). 4 x 77.7 MB at 256x192x192 instead of ~1.9 GB of formatted text.
//
// Text form (the reference's own `result` file): one line per cell, k outer, j,
// i inner, holding "u v w p totime ita ita1" as Fortran list-directed I/O writes and
// reads them. Values are written with 17 significant digits, so a text round trip
// is exact.
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ib3d_internal.cuh"

namespace {

const char kMagic[8] = {'I', 'B', '3', 'D', 'R', 'S', 'T', '1'};

struct Header {
  char magic[8];
  int64_t nx, ny, nz;
  double totime;
  int64_t ita, ita1;
  int64_t nfields;
};
static_assert(sizeof(Header) == 64, "restart header is 64 bytes");

int fail(ib3d_ctx* c, int code, const char* msg) {
  c->err = msg;
  return code;
}

int download4(ib3d_ctx* c, std::vector<double>* f) {
  const size_t n3 = (size_t)c->d.n3;
  const double* src[4] = {c->u, c->v, c->w, c->p};
  for (int q = 0; q < 4; ++q) {
    f[q].resize(n3);
    if (cudaMemcpyAsync(f[q].data(), src[q], n3 * sizeof(double), cudaMemcpyDeviceToHost, c->st) != cudaSuccess)
      return fail(c, IB3D_ERR_CUDA, "restart: device-to-host copy failed");
  }
  if (cudaStreamSynchronize(c->st) != cudaSuccess) return fail(c, IB3D_ERR_CUDA, "restart: stream failed");
  return IB3D_OK;
}

}  // namespace

extern "C" {

int ib3d_write_restart(ib3d_ctx* c, const char* path, double totime, int64_t ita, int64_t ita1) {
  if (!c || !path) return IB3D_ERR_ARG;
  std::vector<double> f[4];
  int rc = download4(c, f);
  if (rc) return rc;
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return fail(c, IB3D_ERR_IO, "ib3d_write_restart: cannot open the file for writing");
  Header h{};
  std::memcpy(h.magic, kMagic, 8);
  h.nx = c->d.nx; h.ny = c->d.ny; h.nz = c->d.nz;
  h.totime = totime; h.ita = ita; h.ita1 = ita1; h.nfields = 4;
  bool ok = std::fwrite(&h, sizeof(h), 1, fp) == 1;
  for (int q = 0; q < 4 && ok; ++q) ok = std::fwrite(f[q].data(), sizeof(double), f[q].size(), fp) == f[q].size();
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? IB3D_OK : fail(c, IB3D_ERR_IO, "ib3d_write_restart: write failed");
}

int ib3d_read_restart(ib3d_ctx* c, const char* path, double* totime, int64_t* ita, int64_t* ita1) {
  if (!c || !path) return IB3D_ERR_ARG;
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return fail(c, IB3D_ERR_IO, "ib3d_read_restart: cannot open the file");
  Header h{};
  if (std::fread(&h, sizeof(h), 1, fp) != 1 || std::memcmp(h.magic, kMagic, 8) != 0 || h.nfields != 4) {
    std::fclose(fp);
    return fail(c, IB3D_ERR_IO, "ib3d_read_restart: not an IB3D restart file");
  }
  if (h.nx != c->d.nx || h.ny != c->d.ny || h.nz != c->d.nz) {
    std::fclose(fp);
    return fail(c, IB3D_ERR_ARG, "ib3d_read_restart: grid size differs from the context's");
  }
  const size_t n3 = (size_t)c->d.n3;
  std::vector<double> f[4];
  bool ok = true;
  for (int q = 0; q < 4 && ok; ++q) {
    f[q].resize(n3);
    ok = std::fread(f[q].data(), sizeof(double), n3, fp) == n3;
  }
  std::fclose(fp);
  if (!ok) return fail(c, IB3D_ERR_IO, "ib3d_read_restart: file is truncated");
  // lastConditions: u, v, w, p from the file and ut = u, vt = v, wt = w (:33-40)
  const int rc = ib3d_upload_fields(c, f[0].data(), f[1].data(), f[2].data(), f[3].data());
  if (rc) return rc;
  if (totime) *totime = h.totime;
  if (ita) *ita = h.ita;
  if (ita1) *ita1 = h.ita1;
  return IB3D_OK;
}

int ib3d_write_result_text(ib3d_ctx* c, const char* path, double totime, int64_t ita, int64_t ita1) {
  if (!c || !path) return IB3D_ERR_ARG;
  std::vector<double> f[4];
  int rc = download4(c, f);
  if (rc) return rc;
  FILE* fp = std::fopen(path, "w");
  if (!fp) return fail(c, IB3D_ERR_IO, "ib3d_write_result_text: cannot open the file for writing");
  bool ok = true;
  const size_t n3 = (size_t)c->d.n3;
  for (size_t q = 0; q < n3 && ok; ++q)   // k outer, i inner: the Fortran layout's own order
    ok = std::fprintf(fp, "%.17g %.17g %.17g %.17g %.17g %" PRId64 " %" PRId64 "\n", f[0][q], f[1][q], f[2][q],
                      f[3][q], totime, ita, ita1) > 0;
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? IB3D_OK : fail(c, IB3D_ERR_IO, "ib3d_write_result_text: write failed");
}

}  // extern "C"

namespace {
// One value of a list-directed record: blanks, tabs and line ends before it, and at
// most one comma among them, separate it from the previous value.
bool read_list_value(FILE* fp, double* out) {
  int ch;
  bool comma = false;
  while ((ch = std::fgetc(fp)) != EOF) {
    if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r') continue;
    if (ch == ',' && !comma) {
      comma = true;
      continue;
    }
    break;
  }
  if (ch == EOF) return false;
  std::ungetc(ch, fp);
  return std::fscanf(fp, "%lf", out) == 1;
}

// The rest of the current line: a list-directed READ that has its values skips what
// is left of the record it stopped in.
void skip_rest_of_record(FILE* fp) {
  int ch;
  while ((ch = std::fgetc(fp)) != EOF && ch != '\n') {
  }
}
}  // namespace

extern "C" {

int ib3d_read_result_text(ib3d_ctx* c, const char* path, double* totime, int64_t* ita, int64_t* ita1) {
  if (!c || !path) return IB3D_ERR_ARG;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return fail(c, IB3D_ERR_IO, "ib3d_read_result_text: cannot open the file");
  const size_t n3 = (size_t)c->d.n3;
  std::vector<double> f[4];
  for (auto& v : f) v.resize(n3);
  double t = 0.0, it = 0.0, it1 = 0.0;
  bool ok = true;
  // list-directed records (READ(1,*) u, v, w, p, totime, ita, ita1 per cell,
  // subLastConditions.f90:24-29): values separated by blanks, a comma or line ends, so
  // a record may continue on the next line; ita, ita1 may be written as integers or
  // reals
  for (size_t q = 0; q < n3 && ok; ++q) {
    double* dst[7] = {&f[0][q], &f[1][q], &f[2][q], &f[3][q], &t, &it, &it1};
    for (int m = 0; m < 7 && ok; ++m) ok = read_list_value(fp, dst[m]);
    if (ok) skip_rest_of_record(fp);
  }
  std::fclose(fp);
  if (!ok) return fail(c, IB3D_ERR_IO, "ib3d_read_result_text: fewer than (nx+2)(ny+2)(nz+2) records of 7 values");
  const int rc = ib3d_upload_fields(c, f[0].data(), f[1].data(), f[2].data(), f[3].data());
  if (rc) return rc;
  if (totime) *totime = t;
  if (ita) *ita = (int64_t)it;
  if (ita1) *ita1 = (int64_t)it1;
  return IB3D_OK;
}

}  // extern "C"
