// fdf_io.cu -- the reference's on-disk formats (host code): the FDFGRID grid file and the
// PETSc binary Vec files its field and swarm writers produce, so that a run of this library
// can start from the reference's grid files and exchange particle fields with its restart
// and post-processing tools.
//
//   FDFGRID (io.c:101-170 ReadGridFile, grid.c:356-383 AssignGridCoordinates): text; an
//   optional "FDFGRID" line, the number of blocks, one "IM JM KM" line per block (cells), then
//   the node coordinates "x y z", one node per line, i fastest, then j, then k.  One block
//   (the first) is read and written.
//   PETSc binary Vec (VecView on one rank, as WriteFieldData io.c:653-700 calls it): the
//   header {VEC_FILE_CLASSID = 1211214, N} as PetscInt, then N PetscScalar values, all
//   big-endian; PetscInt is 8 bytes in a build with 64-bit indices (the reference's own,
//   PETSc 3.19.2-64bit) and 4 otherwise.  A Vec with block size bs > 1 also gets the companion
//   "<file>.info" holding "-vecload_block_size <bs>".
#include "fdf_context.cuh"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr long long VEC_FILE_CLASSID = 1211214;

void put_be(std::vector<unsigned char> &out, unsigned long long v, int bytes) {
  for (int q = bytes - 1; q >= 0; --q) out.push_back((unsigned char)((v >> (8 * q)) & 0xFF));
}

unsigned long long get_be(const unsigned char *p, int bytes) {
  unsigned long long v = 0;
  for (int q = 0; q < bytes; ++q) v = (v << 8) | p[q];
  return v;
}

// block size of a real swarm field (0: not one)
int field_bs(const char *field) {
  if (!strcmp(field, "position") || !strcmp(field, "velocity") || !strcmp(field, "weight")) return 3;
  if (!strcmp(field, "P")) return 1;
  return 0;
}

}  // namespace

extern "C" {

int fdf_WritePetscVec(const char *path, const double *values, int64_t n, int bs, int int64_indices) {
  if (!path || (n > 0 && !values)) return FDF_ERR_ARG_NULL;
  if (n < 0 || bs < 1 || n % bs != 0) return FDF_ERR_ARG_OUTOFRANGE;
  const int ib = int64_indices ? 8 : 4;
  if (!int64_indices && n > 0x7fffffffLL) return FDF_ERR_ARG_OUTOFRANGE;
  FILE *f = fopen(path, "wb");
  if (!f) return FDF_ERR_LIB;
  std::vector<unsigned char> buf;
  buf.reserve(2 * ib);
  put_be(buf, (unsigned long long)VEC_FILE_CLASSID, ib);
  put_be(buf, (unsigned long long)n, ib);
  bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
  const size_t chunk = 1 << 16;
  std::vector<unsigned char> out(chunk * 8);
  for (long long p = 0; ok && p < n; p += (long long)chunk) {
    const long long m = (n - p) < (long long)chunk ? (n - p) : (long long)chunk;
    for (long long q = 0; q < m; ++q) {
      unsigned long long u;
      memcpy(&u, values + p + q, 8);
      for (int b = 0; b < 8; ++b) out[8 * q + b] = (unsigned char)((u >> (8 * (7 - b))) & 0xFF);
    }
    ok = fwrite(out.data(), 1, (size_t)(8 * m), f) == (size_t)(8 * m);
  }
  ok = (fclose(f) == 0) && ok;
  if (!ok) return FDF_ERR_LIB;
  if (bs > 1) {
    const std::string info = std::string(path) + ".info";
    FILE *fi = fopen(info.c_str(), "w");
    if (!fi) return FDF_ERR_LIB;
    const bool ok2 = fprintf(fi, "-vecload_block_size %d\n", bs) > 0;
    if ((fclose(fi) != 0) || !ok2) return FDF_ERR_LIB;
  }
  return FDF_SUCCESS;
}

int fdf_ReadPetscVec(const char *path, double *values, int64_t n_max, int64_t *n, int int64_indices) {
  if (!path || !n) return FDF_ERR_ARG_NULL;
  const int ib = int64_indices ? 8 : 4;
  FILE *f = fopen(path, "rb");
  if (!f) return FDF_ERR_LIB;
  unsigned char hdr[16];
  if (fread(hdr, 1, (size_t)(2 * ib), f) != (size_t)(2 * ib)) { fclose(f); return FDF_ERR_LIB; }
  const unsigned long long cls = get_be(hdr, ib), len = get_be(hdr + ib, ib);
  if ((long long)cls != VEC_FILE_CLASSID) { fclose(f); return FDF_ERR_ARG_WRONG; }   // not a Vec (or other index width)
  *n = (int64_t)len;
  if (!values) { fclose(f); return FDF_SUCCESS; }
  if ((long long)len > n_max) { fclose(f); return FDF_ERR_ARG_OUTOFRANGE; }
  const size_t chunk = 1 << 16;
  std::vector<unsigned char> in(chunk * 8);
  for (unsigned long long p = 0; p < len; p += chunk) {
    const unsigned long long m = (len - p) < chunk ? (len - p) : chunk;
    if (fread(in.data(), 1, (size_t)(8 * m), f) != (size_t)(8 * m)) { fclose(f); return FDF_ERR_LIB; }
    for (unsigned long long q = 0; q < m; ++q) {
      const unsigned long long u = get_be(in.data() + 8 * q, 8);
      memcpy(values + p + q, &u, 8);
    }
  }
  fclose(f);
  return FDF_SUCCESS;
}

int fdf_ReadGridFile(const char *path, int64_t *IM, int64_t *JM, int64_t *KM, double *coor, int64_t coor_len) {
  if (!path || !IM || !JM || !KM) return FDF_ERR_ARG_NULL;
  FILE *f = fopen(path, "r");
  if (!f) return FDF_ERR_LIB;
  char tok[64] = {0};
  long long nblk = 0;
  int rc = FDF_SUCCESS;
  if (fscanf(f, "%63s", tok) != 1) rc = FDF_ERR_LIB;
  if (rc == FDF_SUCCESS) {
    if (!strcmp(tok, "FDFGRID")) {
      if (fscanf(f, "%lld", &nblk) != 1) rc = FDF_ERR_LIB;
    } else {
      nblk = strtoll(tok, nullptr, 10);
    }
  }
  if (nblk == 0) nblk = 1;
  long long dims[3] = {0, 0, 0};
  for (long long b = 0; rc == FDF_SUCCESS && b < nblk; ++b) {
    long long d[3];
    if (fscanf(f, "%lld %lld %lld", &d[0], &d[1], &d[2]) != 3) rc = FDF_ERR_LIB;
    if (b == 0) memcpy(dims, d, sizeof(dims));
  }
  if (rc == FDF_SUCCESS && (dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)) rc = FDF_ERR_ARG_OUTOFRANGE;
  if (rc != FDF_SUCCESS) { fclose(f); return rc; }
  *IM = dims[0]; *JM = dims[1]; *KM = dims[2];
  if (!coor) { fclose(f); return FDF_SUCCESS; }
  const long long nn = (dims[0] + 1) * (dims[1] + 1) * (dims[2] + 1);
  if (3 * nn > coor_len) { fclose(f); return FDF_ERR_ARG_OUTOFRANGE; }
  for (long long q = 0; q < nn; ++q)
    if (fscanf(f, "%le %le %le", &coor[3 * q], &coor[3 * q + 1], &coor[3 * q + 2]) != 3) { fclose(f); return FDF_ERR_LIB; }
  fclose(f);
  return FDF_SUCCESS;
}

int fdf_WriteGridFile(const char *path, int64_t IM, int64_t JM, int64_t KM, const double *coor) {
  if (!path || !coor) return FDF_ERR_ARG_NULL;
  if (IM <= 0 || JM <= 0 || KM <= 0) return FDF_ERR_ARG_OUTOFRANGE;
  FILE *f = fopen(path, "w");
  if (!f) return FDF_ERR_LIB;
  bool ok = fprintf(f, "FDFGRID\n1\n%lld %lld %lld\n", (long long)IM, (long long)JM, (long long)KM) > 0;
  const long long nn = (IM + 1) * (JM + 1) * (KM + 1);
  for (long long q = 0; ok && q < nn; ++q)   // 17 significant digits: the doubles read back exactly
    ok = fprintf(f, "%.17e %.17e %.17e\n", coor[3 * q], coor[3 * q + 1], coor[3 * q + 2]) > 0;
  ok = (fclose(f) == 0) && ok;
  return ok ? FDF_SUCCESS : FDF_ERR_LIB;
}

int fdf_WriteSwarmField(FdfContext *ctx, const char *field, const char *path, int int64_indices) {
  if (!ctx || !field || !path) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_WriteSwarmField: null argument");
  const int bs = field_bs(field);
  if (!bs) return fail(ctx, FDF_ERR_ARG_WRONG, std::string("fdf_WriteSwarmField: not a real swarm field: ") + field);
  int64_t n = 0;
  int r = fdf_GetSwarmSize(ctx, &n);
  if (r) return r;
  std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), w(3 * (size_t)n), P((size_t)n);
  std::vector<int64_t> cell(3 * (size_t)n), pid((size_t)n), st((size_t)n);
  int64_t got = 0;
  r = fdf_GetSwarm(ctx, n, &got, pos.data(), vel.data(), w.data(), P.data(), cell.data(), pid.data(), st.data());
  if (r) return r;
  const double *src = !strcmp(field, "position") ? pos.data() : !strcmp(field, "velocity") ? vel.data()
                    : !strcmp(field, "weight") ? w.data() : P.data();
  r = fdf_WritePetscVec(path, src, got * bs, bs, int64_indices);
  return r ? fail(ctx, r, std::string("fdf_WriteSwarmField: cannot write ") + path) : FDF_SUCCESS;
}

int fdf_ReadSwarmField(FdfContext *ctx, const char *field, const char *path, int int64_indices) {
  if (!ctx || !field || !path) return fail(ctx, FDF_ERR_ARG_NULL, "fdf_ReadSwarmField: null argument");
  const int bs = field_bs(field);
  if (!bs) return fail(ctx, FDF_ERR_ARG_WRONG, std::string("fdf_ReadSwarmField: not a real swarm field: ") + field);
  int64_t n = 0;
  int r = fdf_GetSwarmSize(ctx, &n);
  if (r) return r;
  int64_t len = 0;
  r = fdf_ReadPetscVec(path, nullptr, 0, &len, int64_indices);
  if (r) return fail(ctx, r, std::string("fdf_ReadSwarmField: cannot read ") + path);
  if (len != n * bs)
    return fail(ctx, FDF_ERR_ARG_OUTOFRANGE, "fdf_ReadSwarmField: the file's length does not match the swarm");
  std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), w(3 * (size_t)n), P((size_t)n);
  std::vector<int64_t> cell(3 * (size_t)n), pid((size_t)n), st((size_t)n);
  int64_t got = 0;
  r = fdf_GetSwarm(ctx, n, &got, pos.data(), vel.data(), w.data(), P.data(), cell.data(), pid.data(), st.data());
  if (r) return r;
  double *dst = !strcmp(field, "position") ? pos.data() : !strcmp(field, "velocity") ? vel.data()
              : !strcmp(field, "weight") ? w.data() : P.data();
  r = fdf_ReadPetscVec(path, dst, n * bs, &len, int64_indices);
  if (r) return fail(ctx, r, std::string("fdf_ReadSwarmField: cannot read ") + path);
  const int form = ctx->form;   // the swarm stays in the form it is held in
  ctx->form = ctx->swarm_form;
  r = fdf_SetSwarm(ctx, n, pos.data(), vel.data(), w.data(), P.data(), cell.data(), pid.data(), st.data());
  ctx->form = form;
  return r;
}

}  // extern "C"
