// ati_io.cpp — the reference's on-disk formats over the public C ABI:
// restart files (wrRsta / rdRsta, src/rpt.f90:555-668) and Plot3D multi-block
// grid and solution files (wrP3dG / wrP3dS, src/rpt.f90:115-330).  Host code
// only; every array comes from or goes to the device through ati_get_* /
// ati_set_*, so the files are independent of the precision mode.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ati.h"

// error text of a handle (ati_last_error), set from outside ati_api.cu
void ati_set_handle_error(ati_handle_t *h, const char *msg);

namespace {

struct File {
  FILE *f = nullptr;
  explicit File(const char *path, const char *mode) { f = std::fopen(path, mode); }
  ~File() {
    if (f) std::fclose(f);
  }
};

int io_fail(ati_handle_t *h, const std::string &msg) {
  ati_set_handle_error(h, msg.c_str());
  return ATI_EINVAL;
}

bool put(FILE *f, const void *p, size_t bytes) { return std::fwrite(p, 1, bytes, f) == bytes; }
bool get(FILE *f, void *p, size_t bytes) { return std::fread(p, 1, bytes, f) == bytes; }

// 8-byte header slot holding an int32 in its first 4 bytes (MPI_INTEGER4 written at a REAL8-extent offset)
bool put_i4_slot(FILE *f, int64_t v) {
  unsigned char slot[8] = {0};
  const int32_t i = (int32_t)v;
  std::memcpy(slot, &i, 4);
  return put(f, slot, 8);
}

// blocks of the handle (all cases of a batch) and the case of a block
int nblocks(ati_handle_t *h) {
  int nc = 0, b0 = 0, nb = 0;
  if (ati_case_count(h, &nc) != ATI_OK || ati_case_blocks(h, nc - 1, &b0, &nb) != ATI_OK) return -1;
  return b0 + nb;
}
int block_case(ati_handle_t *h, int blk) {
  int nc = 0;
  if (ati_case_count(h, &nc) != ATI_OK) return -1;
  for (int c = 0; c < nc; c++) {
    int b0 = 0, nb = 0;
    if (ati_case_blocks(h, c, &b0, &nb) != ATI_OK) return -1;
    if (blk >= b0 && blk < b0 + nb) return c;
  }
  return -1;
}

}  // namespace

extern "C" int ati_write_restart(ati_handle_t *h, int blk, const char *path) {
  if (!h || !path) return io_fail(h, "ati_write_restart: bad argument");
  int32_t dims[3];
  int64_t npts = 0;
  int rc = ati_block_dims(h, blk, dims, &npts);
  if (rc) return rc;
  ati_time_t t;
  if ((rc = ati_case_time(h, block_case(h, blk), &t))) return rc;
  std::vector<double> q((size_t)5 * npts);
  if ((rc = ati_get_state(h, blk, q.data()))) return rc;
  File fl(path, "wb");
  if (!fl.f) return io_fail(h, std::string("ati_write_restart: cannot open ") + path);
  const double hd[4] = {t.dt, t.dts, t.dte, t.timo};
  if (!put_i4_slot(fl.f, t.n) || !put_i4_slot(fl.f, t.ndt) || !put(fl.f, hd, sizeof(hd)) ||
      !put(fl.f, q.data(), sizeof(double) * q.size()))
    return io_fail(h, std::string("ati_write_restart: write failed on ") + path);
  return ATI_OK;
}

extern "C" int ati_read_restart(ati_handle_t *h, int blk, const char *path) {
  if (!h || !path) return io_fail(h, "ati_read_restart: bad argument");
  int32_t dims[3];
  int64_t npts = 0;
  int rc = ati_block_dims(h, blk, dims, &npts);
  if (rc) return rc;
  File fl(path, "rb");
  if (!fl.f) return io_fail(h, std::string("ati_read_restart: cannot open ") + path);
  unsigned char s0[8], s1[8];
  double hd[4];
  std::vector<double> q((size_t)5 * npts);
  if (!get(fl.f, s0, 8) || !get(fl.f, s1, 8) || !get(fl.f, hd, sizeof(hd)) ||
      !get(fl.f, q.data(), sizeof(double) * q.size()))
    return io_fail(h, std::string("ati_read_restart: ") + path + " is shorter than 48 + 40 x " +
                   std::to_string(npts) + " bytes");
  int32_t n, ndt;
  std::memcpy(&n, s0, 4);
  std::memcpy(&ndt, s1, 4);
  ati_time_t t;
  t.n = n; t.ndt = ndt; t.dt = hd[0]; t.dts = hd[1]; t.dte = hd[2]; t.timo = hd[3];
  if ((rc = ati_set_state(h, blk, q.data()))) return rc;
  return ati_case_set_time(h, block_case(h, blk), &t);
}

extern "C" int ati_write_plot3d_grid(ati_handle_t *h, const char *path) {
  if (!h || !path) return io_fail(h, "ati_write_plot3d_grid: bad argument");
  const int nb = nblocks(h);
  if (nb < 0) return ATI_EINVAL;
  File fl(path, "wb");
  if (!fl.f) return io_fail(h, std::string("ati_write_plot3d_grid: cannot open ") + path);
  std::vector<int32_t> hdr{nb};
  std::vector<int64_t> np(nb);
  for (int b = 0; b < nb; b++) {
    int32_t d[3];
    int rc = ati_block_dims(h, b, d, &np[b]);
    if (rc) return rc;
    hdr.push_back(d[0] + 1); hdr.push_back(d[1] + 1); hdr.push_back(d[2] + 1);
  }
  if (!put(fl.f, hdr.data(), sizeof(int32_t) * hdr.size())) return io_fail(h, "ati_write_plot3d_grid: write failed");
  for (int b = 0; b < nb; b++) {
    std::vector<double> xyz((size_t)3 * np[b]);
    int rc = ati_get_field(h, b, ATI_F_SS, xyz.data());  // the grid coordinates kept from ati_set_grid
    if (rc) return rc;
    std::vector<float> x4(xyz.begin(), xyz.end());
    if (!put(fl.f, x4.data(), sizeof(float) * x4.size())) return io_fail(h, "ati_write_plot3d_grid: write failed");
  }
  return ATI_OK;
}

extern "C" int ati_write_plot3d_solution(ati_handle_t *h, const char *path) {
  if (!h || !path) return io_fail(h, "ati_write_plot3d_solution: bad argument");
  const int nb = nblocks(h);
  if (nb < 0) return ATI_EINVAL;
  int rc = 0;
  File fl(path, "wb");
  if (!fl.f) return io_fail(h, std::string("ati_write_plot3d_solution: cannot open ") + path);
  std::vector<int32_t> hdr{nb};
  std::vector<int64_t> np(nb);
  for (int b = 0; b < nb; b++) {
    int32_t d[3];
    if ((rc = ati_block_dims(h, b, d, &np[b]))) return rc;
    hdr.push_back(d[0] + 1); hdr.push_back(d[1] + 1); hdr.push_back(d[2] + 1);
  }
  if (!put(fl.f, hdr.data(), sizeof(int32_t) * hdr.size())) return io_fail(h, "ati_write_plot3d_solution: write failed");
  for (int b = 0; b < nb; b++) {
    // Mach, AoA, Re and time of the block's case
    const int cs = block_case(h, b);
    ati_config_t cfg;
    ati_time_t t;
    double umf[3], aoa;
    if ((rc = ati_case_config(h, cs, &cfg)) || (rc = ati_case_time(h, cs, &t)) || (rc = ati_case_frame(h, cs, umf, &aoa)))
      return rc;
    const double mach = std::sqrt(cfg.amach1 * cfg.amach1 + cfg.amach2 * cfg.amach2 + cfg.amach3 * cfg.amach3);
    const int64_t n = np[b];
    std::vector<double> q((size_t)5 * n), p((size_t)n);
    if ((rc = ati_get_state(h, b, q.data()))) return rc;
    if ((rc = ati_get_field(h, b, ATI_F_P, p.data()))) return rc;
    const float head[4] = {(float)mach, (float)aoa, (float)cfg.reoo, (float)t.timo};
    std::vector<float> q4((size_t)5 * n);
    for (int64_t l = 0; l < n; l++) {
      q4[l] = (float)q[l];
      for (int m = 1; m <= 3; m++) q4[m * n + l] = (float)(q[m * n + l] / q[l] + umf[m - 1]);
      q4[4 * n + l] = (float)p[l];
    }
    if (!put(fl.f, head, sizeof(head)) || !put(fl.f, q4.data(), sizeof(float) * q4.size()))
      return io_fail(h, "ati_write_plot3d_solution: write failed");
  }
  return ATI_OK;
}
