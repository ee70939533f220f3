// Restart files in the reference's .ic format (host only): the binary image
// ReadIc reads (src/read_ic.c:3-39) and PrintInit writes
// (src/print.c:213-330) -- per element an ic_struct of five doubles
// (cmc, sneqv, surf, unsat, gw; src/include/elem_struct.h:731-749 without
// _FBR_/_NOAH_), then per river segment a river_ic_struct of two (stage, gw;
// src/include/river_struct.h:71-75), native byte order.
#include <cstdio>
#include <vector>

#include "pihm_gpu.h"

extern "C" {

int pihm_ic_write(const char *path, int32_t nelem, int32_t nriver, const double *y, const double *cmc,
                  const double *sneqv) {
  if (!path || !y || nelem <= 0 || nriver < 0) return PIHM_GPU_ERR_ARG;
  std::vector<double> buf(5 * (size_t)nelem + 2 * (size_t)nriver);
  for (int32_t i = 0; i < nelem; i++) {
    double *r = &buf[5 * (size_t)i];
    r[0] = cmc ? cmc[i] : 0.0;
    r[1] = sneqv ? sneqv[i] : 0.0;
    r[2] = y[i];
    r[3] = y[nelem + i];
    r[4] = y[2 * (size_t)nelem + i];
  }
  double *rv = &buf[5 * (size_t)nelem];
  for (int32_t s = 0; s < nriver; s++) {
    rv[2 * s] = y[3 * (size_t)nelem + s];
    rv[2 * s + 1] = y[3 * (size_t)nelem + nriver + s];
  }
  FILE *f = std::fopen(path, "wb");
  if (!f) return PIHM_GPU_ERR_ARG;
  const size_t n = std::fwrite(buf.data(), sizeof(double), buf.size(), f);
  const int closed = std::fclose(f);
  return (n == buf.size() && closed == 0) ? PIHM_GPU_OK : PIHM_GPU_ERR_ARG;
}

int pihm_ic_read(const char *path, int32_t nelem, int32_t nriver, double *y, double *cmc, double *sneqv) {
  if (!path || !y || nelem <= 0 || nriver < 0) return PIHM_GPU_ERR_ARG;
  FILE *f = std::fopen(path, "rb");
  if (!f) return PIHM_GPU_ERR_ARG;
  const size_t want = 5 * (size_t)nelem + 2 * (size_t)nriver;
  // the reference refuses a file whose size does not match (src/read_ic.c:13-24)
  if (std::fseek(f, 0L, SEEK_END) != 0 || std::ftell(f) != (long)(sizeof(double) * want) ||
      std::fseek(f, 0L, SEEK_SET) != 0) {
    std::fclose(f);
    return PIHM_GPU_ERR_MESH;
  }
  std::vector<double> buf(want);
  const size_t n = std::fread(buf.data(), sizeof(double), want, f);
  std::fclose(f);
  if (n != want) return PIHM_GPU_ERR_MESH;
  for (int32_t i = 0; i < nelem; i++) {
    const double *r = &buf[5 * (size_t)i];
    if (cmc) cmc[i] = r[0];
    if (sneqv) sneqv[i] = r[1];
    y[i] = r[2];
    y[nelem + i] = r[3];
    y[2 * (size_t)nelem + i] = r[4];
  }
  const double *rv = &buf[5 * (size_t)nelem];
  for (int32_t s = 0; s < nriver; s++) {
    y[3 * (size_t)nelem + s] = rv[2 * s];
    y[3 * (size_t)nelem + nriver + s] = rv[2 * s + 1];
  }
  return PIHM_GPU_OK;
}

}  // extern "C"
