// hyc_za.cpp -- HYCOM .a/.b field input (mod_za_sm.h:678-770 zaiord,
// :944-965 zaiordd; mod_restart.F90:561-620 restart_in3d), so that fields
// of a real HYCOM run (restart or archive files) can feed the advection
// instead of synthetic ones.
//
// A .a file is a sequence of records of n2drec IEEE real*4 words, big
// endian, with n2drec = idm*jdm rounded up to a multiple of 4096
// (mod_za_sm.h:497-498); record r holds one idm x jdm field, i fastest.
// 2^100 marks data voids.  The matching .b file has one text line per
// record after its header, "cfield  : ... = layer level hmin hmax" for a
// restart file.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdarg>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/hycom_adv.h"
#include "hyc_internal.h"

namespace {

constexpr float kSpval = 1.2676506002282294e30f;  // 2^100, mod_za_sm.h:725

uint32_t be32(const unsigned char *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
}

int za_fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  hyc::set_library_error(buf);
  return code;
}

}  // namespace

extern "C" {

int hyc_za_read(const char *path, int32_t idm, int32_t jdm, int32_t nbdy, int32_t record, const int32_t *mask,
                double *h, int32_t where, double *hmin, double *hmax) {
  if (!path || idm < 1 || jdm < 1 || nbdy < 0 || record < 1 || !h || (where != HYC_HOST && where != HYC_DEVICE))
    return za_fail(HYC_ERR_ARG, "hyc_za_read: bad arguments");
  const long long n = (long long)idm * jdm;
  const long long n2drec = (n + 4095) / 4096 * 4096;
  FILE *f = fopen(path, "rb");
  if (!f) return za_fail(HYC_ERR_ARG, "hyc_za_read: cannot open %s: %s", path, strerror(errno));
  std::vector<unsigned char> raw((size_t)n * 4);
  const long long off = (long long)(record - 1) * n2drec * 4;
  bool ok = fseeko(f, (off_t)off, SEEK_SET) == 0 && fread(raw.data(), 1, raw.size(), f) == raw.size();
  fclose(f);
  if (!ok) return za_fail(HYC_ERR_ARG, "hyc_za_read: cannot read record %d of %s", record, path);
  const int ld1 = idm + 2 * nbdy;
  const long long slice = (long long)ld1 * (jdm + 2 * nbdy);
  // zaiord (mod_za_sm.h:744-769): masked points only, or every point with
  // data voids left out of the range
  std::vector<double> w((size_t)n);
  double lo = (double)kSpval, hi = -(double)kSpval;
  for (long long t = 0; t < n; t++) {
    const uint32_t u = be32(&raw[(size_t)t * 4]);
    float v;
    memcpy(&v, &u, 4);
    w[(size_t)t] = (double)v;
    const int i = (int)(t % idm), j = (int)(t / idm);
    const long long o = (long long)(i + nbdy) + (long long)(j + nbdy) * ld1;
    if (mask) {
      if (mask[o] != 0) {
        lo = std::fmin(lo, (double)v);
        hi = std::fmax(hi, (double)v);
      }
    } else if (v != kSpval) {
      lo = std::fmin(lo, (double)v);
      hi = std::fmax(hi, (double)v);
    }
  }
  if (mask && hi == (double)kSpval)  // mod_za_sm.h:772-780
    return za_fail(HYC_ERR_ARG, "hyc_za_read: record %d of %s has 2.0**100 inside the mask", record, path);
  // store into the interior of h (masked: sea points only)
  std::vector<double> host;
  double *dst = h;
  if (where == HYC_DEVICE) {
    host.assign((size_t)slice, 0.0);
    if (mask) {  // keep the unmasked points of the device array
      cudaError_t e = cudaMemcpy(host.data(), h, (size_t)slice * 8, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return za_fail(HYC_ERR_CUDA, "hyc_za_read: %s", cudaGetErrorString(e));
    }
    dst = host.data();
  }
  for (int j = 0; j < jdm; j++)
    for (int i = 0; i < idm; i++) {
      const long long o = (long long)(i + nbdy) + (long long)(j + nbdy) * ld1;
      if (!mask || mask[o] != 0) dst[o] = w[(size_t)i + (size_t)j * idm];
    }
  if (where == HYC_DEVICE) {
    cudaError_t e = cudaMemcpy2D(h + nbdy + (long long)nbdy * ld1, (size_t)ld1 * 8, host.data() + nbdy +
                                 (long long)nbdy * ld1, (size_t)ld1 * 8, (size_t)idm * 8, (size_t)jdm,
                                 cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return za_fail(HYC_ERR_CUDA, "hyc_za_read: %s", cudaGetErrorString(e));
  }
  if (hmin) *hmin = lo;
  if (hmax) *hmax = hi;
  return HYC_OK;
}

int hyc_za_parse_b(const char *line, char *cfield, int32_t *layer, int32_t *level, double *hmin, double *hmax) {
  if (!line) return za_fail(HYC_ERR_ARG, "hyc_za_parse_b: null line");
  const char *eq = strchr(line, '=');
  if (!eq) return za_fail(HYC_ERR_ARG, "hyc_za_parse_b: no '=' in \"%s\"", line);
  if (cfield) {  // the first 8 characters name the field (restart_in3d, mod_restart.F90:594)
    size_t k = 0;
    for (; k < 8 && line[k] && line[k] != '\n'; k++) cfield[k] = line[k];
    for (; k < 8; k++) cfield[k] = ' ';
    cfield[8] = '\0';
  }
  char *end = nullptr;
  const char *p = eq + 1;
  const long lay = strtol(p, &end, 10);
  if (end == p) return za_fail(HYC_ERR_ARG, "hyc_za_parse_b: no layer in \"%s\"", line);
  p = end;
  const long lev = strtol(p, &end, 10);
  if (end == p) return za_fail(HYC_ERR_ARG, "hyc_za_parse_b: no level in \"%s\"", line);
  p = end;
  const double a = strtod(p, &end);
  if (end == p) return za_fail(HYC_ERR_ARG, "hyc_za_parse_b: no minimum in \"%s\"", line);
  p = end;
  const double b = strtod(p, &end);
  if (end == p) return za_fail(HYC_ERR_ARG, "hyc_za_parse_b: no maximum in \"%s\"", line);
  if (layer) *layer = (int32_t)lay;
  if (level) *level = (int32_t)lev;
  if (hmin) *hmin = a;
  if (hmax) *hmax = b;
  return HYC_OK;
}

int hyc_za_check(double hmin_a, double hmax_a, double hmin_b, double hmax_b) {
  // restart_in3d (mod_restart.F90:604-605): 1e-4 relative agreement
  if (std::fabs(hmin_a - hmin_b) > std::fabs(hmin_b) * 1.e-4 || std::fabs(hmax_a - hmax_b) > std::fabs(hmax_b) * 1.e-4)
    return za_fail(HYC_ERR_ARG, "range of the .a field (%g, %g) disagrees with the .b line (%g, %g)", hmin_a, hmax_a,
                   hmin_b, hmax_b);
  return HYC_OK;
}

}  // extern "C"
