// hyc_ens_util.cu -- data movement and diagnostics of the ensemble form:
// conversion between the reference layout and the ensemble layout, and the
// FP64 tracer-content sums.
#include <cuda_runtime.h>

#include <cstdint>

#include "hyc_device.cuh"
#include "hyc_ens.h"

namespace hyc {

// ---------------------------------------------------------------------------
// grid table of the strip kernel's diffusion epilogue: row r holds, per
// cell, temdf2*aspux*scuy of row r-4 (0 where iu = 0) and temdf2*aspvy*scvx
// of row r-3 (0 where iv = 0), as in tsdff_2x (mod_tsadvc.F90:2274-2287),
// rounded to FP32; rows before the grid and the padding columns are 0
// ---------------------------------------------------------------------------
__global__ void diff_table_kernel(const double *aspux, const double *aspvy, const double *scuy, const double *scvx,
                                  const uint8_t *msk, double temdf2, int ld1r, int ld1, int ld2, float2 *out) {
  const long long n = (long long)ld1 * ld2;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(t / ld1), i = (int)(t - (long long)r * ld1);
    float au = 0.f, av = 0.f;
    if (i < ld1r) {
      const int ru = r - 4, rv = r - 3;
      if (ru >= 0 && (msk[i + (long long)ru * ld1] & kIU)) {
        const long long o = i + (long long)ru * ld1r;
        au = (float)(temdf2 * aspux[o] * scuy[o]);
      }
      if (rv >= 0 && (msk[i + (long long)rv * ld1] & kIV)) {
        const long long o = i + (long long)rv * ld1r;
        av = (float)(temdf2 * aspvy[o] * scvx[o]);
      }
    }
    out[t] = make_float2(au, av);
  }
}

cudaError_t launch_diff_table(const double *aspux, const double *aspvy, const double *scuy, const double *scvx,
                              const uint8_t *msk, double temdf2, int ld1r, int ld1, int ld2, float2 *out,
                              cudaStream_t s) {
  const long long n = (long long)ld1 * ld2;
  int bx = (int)((n + 255) / 256);
  if (bx > 2048) bx = 2048;
  diff_table_kernel<<<bx, 256, 0, s>>>(aspux, aspvy, scuy, scvx, msk, temdf2, ld1r, ld1, ld2, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// format conversion between the reference layout (FP64, pitch ld1) and the
// ensemble layout (FP32 or FP64, pitch ld1p), nslices slices
// ---------------------------------------------------------------------------
template <class S, class D>
__global__ void repitch_kernel(const S *src, long long spitch, long long sslice, D *dst, long long dpitch,
                               long long dslice, int w, int h) {
  const long long n = (long long)w * h;
  const S *s = src + blockIdx.y * sslice;
  D *d = dst + blockIdx.y * dslice;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / w), i = (int)(t - (long long)j * w);
    d[i + j * dpitch] = (D)s[i + j * spitch];
  }
}

cudaError_t launch_repitch(const void *src, int src_fp32, long long spitch, long long sslice, void *dst, int dst_fp32,
                           long long dpitch, long long dslice, int w, int h, int nslices, cudaStream_t s) {
  long long n = (long long)w * h;
  int bx = (int)((n + 255) / 256);
  if (bx > 2048) bx = 2048;
  for (int z0 = 0; z0 < nslices; z0 += 65535) {
    int nz = nslices - z0 < 65535 ? nslices - z0 : 65535;
    dim3 g(bx, nz);
    if (src_fp32 && dst_fp32)
      repitch_kernel<float, float><<<g, 256, 0, s>>>((const float *)src + z0 * sslice, spitch, sslice,
                                                    (float *)dst + z0 * dslice, dpitch, dslice, w, h);
    else if (src_fp32)
      repitch_kernel<float, double><<<g, 256, 0, s>>>((const float *)src + z0 * sslice, spitch, sslice,
                                                     (double *)dst + z0 * dslice, dpitch, dslice, w, h);
    else if (dst_fp32)
      repitch_kernel<double, float><<<g, 256, 0, s>>>((const double *)src + z0 * sslice, spitch, sslice,
                                                     (float *)dst + z0 * dslice, dpitch, dslice, w, h);
    else
      repitch_kernel<double, double><<<g, 256, 0, s>>>((const double *)src + z0 * sslice, spitch, sslice,
                                                      (double *)dst + z0 * dslice, dpitch, dslice, w, h);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// tracer content of one FP32 or FP64 slice set, FP64 two-sum compensated:
//   sum over interior sea cells of fld * (fc + onemu) * scp2, where fc is
//   fco (old level: from dp and the continuity divergence) or fcn = max(dp,0)
// one CTA per (slice); partials per CTA, summed on the host in order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void acc2(double &hi, double &lo, double x) {
  const double s = hi + x;
  const double bb = s - hi;
  lo += (hi - (s - bb)) + (x - bb);
  hi = s;
}

template <class T, class F>
__global__ void content_kernel(const T *fld, const F *uflx, const F *vflx, const double *dp, const double *scp2,
                               const double *scp2i, const uint8_t *msk, int ii, int jj, int nb, int ld1,
                               long long slice, int use_fco, double dt2, double *partial) {
  const int k = blockIdx.x;
  const T *f = fld + k * slice;
  const F *u = uflx + k * slice, *v = vflx + k * slice;
  const double *d = dp + k * slice;
  double hi = 0.0, lo = 0.0;
  const long long n = (long long)ii * jj;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    const int j = (int)(t / ii), i = (int)(t - (long long)j * ii);
    const long long o = (long long)(i + nb) + (long long)(j + nb) * ld1;
    if (!(msk[o] & kIP)) continue;
    double fc;
    if (use_fco) {
      const double fdv = (((double)u[o + 1] - (double)u[o]) + ((double)v[o + ld1] - (double)v[o])) * dt2 * scp2i[o];
      fc = fmax(d[o] + fdv, 0.0);
    } else {
      fc = fmax(d[o], 0.0);
    }
    acc2(hi, lo, (double)f[o] * (fc + kOnemu) * scp2[o]);
  }
  __shared__ double sh[256], sl[256];
  sh[threadIdx.x] = hi;
  sl[threadIdx.x] = lo;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double h2 = sh[threadIdx.x], l2 = sl[threadIdx.x];
      acc2(h2, l2, sh[threadIdx.x + w]);
      sh[threadIdx.x] = h2;
      sl[threadIdx.x] = l2 + sl[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * k] = sh[0];
    partial[2 * k + 1] = sl[0];
  }
}

cudaError_t launch_content(const void *fld, int fld_fp32, const void *uflx, const void *vflx, int flx_fp32,
                           const double *dp, const double *scp2, const double *scp2i, const uint8_t *msk, int ii,
                           int jj, int nb, int ld1, long long slice, int kdm, int use_fco, double dt2,
                           double *partial, cudaStream_t s) {
  if (fld_fp32 && flx_fp32)
    content_kernel<float, float><<<kdm, 256, 0, s>>>((const float *)fld, (const float *)uflx, (const float *)vflx, dp,
                                                     scp2, scp2i, msk, ii, jj, nb, ld1, slice, use_fco, dt2, partial);
  else
    content_kernel<double, double><<<kdm, 256, 0, s>>>((const double *)fld, (const double *)uflx,
                                                       (const double *)vflx, dp, scp2, scp2i, msk, ii, jj, nb, ld1,
                                                       slice, use_fco, dt2, partial);
  return cudaGetLastError();
}

}  // namespace hyc
