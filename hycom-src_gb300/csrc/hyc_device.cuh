// hyc_device.cuh -- device-side helpers shared by the advection kernels.
//
// Reference layout (mod_cb_arrays.F90, mod_dimensions.F90): a 2-D slice is
// a(1-nbdy:idm+nbdy, 1-nbdy:jdm+nbdy), column-major.  Fortran (i,j) maps to
// offset (i+nbdy-1) + (j+nbdy-1)*ld1.
//
// Comparisons on the FP64 data run on the integer pipes.  On GB300 the FP64
// pipe issues about 1/72 of the FP32 rate (a DMNMX or DSETP costs as much
// as a DFMA), while 64-bit integer compares and selects run an order of
// magnitude faster, so min/max/sign tests are done on the IEEE bit patterns.
// For non-NaN doubles the map  key(x) = bits(x) ^ ((bits(x) >> 63) >>> 1)
// is strictly increasing in x (with -0 just below +0), so a signed 64-bit
// compare of keys orders doubles.  Results equal the reference's
// max()/min() except possibly in the sign of a zero, which never changes a
// later value of this path (no division by these zeros happens).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace hyc {

constexpr double kOnemu = 9806.e-12;  // 1 micrometre in Pa, mod_tsadvc.F90:236
constexpr double kEpsil = 1.e-10;     // mod_tsadvc.F90:1027

__device__ __forceinline__ long long dkey(double x) {
  long long b = __double_as_longlong(x);
  return b ^ ((long long)((unsigned long long)(b >> 63) >> 1));
}
// max(a,b) / min(a,b) of the reference (mod_tsadvc.F90 passim)
__device__ __forceinline__ double kmax(double a, double b) { return dkey(a) > dkey(b) ? a : b; }
__device__ __forceinline__ double kmin(double a, double b) { return dkey(a) < dkey(b) ? a : b; }
// max(0.0,x) and min(0.0,x)
__device__ __forceinline__ double pos0(double x) { return __double_as_longlong(x) > 0 ? x : 0.0; }
__device__ __forceinline__ double neg0(double x) { return __double_as_longlong(x) < 0 ? x : 0.0; }
// x >= 0.0 (true for -0.0 too), x < 0.0 (false for -0.0), x > 0.0
__device__ __forceinline__ bool ge0(double x) {
  long long b = __double_as_longlong(x);
  return b >= 0 || b == (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool lt0(double x) {
  long long b = __double_as_longlong(x);
  return b < 0 && b != (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool gt0(double x) { return __double_as_longlong(x) > 0; }
__device__ __forceinline__ bool klt(double a, double b) { return dkey(a) < dkey(b); }

// FP32 versions (FMNMX is cheap on the FP32 pipe)
__device__ __forceinline__ float kmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float kmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float pos0(float x) { return fmaxf(x, 0.0f); }
__device__ __forceinline__ float neg0(float x) { return fminf(x, 0.0f); }
__device__ __forceinline__ bool ge0(float x) { return x >= 0.0f; }
__device__ __forceinline__ bool lt0(float x) { return x < 0.0f; }
__device__ __forceinline__ bool gt0(float x) { return x > 0.0f; }
__device__ __forceinline__ bool klt(float a, float b) { return a < b; }

// Correctly rounded q/h given r = RN(1/h) (one reciprocal per cell shared by
// every tracer of the layer).  y0 = RN(q*r) is within 1.5 ulp; one
// residual correction makes it faithful; a second one is Markstein's
// theorem (y faithful, r = RN(1/h)  =>  RN(y + r*RN(q - h*y)) = RN(q/h)),
// so the result equals IEEE q/h bit for bit for normal operands.  1 DMUL +
// 4 DFMA instead of a full division.
__device__ __forceinline__ double div_rcp(double q, double h, double r) {
  double y = __dmul_rn(q, r);
  double e = __fma_rn(-y, h, q);
  y = __fma_rn(e, r, y);
  e = __fma_rn(-y, h, q);
  return __fma_rn(e, r, y);
}

}  // namespace hyc
