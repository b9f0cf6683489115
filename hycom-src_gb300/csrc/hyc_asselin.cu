// hyc_asselin.cu -- Robert-Asselin time filter of the scalar fields
// (mod_asselin.F90: asselin_save :28-82 at the start of a step,
// asselin_filter :84-268 at its end).
//
// Both are pointwise in (i,j): one thread per interior cell walks the
// layers, so the per-cell factors (oneta of both levels and the reciprocal
// of oneta(m) that turns the filtered thickness back into dp) are computed
// once per cell and reused by every layer.  FP64, built without FMA
// contraction, in the reference's operation order: the filtered values equal
// the oracle's bit for bit (the division by oneta(m) is the correctly
// rounded div_rcp of hyc_device.cuh).  Only temperature-advecting hybrid
// layers are supported: the 17-term equation of state has no tofsig.
#include <cuda_runtime.h>

#include <cstdint>

#include "hyc_args.h"
#include "hyc_device.cuh"
#include "hyc_eos.cuh"
#include "hyc_internal.h"

namespace hyc {

namespace {

constexpr double kOnezm = 9806.e-20;  // onezm, mod_asselin.F90:95

__device__ __forceinline__ long long acell(const AsselinArgs &A, long long t) {
  const int j = 1 + (int)(t / A.ii), i = 1 + (int)(t - (long long)(j - 1) * A.ii);
  return (long long)(i + A.nb - 1) + (long long)(j + A.nb - 1) * A.ld1;
}

// oneta(:,:,l) = max(oneta0, 1 + pbavg(:,:,l)/pbot) (mod_asselin.F90:50-51, :114-115)
__device__ __forceinline__ double oneta_of(const AsselinArgs &A, long long c, int l) {
  return kmax(A.oneta0, 1.0 + A.pbavg[(long long)l * A.slice + c] / A.pbot[c]);
}

// asselin_save: oneta/onetao at sea points, level n of every scalar into the
// t-1 copies at every interior point (:45-75)
__global__ void asselin_save_kernel(const AsselinArgs A) {
  const long long n = (long long)A.ii * A.jj, sl = A.slice;
  const int kk = A.kdm, mm = A.m - 1, nn = A.n - 1;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long c = acell(A, t);
    if (A.msk[c] & kIP) {
      const double on = oneta_of(A, c, nn), om = oneta_of(A, c, mm);
      A.oneta[nn * sl + c] = on;
      A.oneta[mm * sl + c] = om;
      A.onetao[nn * sl + c] = on;
      A.onetao[mm * sl + c] = om;
    }
    for (int k = 0; k < kk; k++) {
      const long long lk = k * sl + c, ln = ((long long)k + (long long)nn * kk) * sl + c;
      A.otemp[lk] = A.temp[ln];
      A.osaln[lk] = A.saln[ln];
      A.oth3d[lk] = A.th3d[ln];
      for (int q = 0; q < A.ntracr; q++)
        A.otracer[(long long)q * kk * sl + lk] = A.tracer[(long long)q * 2 * kk * sl + ln];
      if (A.mxlmy) {  // q2(…,k,n) with k 1-based in 0:kk+1
        const long long o = (long long)(k + 1) * sl + c, qn = ((long long)(k + 1) + (long long)nn * (kk + 2)) * sl + c;
        A.oq2[o] = A.q2[qn];
        A.oq2l[o] = A.q2l[qn];
      }
    }
  }
}

// the scalar filter that keeps a constant field constant (:147-155)
__device__ __forceinline__ double ra_scalar(double fo, double fm, double fn, double dpold, double dpmid, double dpnew,
                                            double hra, double qdpmidn) {
  const double smin = kmin(kmin(fo, fm), fn);
  const double dpsold = dpold * (fo - smin), dpsmid = dpmid * (fm - smin), dpsnew = dpnew * (fn - smin);
  const double q = hra * (dpsold + dpsnew - 2.0 * dpsmid);
  return smin + (dpsmid + q) * qdpmidn;
}

// asselin_filter for advflg = 0 hybrid layers (:106-236)
__global__ void asselin_filter_kernel(const AsselinArgs A) {
  const long long n = (long long)A.ii * A.jj, sl = A.slice;
  const int kk = A.kdm, mm = A.m - 1, nn = A.n - 1;
  const double hra = 0.5 * A.ra2fac;  // the leading 0.5*ra2fac of every q (:131, :154, ...)
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long c = acell(A, t);
    if (!(A.msk[c] & kIP)) continue;
    const double on = oneta_of(A, c, nn), om = oneta_of(A, c, mm);
    A.oneta[nn * sl + c] = on;
    A.oneta[mm * sl + c] = om;
    const double ron = __drcp_rn(om);
    const double oon = A.onetao[nn * sl + c], oom = A.onetao[mm * sl + c];
    for (int k = 0; k < kk; k++) {
      const long long lk = k * sl + c, lm = ((long long)k + (long long)mm * kk) * sl + c,
                      ln = ((long long)k + (long long)nn * kk) * sl + c;
      const double dpold = A.dpo[ln] * oon, dpmid = A.dpo[lm] * oom, dpnew = A.dp[ln] * on;
      const double q = hra * (dpold + dpnew - 2.0 * dpmid);
      const double dpmidn = dpmid + q;
      A.dp[lm] = div_rcp(dpmidn, om, ron);
      if (!(dpmidn > kOnezm)) continue;
      const double qdpmidn = __drcp_rn(dpmidn);
      const double s = ra_scalar(A.osaln[lk], A.saln[lm], A.saln[ln], dpold, dpmid, dpnew, hra, qdpmidn);
      const double tm = ra_scalar(A.otemp[lk], A.temp[lm], A.temp[ln], dpold, dpmid, dpnew, hra, qdpmidn);
      A.saln[lm] = s;
      A.temp[lm] = tm;
      A.th3d[lm] = sig17(tm, s) - A.thbase;
      for (int q2i = 0; q2i < A.ntracr; q2i++) {
        double *f = A.tracer + (long long)q2i * 2 * kk * sl;
        const double *fo = A.otracer + (long long)q2i * kk * sl;
        f[lm] = ra_scalar(fo[lk], f[lm], f[ln], dpold, dpmid, dpnew, hra, qdpmidn);
      }
      if (A.mxlmy) {
        const long long o = (long long)(k + 1) * sl + c, qm = ((long long)(k + 1) + (long long)mm * (kk + 2)) * sl + c,
                        qn = ((long long)(k + 1) + (long long)nn * (kk + 2)) * sl + c;
        double so = dpold * A.oq2[o], sm = dpmid * A.q2[qm], sn = dpnew * A.q2[qn];
        A.q2[qm] = (sm + hra * (so + sn - 2.0 * sm)) * qdpmidn;
        so = dpold * A.oq2l[o];
        sm = dpmid * A.q2l[qm];
        sn = dpnew * A.q2l[qn];
        A.q2l[qm] = (sm + hra * (so + sn - 2.0 * sm)) * qdpmidn;
      }
    }
  }
}

unsigned grid_of(long long n) {
  long long b = (n + 255) / 256;
  return (unsigned)(b > 65535 * 4 ? 65535 * 4 : (b < 1 ? 1 : b));
}

}  // namespace

cudaError_t launch_asselin(const AsselinArgs &a, bool filter, cudaStream_t s) {
  const long long n = (long long)a.ii * a.jj;
  if (filter)
    asselin_filter_kernel<<<grid_of(n), 256, 0, s>>>(a);
  else
    asselin_save_kernel<<<grid_of(n), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hyc
