// hyc_fct2c.cu -- advem_fct2c (mod_tsadvc.F90:999-1368): FCT2 with the
// barotropic mass flux (btrmas), whose low-order part is a donor-cell scheme
// sub-cycled five times with a local time step per cell.
//
// FP64, one kernel per stage over whole slices, as the reference sweeps its
// arrays (the sub-cycling refreshes the halo of hloc and fldlo between
// iterations, mod_tsadvc.F90:1181-1182, which a fused tile would have to
// replace by an 8-cell halo; this is the first GPU form of the scheme).
// A launch covers up to 16 (field, layer) pairs; every pair has its own 13
// work slices (the reference's module arrays uloc, vloc, hloc, dtloc,
// ucumdt, vcumdt, flxcum, flycum, lcalc, fldlo, flx, fly, fax, fay, rp, rm,
// with fax/fay/rp/rm reusing the dead uloc/vloc/flx/fly).  The stages keep
// the reference's margins and operation order and are built without FMA
// contraction, so results equal the oracle's bit for bit.
#include <cuda_runtime.h>

#include <cstdint>

#include "hyc_args.h"
#include "hyc_internal.h"

namespace hyc {

namespace {

constexpr double kEps = 1.e-10;  // epsil, mod_tsadvc.F90:1027
constexpr int kMb = 5;           // mbdy_advtyp(2)

// the reference's max/min of two reals (mod_tsadvc.F90 passim)
__device__ __forceinline__ double mx2(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double mn2(double a, double b) { return a < b ? a : b; }

enum { A_FCO, A_FCN, A_HLOC, A_FLDLO, A_DTLOC, A_UCUM, A_VCUM, A_ULOC, A_VLOC, A_FLX, A_FLY, A_FXC, A_FYC, A_N };
// after the sub-iterations: fax, fay, rp, rm live in uloc, vloc, flx, fly
enum { A_FAX = A_ULOC, A_FAY = A_VLOC, A_RP = A_FLX, A_RM = A_FLY };

__device__ __forceinline__ double *W(const Fct2cArgs &A, int arr, int p) {
  return A.work + ((long long)arr * A.npair + p) * A.slice;
}

// cell (i,j) of the margin region [1-m, ii+m] x [1-m, jj+m] for thread t;
// false beyond the region
__device__ __forceinline__ bool cell_of(const Fct2cArgs &A, int m, long long t, int &i, int &j, long long &c) {
  const int w = A.ii + 2 * m;
  const long long n = (long long)w * (A.jj + 2 * m);
  if (t >= n) return false;
  j = (int)(t / w);
  i = (int)(t - (long long)j * w);
  i += 1 - m;
  j += 1 - m;
  c = (long long)(i + A.nb - 1) + (long long)(j + A.nb - 1) * A.ld1;
  return true;
}

// thickness (mod_tsadvc.F90:1905-1942, with onetamas(m), :1804-1810) and the
// whole-array initialisation of the work arrays (:1068-1081)
__global__ void fct2c_init(Fct2cArgs A) {
  const int p = blockIdx.y;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.slice) return;
  const long long sl = A.slice;
  const int ld1 = A.ld1;
  const int a = (int)(t % ld1), b = (int)(t / ld1);
  double fco, fcn;
  if (A.mode == 0) {
    const long long k = A.k[p];
    const double *u = A.uflx + k * sl, *v = A.vflx + k * sl;
    const double ota = A.oneta ? A.oneta[t] : 1.0;
    const double o = ota * A.dpn[k * sl + t];
    double fdv = 0.0;
    if (a < ld1 - 1 && b < A.ld2 - 1) fdv = ((u[t + 1] - u[t]) + (v[t + ld1] - v[t])) * A.dt2 * A.scali[t];
    fco = mx2(o + fdv, 0.0);
    fcn = mx2(o, 0.0);
  } else {
    fco = A.fco[t];
    fcn = A.fcn[t];
  }
  W(A, A_FCO, p)[t] = fco;
  W(A, A_FCN, p)[t] = fcn;
  W(A, A_HLOC, p)[t] = fco;
  W(A, A_FLDLO, p)[t] = A.fld[p][t];
  W(A, A_DTLOC, p)[t] = 0.0;
  W(A, A_UCUM, p)[t] = 0.0;
  W(A, A_VCUM, p)[t] = 0.0;
  W(A, A_ULOC, p)[t] = 0.0;
  W(A, A_VLOC, p)[t] = 0.0;
  W(A, A_FLX, p)[t] = 0.0;
  W(A, A_FLY, p)[t] = 0.0;
  W(A, A_FXC, p)[t] = 0.0;
  W(A, A_FYC, p)[t] = 0.0;
  A.lcalc[p * sl + t] = 1;
}

__device__ __forceinline__ const double *U_(const Fct2cArgs &A, int p) {
  return A.mode == 0 ? A.uflx + (long long)A.k[p] * A.slice : A.uflx;
}
__device__ __forceinline__ const double *V_(const Fct2cArgs &A, int p) {
  return A.mode == 0 ? A.vflx + (long long)A.k[p] * A.slice : A.vflx;
}

// local time step per cell (:1086-1099)
__global__ void fct2c_dt(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, kMb, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  if (!(A.msk[c] & kIP)) return;
  const double *u = U_(A, p), *v = V_(A, p);
  const int ld = A.ld1;
  const double q = mx2(u[c + 1], 0.0) - mn2(u[c], 0.0) + mx2(v[c + ld], 0.0) - mn2(v[c], 0.0);
  double *dt = W(A, A_DTLOC, p);
  if (q > 0.0)
    dt[c] = mn2(A.dt2, W(A, A_HLOC, p)[c] / (q * A.scali[c]));
  else
    dt[c] = A.dt2;
}

// partial-step donor fluxes and their sums (:1101-1149)
__global__ void fct2c_flux(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, kMb - 1, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  const uint8_t m = A.msk[c];
  const double *u = U_(A, p), *v = V_(A, p);
  const int ld = A.ld1;
  const double dt2 = A.dt2;
  const double *dt = W(A, A_DTLOC, p), *lo = W(A, A_FLDLO, p);
  if (m & kIU) {
    double *ucum = W(A, A_UCUM, p), *uloc = W(A, A_ULOC, p), *flx = W(A, A_FLX, p), *fxc = W(A, A_FXC, p);
    if (ucum[c] != dt2) {
      if (u[c] >= 0) {
        uloc[c] = mn2(dt2 - ucum[c], dt[c - 1]) * u[c];
        flx[c] = lo[c - 1] * uloc[c];
        ucum[c] = ucum[c] + mn2(dt2 - ucum[c], dt[c - 1]);
      } else {
        uloc[c] = mn2(dt2 - ucum[c], dt[c]) * u[c];
        flx[c] = lo[c] * uloc[c];
        ucum[c] = ucum[c] + mn2(dt2 - ucum[c], dt[c]);
      }
      fxc[c] = fxc[c] + flx[c];
    } else {
      uloc[c] = 0.0;
      flx[c] = 0.0;
    }
  }
  if (m & kIV) {
    double *vcum = W(A, A_VCUM, p), *vloc = W(A, A_VLOC, p), *fly = W(A, A_FLY, p), *fyc = W(A, A_FYC, p);
    if (vcum[c] != dt2) {
      if (v[c] >= 0) {
        vloc[c] = mn2(dt2 - vcum[c], dt[c - ld]) * v[c];
        fly[c] = lo[c - ld] * vloc[c];
        vcum[c] = vcum[c] + mn2(dt2 - vcum[c], dt[c - ld]);
      } else {
        vloc[c] = mn2(dt2 - vcum[c], dt[c]) * v[c];
        fly[c] = lo[c] * vloc[c];
        vcum[c] = vcum[c] + mn2(dt2 - vcum[c], dt[c]);
      }
      fyc[c] = fyc[c] + fly[c];
    } else {
      vloc[c] = 0.0;
      fly[c] = 0.0;
    }
  }
}

// low-order update of fldlo and hloc (:1153-1176)
__global__ void fct2c_cell(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, kMb - 2, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  if (!(A.msk[c] & kIP)) return;
  uint8_t *lc = A.lcalc + (long long)p * A.slice;
  if (!lc[c]) return;
  const int ld = A.ld1;
  const double dt2 = A.dt2;
  double *h = W(A, A_HLOC, p), *lo = W(A, A_FLDLO, p);
  const double *uloc = W(A, A_ULOC, p), *vloc = W(A, A_VLOC, p), *flx = W(A, A_FLX, p), *fly = W(A, A_FLY, p);
  const double *ucum = W(A, A_UCUM, p), *vcum = W(A, A_VCUM, p);
  const double qp = h[c] - (uloc[c + 1] - uloc[c] + vloc[c + ld] - vloc[c]) * A.scali[c];
  if (qp > 0.0)
    lo[c] = ((kEps + h[c]) * lo[c] - (flx[c + 1] - flx[c] + fly[c + ld] - fly[c]) * A.scali[c]) / (kEps + qp);
  h[c] = qp;
  lc[c] = ucum[c + 1] != dt2 || ucum[c] != dt2 || vcum[c + ld] != dt2 || vcum[c] != dt2;
}

// antidiffusive fluxes (:1199-1215); faces that are not between two sea
// cells carry none (the section-edge zeroing :1223-1243 covers every such
// face a sea cell reads)
__global__ void fct2c_anti(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, kMb - 2, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  const uint8_t m = A.msk[c];
  const double *u = U_(A, p), *v = V_(A, p);
  const double *fc = A.fldc[p];
  const int ld = A.ld1;
  const double dt2 = A.dt2;
  double *fax = W(A, A_FAX, p), *fay = W(A, A_FAY, p);
  const double *fxc = W(A, A_FXC, p), *fyc = W(A, A_FYC, p);
  if (m & kIU) {
    const double fhx = u[c] * 0.5 * (fc[c] + fc[c - 1]);
    fax[c] = fhx - fxc[c] / dt2;
  } else {
    fax[c] = 0.0;
  }
  if (m & kIV) {
    const double fhy = v[c] * 0.5 * (fc[c] + fc[c - ld]);
    fay[c] = fhy - fyc[c] / dt2;
  } else {
    fay[c] = 0.0;
  }
}

// Zalesak ratios (:1257-1303), true i+1/j+1 neighbours
__global__ void fct2c_ratio(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, kMb - 3, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  if (!(A.msk[c] & kIP)) return;
  const int ld = A.ld1;
  const double *lo = W(A, A_FLDLO, p), *h = W(A, A_HLOC, p), *fax = W(A, A_FAX, p), *fay = W(A, A_FAY, p);
  const long long ca = (A.msk[c - 1] & kIP) ? c - 1 : c, cb = (A.msk[c + 1] & kIP) ? c + 1 : c;
  const long long cja = (A.msk[c - ld] & kIP) ? c - ld : c, cjb = (A.msk[c + ld] & kIP) ? c + ld : c;
  const double fqmax = mx2(mx2(mx2(mx2(lo[c], lo[ca]), lo[cb]), lo[cja]), lo[cjb]);
  const double fqmin = mn2(mn2(mn2(mn2(lo[c], lo[ca]), lo[cb]), lo[cja]), lo[cjb]);
  const double famax = mx2(0.0, fax[c]) - mn2(0.0, fax[c + 1]) + mx2(0.0, fay[c]) - mn2(0.0, fay[c + ld]);
  const double famin = mx2(0.0, fax[c + 1]) - mn2(0.0, fax[c]) + mx2(0.0, fay[c + ld]) - mn2(0.0, fay[c]);
  const double qdt2 = 1.0 / A.dt2;
  double rp, rm;
  if (famax > kEps) {
    const double qp = (fqmax - lo[c]) * h[c] * A.scal[c] * qdt2;
    rp = (qp < famax) ? qp / famax : 1.0;
  } else {
    rp = 0.0;
  }
  if (famin > kEps) {
    const double qm = (lo[c] - fqmin) * h[c] * A.scal[c] * qdt2;
    rm = (qm < famin) ? qm / famin : 1.0;
  } else {
    rm = 0.0;
  }
  W(A, A_RP, p)[c] = rp;
  W(A, A_RM, p)[c] = rm;
}

// limited antidiffusive fluxes (:1308-1332), in place
__global__ void fct2c_limit(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, kMb - 4, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  const uint8_t m = A.msk[c];
  const int ld = A.ld1;
  const double *rp = W(A, A_RP, p), *rm = W(A, A_RM, p);
  double *fax = W(A, A_FAX, p), *fay = W(A, A_FAY, p);
  if (m & kIU) {
    const double fact = fax[c] < 0.0 ? mn2(rp[c - 1], rm[c]) : mn2(rp[c], rm[c - 1]);
    fax[c] = fact * fax[c];
  }
  if (m & kIV) {
    const double fact = fay[c] < 0.0 ? mn2(rp[c - ld], rm[c]) : mn2(rp[c], rm[c - ld]);
    fay[c] = fact * fay[c];
  }
}

// corrected update of the interior sea cells (:1340-1359)
__global__ void fct2c_update(Fct2cArgs A) {
  const int p = blockIdx.y;
  int i, j;
  long long c;
  if (!cell_of(A, 0, (long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, c)) return;
  if (!(A.msk[c] & kIP)) return;
  const int ld = A.ld1;
  const double *lo = W(A, A_FLDLO, p), *h = W(A, A_HLOC, p), *fax = W(A, A_FAX, p), *fay = W(A, A_FAY, p);
  const double flxdiv = ((fax[c + 1] - fax[c]) + (fay[c + ld] - fay[c])) * A.dt2 * A.scali[c];
  double *f = A.fld[p];
  if (h[c] > 0.)
    f[c] = ((kEps + h[c]) * lo[c] - flxdiv) / (kEps + h[c]);
  else
    f[c] = lo[c];
}

template <class K>
cudaError_t go(K kern, const Fct2cArgs &A, int margin, cudaStream_t s) {
  const long long n = (long long)(A.ii + 2 * margin) * (A.jj + 2 * margin);
  dim3 grid((unsigned)((n + 255) / 256), A.npair);
  kern<<<grid, 256, 0, s>>>(A);
  return cudaGetLastError();
}

}  // namespace

size_t fct2c_work_bytes(long long slice) { return (size_t)slice * (A_N * sizeof(double) + 1); }

cudaError_t launch_fct2c(const Fct2cArgs &A, int nreg, int *launches, cudaStream_t s) {
  cudaError_t e;
  int nl = 0;
  {
    dim3 grid((unsigned)((A.slice + 255) / 256), A.npair);
    fct2c_init<<<grid, 256, 0, s>>>(A);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    nl++;
  }
  for (int it = 0; it < 5; it++) {  // :1083-1192
    if ((e = go(fct2c_dt, A, kMb, s)) != cudaSuccess) return e;
    if ((e = go(fct2c_flux, A, kMb - 1, s)) != cudaSuccess) return e;
    if ((e = go(fct2c_cell, A, kMb - 2, s)) != cudaSuccess) return e;
    // xctilr(hloc), xctilr(fldlo), :1181-1182
    if ((e = launch_xctilr(A.work + (long long)A_HLOC * A.npair * A.slice, A.slice, A.npair, A.ii, A.jj, A.nb, A.ld1,
                           kMb, kMb, nreg, s)) != cudaSuccess)
      return e;
    if ((e = launch_xctilr(A.work + (long long)A_FLDLO * A.npair * A.slice, A.slice, A.npair, A.ii, A.jj, A.nb,
                           A.ld1, kMb, kMb, nreg, s)) != cudaSuccess)
      return e;
    nl += 5;
  }
  if ((e = go(fct2c_anti, A, kMb - 2, s)) != cudaSuccess) return e;
  if ((e = go(fct2c_ratio, A, kMb - 3, s)) != cudaSuccess) return e;
  if ((e = go(fct2c_limit, A, kMb - 4, s)) != cudaSuccess) return e;
  if ((e = go(fct2c_update, A, 0, s)) != cudaSuccess) return e;
  nl += 4;
  if (launches) *launches += nl;
  return cudaSuccess;
}

}  // namespace hyc
