// hyc_cnuity.cu -- the continuity equation (cnuity.F90:14-1419): flux-
// corrected transport of the layer thicknesses, the barotropic restoration
// and bottom-pressure restoring (not btrmas), biharmonic or Laplacian
// interface-depth diffusion, the cumulative fluxes, the btrmas restoring and
// the Robert-Asselin filter of dp.
//
// The reference is a sequence of sweeps over the slice whose margins shrink
// from 6 to 0 within a layer, with a vertical recurrence (util3 = depth of
// the layer's top, p = interface pressures) from one layer to the next.  The
// first GPU form keeps that structure: one kernel per sweep over the same
// margin, layer after layer, so every value the reference computes (halo
// cells included) is computed here, in the same operation order, FP64
// without FMA contraction: the results equal the oracle's bit for bit.  The
// sweeps are memory-bound (about 55 slice reads/writes per cell and layer
// against 11 for a fused form); a tile kernel that walks the layers with a
// six-cell halo is the next form.
//
// Work slices (CnuityArgs::w): uflux, vflux, uflux2, vflux2, utotn, vtotn,
// util1, util2, util3, pold, oneta_u, oneta_v, onetamas(:,:,1:2).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "hyc_args.h"
#include "hyc_device.cuh"
#include "hyc_internal.h"

namespace hyc {

namespace {

enum { W_UF, W_VF, W_UF2, W_VF2, W_UTN, W_VTN, W_U1, W_U2, W_U3, W_POLD, W_OU, W_OV, W_OM, W_N = W_OM + 2 };

constexpr double kOnem = 9.806 / (1.0 / 1000.0);  // onem = g/svref, mod_cb_arrays.F90:843-846
constexpr double kOnecm = kOnem * 0.01;
constexpr double kEpsilCb = 1.0e-11;   // epsil, mod_cb_arrays.F90:853
constexpr double kEpsilCn = 1.e-14;    // epsil_cnuity, cnuity.F90:52

struct Cell {
  int i, j;
  long long c;
};

// thread -> cell of the box i in [1-M, ii+M], j in [1-M, jj+M]; false when outside
__device__ __forceinline__ bool cell_of(const CnuityArgs &A, int M, Cell &x) {
  const int bi = blockIdx.x * blockDim.x + threadIdx.x, bj = blockIdx.y * blockDim.y + threadIdx.y;
  if (bi >= A.ii + 2 * M || bj >= A.jj + 2 * M) return false;
  x.i = 1 - M + bi;
  x.j = 1 - M + bj;
  x.c = (long long)(x.i + A.nb - 1) + (long long)(x.j + A.nb - 1) * A.ld1;
  return true;
}

__device__ __forceinline__ double *W(const CnuityArgs &A, int s) { return A.w + (long long)s * A.slice; }

// the reference's max/min of two reals (ordered as written; signs of zero
// never reach a result of this path)
__device__ __forceinline__ double mx(double a, double b) { return kmax(a, b); }
__device__ __forceinline__ double mn(double a, double b) { return kmin(a, b); }

// :112-157 at margin 6
__global__ void cn_init(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 6, x)) return;
  const long long c = x.c, sl = A.slice;
  const int mm = A.m - 1, nn = A.n - 1;
  const uint8_t mk = A.msk[c];
  double *om = W(A, W_OM);
  // the outermost halo column/row has no west/south neighbour; its u/v
  // factors are never read
  const bool w = x.i > 1 - A.nb, s = x.j > 1 - A.nb;
  if (A.btrmas) {
    om[c] = A.oneta[c];
    om[c + sl] = A.oneta[c + sl];
    if ((mk & kIU) && w) {
      const double a = A.oneta[c + mm * sl], b = A.oneta[c - 1 + mm * sl];
      W(A, W_OU)[c] = A.pbot[c] == A.pbot[c - 1] ? 0.5 * (a + b) : (A.pbot[c] == A.depthu[c] ? a : b);
    }
    if ((mk & kIV) && s) {
      const double a = A.oneta[c + mm * sl], b = A.oneta[c - A.ld1 + mm * sl];
      W(A, W_OV)[c] = A.pbot[c] == A.pbot[c - A.ld1] ? 0.5 * (a + b) : (A.pbot[c] == A.depthv[c] ? a : b);
    }
  } else {
    om[c] = 1.0;
    om[c + sl] = 1.0;
    W(A, W_OU)[c] = 1.0;
    W(A, W_OV)[c] = 1.0;
  }
  W(A, W_UTN)[c] = 0.0;
  W(A, W_VTN)[c] = 0.0;
  W(A, W_U3)[c] = 0.0;
  for (int k = 0; k < A.kdm; k++) {
    const long long o = ((long long)k + (long long)nn * A.kdm) * sl + c;
    A.dpo[o] = A.dp[o];
  }
}

// loop 76, :240-285 at margin 5: low-order and antidiffusive fluxes of layer k.
// BT = btrmas.  Without it onetamas and the face factors oneta_u/v are 1.0
// (:142-145), and x*1.0 == x exactly, so those products (and their loads)
// are skipped; the FP64 pipe bounds this kernel.
template <bool BT>
__global__ void cn_flux(const CnuityArgs A, int k) {
  Cell x;
  if (!cell_of(A, 5, x)) return;
  const long long c = x.c, sl = A.slice, ld = A.ld1;
  const int mm = A.m - 1, nn = A.n - 1;
  const uint8_t mk = A.msk[c];
  const double *dk = A.dp + ((long long)k + (long long)nn * A.kdm) * sl;
  const double *u3 = W(A, W_U3), *omn = W(A, W_OM) + nn * sl;
  const long long lm = ((long long)k + (long long)mm * A.kdm) * sl;
  if (mk & kIU) {
    const double utotm = (A.u[lm + c] + A.ubavg[mm * sl + c]) * A.scuy[c];
    const long long cq = ge0(utotm) ? c - 1 : c;
    const double q0 = mn(dk[cq], mx(0., A.depthu[c] - u3[cq]));
    const double uf = utotm * (BT ? q0 * omn[cq] : q0);
    W(A, W_UF)[c] = uf;
    const double ud = utotm * A.dpu[lm + c];
    W(A, W_UF2)[c] = (BT ? ud * W(A, W_OU)[c] : ud) - uf;
    A.uflx[(long long)k * sl + c] = uf;
  }
  if (mk & kIV) {
    const double vtotm = (A.v[lm + c] + A.vbavg[mm * sl + c]) * A.scvx[c];
    const long long cq = ge0(vtotm) ? c - ld : c;
    const double q0 = mn(dk[cq], mx(0., A.depthv[c] - u3[cq]));
    const double vf = vtotm * (BT ? q0 * omn[cq] : q0);
    W(A, W_VF)[c] = vf;
    const double vd = vtotm * A.dpv[lm + c];
    W(A, W_VF2)[c] = (BT ? vd * W(A, W_OV)[c] : vd) - vf;
    A.vflx[(long long)k * sl + c] = vf;
  }
}

// per-warp minimum of a key, one atomic per warp (dpkmin rows j = 1..jj)
__device__ __forceinline__ void row_min(const CnuityArgs &A, const Cell &x, bool in, double v, int slot) {
  long long k = (in && x.j >= 1 && x.j <= A.jj) ? dkey(v) : LLONG_MAX;
  for (int o = 16; o > 0; o >>= 1) {
    const long long t = __shfl_xor_sync(0xffffffffu, k, o);
    k = t < k ? t : k;
  }
  if ((threadIdx.x & 31) == 0 && k != LLONG_MAX) atomicMin(&A.keys[slot], k);
}

// loop 19, :294-315 at margin 4: low-order update of dp(k,n) (BT as cn_flux)
template <bool BT>
__global__ void cn_low(const CnuityArgs A, int k) {
  Cell x;
  const bool in = cell_of(A, 4, x);
  bool sea = false;
  double d = 0.0;
  if (in && (A.msk[x.c] & kIP)) {
    const long long c = x.c, sl = A.slice, ld = A.ld1;
    const int mm = A.m - 1, nn = A.n - 1;
    double *dk = A.dp + ((long long)k + (long long)nn * A.kdm) * sl;
    const double *uf = W(A, W_UF), *vf = W(A, W_VF);
    W(A, W_U3)[c] = W(A, W_U3)[c] + dk[c];
    d = (BT ? dk[c] * W(A, W_OM)[nn * sl + c] : dk[c]) -
        ((uf[c + 1] - uf[c]) + (vf[c + ld] - vf[c])) * A.delt1 * A.scp2i[c];
    dk[c] = d;
    A.dpo[((long long)k + (long long)mm * A.kdm) * sl + c] = d;
    sea = true;
  }
  if (A.keys) row_min(A, x, in && sea, d, k);
}

// :400-430 at margin 4: the limiter's ratios
__global__ void cn_ratio(const CnuityArgs A, int k) {
  Cell x;
  if (!cell_of(A, 4, x)) return;
  const long long c = x.c, sl = A.slice, ld = A.ld1;
  if (!(A.msk[c] & kIP)) return;
  const int nn = A.n - 1;
  const double *dk = A.dp + ((long long)k + (long long)nn * A.kdm) * sl;
  // ipim1 etc. (bigrid.F90:316-340): the neighbour if sea, else the point itself
  const uint8_t *ms = A.msk;
  const long long ca = (ms[c - 1] & kIP) ? c - 1 : c, cb = (ms[c + 1] & kIP) ? c + 1 : c,
                  cja = (ms[c - ld] & kIP) ? c - ld : c, cjb = (ms[c + ld] & kIP) ? c + ld : c;
  const double d = dk[c];
  const double u1 = mx(mx(mx(mx(d, dk[ca]), dk[cb]), dk[cja]), dk[cjb]);
  const double u2 = mx(0., mn(mn(mn(mn(d, dk[ca]), dk[cb]), dk[cja]), dk[cjb]));
  const double *f2u = W(A, W_UF2), *f2v = W(A, W_VF2);
  W(A, W_U1)[c] = (u1 - d) / ((((pos0(f2u[c]) - neg0(f2u[c + 1])) + (pos0(f2v[c]) - neg0(f2v[c + ld]))) + kEpsilCb) *
                              A.delt1 * A.scp2i[c]);
  W(A, W_U2)[c] = (u2 - d) / ((((neg0(f2u[c]) - pos0(f2u[c + 1])) + (neg0(f2v[c]) - pos0(f2v[c + ld]))) - kEpsilCb) *
                              A.delt1 * A.scp2i[c]);
}

// :442-472 at margin 3: clip the antidiffusive fluxes
__global__ void cn_clip(const CnuityArgs A, int k) {
  Cell x;
  if (!cell_of(A, 3, x)) return;
  const long long c = x.c, sl = A.slice, ld = A.ld1;
  const uint8_t mk = A.msk[c];
  const double *u1 = W(A, W_U1), *u2 = W(A, W_U2);
  if (mk & kIU) {
    const double f2 = W(A, W_UF2)[c];
    const double clip = ge0(f2) ? mn(mn(1., u1[c]), u2[c - 1]) : mn(mn(1., u2[c]), u1[c - 1]);
    W(A, W_UTN)[c] = W(A, W_UTN)[c] + f2 * (1. - clip);
    const double uf = f2 * clip;
    W(A, W_UF)[c] = uf;
    A.uflx[(long long)k * sl + c] = A.uflx[(long long)k * sl + c] + uf;
  }
  if (mk & kIV) {
    const double f2 = W(A, W_VF2)[c];
    const double clip = ge0(f2) ? mn(mn(1., u1[c]), u2[c - ld]) : mn(mn(1., u2[c]), u1[c - ld]);
    W(A, W_VTN)[c] = W(A, W_VTN)[c] + f2 * (1. - clip);
    const double vf = f2 * clip;
    W(A, W_VF)[c] = vf;
    A.vflx[(long long)k * sl + c] = A.vflx[(long long)k * sl + c] + vf;
  }
}

// loop 15 (:480-498, margin 2) and loop 14 (:650-665, margin 0): flux update
// of dp(k,n) and p(k+1)
__global__ void cn_update(const CnuityArgs A, int k, int M, int slot) {
  Cell x;
  const bool in = cell_of(A, M, x);
  bool sea = false;
  double d = 0.0;
  if (in && (A.msk[x.c] & kIP)) {
    const long long c = x.c, sl = A.slice, ld = A.ld1;
    const int nn = A.n - 1;
    double *dk = A.dp + ((long long)k + (long long)nn * A.kdm) * sl;
    const double *uf = W(A, W_UF), *vf = W(A, W_VF);
    d = dk[c] - ((uf[c + 1] - uf[c]) + (vf[c + ld] - vf[c])) * A.delt1 * A.scp2i[c];
    dk[c] = d;
    A.p[(long long)(k + 1) * sl + c] = A.p[(long long)k * sl + c] + d;
    sea = true;
  }
  if (A.keys && slot >= 0) row_min(A, x, in && sea, d, slot);
}

// loop 77: RN(1/p(kk+1)) of every sea cell at margin 2, into util1 (free
// until the interface diffusion).  p(kk+1) does not change during loop 77
// before its last layer's fluxes are formed, so one reciprocal per cell
// serves every layer's division dp/p(kk+1).
__global__ void cn_rpb(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 2, x)) return;
  const long long c = x.c;
  if (!(A.msk[c] & kIP)) return;
  W(A, W_U1)[c] = 1. / A.p[(long long)A.kdm * A.slice + c];
}

// loop 77, :595-645 at margin 1: the barotropic correction fluxes of layer k.
// q = dp/p(kk+1) by div_rcp with the cell's reciprocal: the IEEE quotient
// bit for bit, for 5 FP64 operations instead of a division.
__global__ void cn_btflux(const CnuityArgs A, int k) {
  Cell x;
  if (!cell_of(A, 1, x)) return;
  const long long c = x.c, sl = A.slice, ld = A.ld1;
  const uint8_t mk = A.msk[c];
  const int nn = A.n - 1;
  const double *dk = A.dp + ((long long)k + (long long)nn * A.kdm) * sl, *pb = A.p + (long long)A.kdm * sl;
  const double *rpb = W(A, W_U1);
  if (mk & kIU) {
    const double ut = W(A, W_UTN)[c];
    const long long cu = ge0(ut) ? c - 1 : c;
    const double uf = ut * div_rcp(dk[cu], pb[cu], rpb[cu]);
    W(A, W_UF)[c] = uf;
    A.uflx[(long long)k * sl + c] = A.uflx[(long long)k * sl + c] + uf;
  }
  if (mk & kIV) {
    const double vt = W(A, W_VTN)[c];
    const long long cv = ge0(vt) ? c - ld : c;
    const double vf = vt * div_rcp(dk[cv], pb[cv], rpb[cv]);
    W(A, W_VF)[c] = vf;
    A.vflx[(long long)k * sl + c] = A.vflx[(long long)k * sl + c] + vf;
  }
}

// :709-735 at margin 0: bottom-pressure restoring (not btrmas)
__global__ void cn_bottom(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 0, x)) return;
  const long long c = x.c, sl = A.slice;
  if (!(A.msk[c] & kIP)) return;
  const int nn = A.n - 1;
  const double q = A.pbot[c] / A.p[(long long)A.kdm * sl + c];
  for (int k = 0; k < A.kdm; k++) {
    double *d = A.dp + ((long long)k + (long long)nn * A.kdm) * sl + c;
    *d = *d * q;
    A.p[(long long)(k + 1) * sl + c] = A.p[(long long)k * sl + c] + *d;
  }
}

// :770-785 / :993-1010 at margin 6: start of the interface diffusion
__global__ void cn_thk_init(const CnuityArgs A, int bih, int iflip) {
  Cell x;
  if (!cell_of(A, 6, x)) return;
  const long long c = x.c;
  const uint8_t mk = A.msk[c];
  if (mk & kIU) W(A, W_UF)[c] = 0.;
  if (mk & kIV) W(A, W_VF)[c] = 0.;
  if (mk & kIP) {
    if (!bih) W(A, W_VF)[c] = 0.;
    W(A, W_POLD)[c] = iflip == 1 ? A.p[(long long)A.kdm * A.slice + c] : 0.;
  }
}

// ipim1x etc. (bigrid.F90:343-368): W (E, S, N) if sea, else the opposite
// neighbour if sea, else the point itself
__device__ __forceinline__ long long nbx(const CnuityArgs &A, long long c, long long d) {
  if (A.msk[c + d] & kIP) return c + d;
  if (A.msk[c - d] & kIP) return c - d;
  return c;
}

// loop 13, :790-830 at margin 5: biharmonic smoothing operands at interface k (1-based)
__global__ void cn_thk_util(const CnuityArgs A, int k) {
  Cell x;
  if (!cell_of(A, 5, x)) return;
  const long long c = x.c, sl = A.slice, ld = A.ld1;
  if (!(A.msk[c] & kIP)) return;
  const int nn = A.n - 1;
  const double *dk = A.dp + ((long long)(k - 1) + (long long)nn * A.kdm) * sl,
               *dkm = A.dp + ((long long)(k - 2) + (long long)nn * A.kdm) * sl, *pk = A.p + (long long)(k - 1) * sl;
  double u1, u2;
  if (mn(dk[c], dkm[c]) < kOnecm) {
    u1 = 0.0;
    u2 = 0.0;
  } else {
    const long long ca = nbx(A, c, -1), cb = nbx(A, c, 1), cja = nbx(A, c, -ld), cjb = nbx(A, c, ld);
    u1 = pk[c] - .5 * (pk[ca] + pk[cb]);
    u2 = pk[c] - .5 * (pk[cja] + pk[cjb]);
    if (gt0(u1)) {
      if (mn(dk[ca], dk[cb]) < kOnecm) u1 = 0.0;
    } else {
      if (mn(dkm[ca], dkm[cb]) < kOnecm) u1 = 0.0;
    }
    if (gt0(u2)) {
      if (mn(dk[cja], dk[cjb]) < kOnecm) u2 = 0.0;
    } else {
      if (mn(dkm[cja], dkm[cjb]) < kOnecm) u2 = 0.0;
    }
  }
  W(A, W_U1)[c] = u1;
  W(A, W_U2)[c] = u2;
}

// :838-900 (biharmonic) / :1030-1060 (Laplacian) at margin 4: limited
// interface fluxes at interface k (1-based).  The per-cell terms of the
// face bounds, G = .25*(p(kk+1)-p(k))*scp2 and (biharmonic) H =
// .25*(p(k)-pold)*scp2 (iflip 0) or .25*(pold-p(k))*scp2 (iflip 1), are
// formed once per cell in shared memory, each by the reference's own
// operations, and every face takes them from there (each is used by up to
// four faces): flxhi = G(i), flxlo = -G(i-1) (negation is exact), and the
// biharmonic bounds uflux + H, uflux - H of the cells the reference names.
constexpr int kTX = 32, kTY = 8;  // the block of every cnuity launch
__global__ void __launch_bounds__(kTX * kTY) cn_thk_flux(const CnuityArgs A, int k, int bih, int iflip) {
  __shared__ double sG[kTY + 1][kTX + 1], sH[kTY + 1][kTX + 1];
  Cell x;
  const bool in = cell_of(A, 4, x);
  const int tx = threadIdx.x + 1, ty = threadIdx.y + 1;
  const long long sl = A.slice, ld = A.ld1;
  const double *pk = A.p + (long long)(k - 1) * sl, *ptop = A.p + (long long)A.kdm * sl;
  const double *pold = W(A, W_POLD), *scp2 = A.scp2;
  auto terms = [&](long long c, int sy, int sx) {
    sG[sy][sx] = .25 * (ptop[c] - pk[c]) * scp2[c];
    if (bih) sH[sy][sx] = iflip == 0 ? .25 * (pk[c] - pold[c]) * scp2[c] : .25 * (pold[c] - pk[c]) * scp2[c];
  };
  // the box starts at margin 4, so the west and south neighbours of its
  // first column and row (margin 5) lie inside the array
  if (in) {
    terms(x.c, ty, tx);
    if (tx == 1) terms(x.c - 1, ty, 0);
    if (ty == 1) terms(x.c - ld, 0, tx);
  }
  __syncthreads();
  if (!in) return;
  const long long c = x.c;
  const uint8_t mk = A.msk[c];
  const double dtinv = A.dtinv;
  double *uk1 = A.uflx + (long long)(k - 2) * sl, *uk = A.uflx + (long long)(k - 1) * sl;
  double *vk1 = A.vflx + (long long)(k - 2) * sl, *vk = A.vflx + (long long)(k - 1) * sl;
  const double g = sG[ty][tx];
  if (mk & kIU) {
    double *uf = W(A, W_UF);
    double flxhi = g, flxlo = -sG[ty][tx - 1];
    double f;
    if (bih) {
      const double hw = sH[ty][tx - 1], h = sH[ty][tx];
      flxhi = mn(flxhi, uf[c] + (iflip == 0 ? hw : h));
      flxlo = mx(flxlo, uf[c] - (iflip == 0 ? h : hw));
      const double thkdfu = A.delt1 * A.thkdfu[c];
      f = mn(flxhi, mx(flxlo, thkdfu * (W(A, W_U1)[c - 1] - W(A, W_U1)[c])));
    } else {
      const double thkdfu = A.delt1 * A.thkdfu[c];
      f = mn(flxhi, mx(flxlo, thkdfu * (pk[c - 1] - pk[c])));
    }
    uf[c] = f;
    uk1[c] = uk1[c] + f * dtinv;
    uk[c] = uk[c] - f * dtinv;
  }
  if (mk & kIV) {
    double *vf = W(A, W_VF);
    double flxhi = g, flxlo = -sG[ty - 1][tx];
    double f;
    if (bih) {
      const double hs = sH[ty - 1][tx], h = sH[ty][tx];
      flxhi = mn(flxhi, vf[c] + (iflip == 0 ? hs : h));
      flxlo = mx(flxlo, vf[c] - (iflip == 0 ? h : hs));
      const double thkdfv = A.delt1 * A.thkdfv[c];
      f = mn(flxhi, mx(flxlo, thkdfv * (W(A, W_U2)[c - ld] - W(A, W_U2)[c])));
    } else {
      const double thkdfv = A.delt1 * A.thkdfv[c];
      f = mn(flxhi, mx(flxlo, thkdfv * (pk[c - ld] - pk[c])));
    }
    vf[c] = f;
    vk1[c] = vk1[c] + f * dtinv;
    vk[c] = vk[c] - f * dtinv;
  }
}

// :905-920 at margin 4: move interface k (1-based)
__global__ void cn_thk_p(const CnuityArgs A, int k) {
  Cell x;
  if (!cell_of(A, 4, x)) return;
  const long long c = x.c, ld = A.ld1;
  if (!(A.msk[c] & kIP)) return;
  double *pk = A.p + (long long)(k - 1) * A.slice;
  const double *uf = W(A, W_UF), *vf = W(A, W_VF);
  W(A, W_POLD)[c] = pk[c];
  pk[c] = pk[c] - ((uf[c + 1] - uf[c]) + (vf[c + ld] - vf[c])) * A.scp2i[c];
}

// :925-950 at margin 4: interfaces kept ordered, dp(n) from p
__global__ void cn_thk_final(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 4, x)) return;
  const long long c = x.c, sl = A.slice;
  if (!(A.msk[c] & kIP)) return;
  const int nn = A.n - 1;
  for (int k = 0; k < A.kdm; k++) {
    double *p1 = A.p + (long long)(k + 1) * sl + c;
    const double p0 = A.p[(long long)k * sl + c];
    if (*p1 < p0) *p1 = p0;
    A.dp[((long long)k + (long long)nn * A.kdm) * sl + c] = *p1 - p0;
  }
}

// :1326-1348 at margin 0: cumulative fluxes
__global__ void cn_cumul(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 0, x)) return;
  const long long c = x.c, sl = A.slice;
  const uint8_t mk = A.msk[c];
  const int nn = A.n - 1;
  for (int k = 0; k < A.kdm; k++) {
    const long long ck = (long long)k * sl + c;
    if (mk & kIU) A.uflxav[ck] = A.uflxav[ck] + A.uflx[ck];
    if (mk & kIV) A.vflxav[ck] = A.vflxav[ck] + A.vflx[ck];
    if (mk & kIP) A.dpav[ck] = A.dpav[ck] + A.dp[((long long)k + (long long)nn * A.kdm) * sl + c];
  }
}

// :1350-1385 at margin 1: btrmas restoring (dp back to dp')
__global__ void cn_btrmas(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 1, x)) return;
  const long long c = x.c, sl = A.slice;
  if (!(A.msk[c] & kIP)) return;
  const int nn = A.n - 1;
  const double cnt = A.p[(long long)A.kdm * sl + c] / A.pbot[c];
  A.onetacnt[c] = cnt;
  double *dn = A.dp + (long long)nn * A.kdm * sl + c;
  if (cnt > kEpsilCn) {
    const double q = 1.0 / cnt;
    for (int k = 0; k < A.kdm; k++) {
      dn[(long long)k * sl] = dn[(long long)k * sl] * q;
      A.p[(long long)(k + 1) * sl + c] = A.p[(long long)k * sl + c] + dn[(long long)k * sl];
    }
  } else {
    dn[0] = A.pbot[c];
    A.p[sl + c] = A.p[c] + dn[0];
    for (int k = 1; k < A.kdm; k++) {
      dn[(long long)k * sl] = 0.0;
      A.p[(long long)(k + 1) * sl + c] = A.p[(long long)k * sl + c] + dn[(long long)k * sl];
    }
  }
}

// :1387-1410 at margin 6: Robert-Asselin filter of dp
__global__ void cn_ra(const CnuityArgs A) {
  Cell x;
  if (!cell_of(A, 6, x)) return;
  const long long c = x.c, sl = A.slice;
  if (!(A.msk[c] & kIP)) return;
  const int mm = A.m - 1, nn = A.n - 1;
  for (int k = 0; k < A.kdm; k++) {
    const long long om = ((long long)k + (long long)mm * A.kdm) * sl + c, on = ((long long)k + (long long)nn * A.kdm) * sl + c;
    const double dpold = A.dpo[on], dpmid = A.dp[om], dpnew = A.dp[on];
    const double q = 0.5 * A.ra2fac * (dpold + dpnew - 2.0 * dpmid);
    A.dpo[om] = dpmid;
    A.dp[om] = dpmid + q;
  }
}

dim3 grid_for(const CnuityArgs &a, int M) {
  return dim3((unsigned)((a.ii + 2 * M + kTX - 1) / kTX), (unsigned)((a.jj + 2 * M + kTY - 1) / kTY));
}

}  // namespace

size_t cnuity_work_slices() { return W_N; }

cudaError_t launch_cnuity_layers(const CnuityArgs &a, int *launches, cudaStream_t s) {
  const dim3 b(kTX, kTY);
  int nl = 0;
  cn_init<<<grid_for(a, 6), b, 0, s>>>(a);
  nl++;
  for (int k = 0; k < a.kdm; k++) {  // loop 76
    if (a.btrmas) {
      cn_flux<true><<<grid_for(a, 5), b, 0, s>>>(a, k);
      cn_low<true><<<grid_for(a, 4), b, 0, s>>>(a, k);
    } else {
      cn_flux<false><<<grid_for(a, 5), b, 0, s>>>(a, k);
      cn_low<false><<<grid_for(a, 4), b, 0, s>>>(a, k);
    }
    cn_ratio<<<grid_for(a, 4), b, 0, s>>>(a, k);
    cn_clip<<<grid_for(a, 3), b, 0, s>>>(a, k);
    cn_update<<<grid_for(a, 2), b, 0, s>>>(a, k, 2, a.kdm + k);
    nl += 5;
  }
  *launches += nl;
  return cudaGetLastError();
}

cudaError_t launch_cnuity_rest(const CnuityArgs &a, int *launches, cudaStream_t s) {
  const dim3 b(kTX, kTY);
  int nl = 0;
  if (!a.btrmas) {
    cn_rpb<<<grid_for(a, 2), b, 0, s>>>(a);
    nl++;
    for (int k = 0; k < a.kdm; k++) {  // loop 77
      cn_btflux<<<grid_for(a, 1), b, 0, s>>>(a, k);
      cn_update<<<grid_for(a, 0), b, 0, s>>>(a, k, 0, -1);
      nl += 2;
    }
    cn_bottom<<<grid_for(a, 0), b, 0, s>>>(a);
    nl++;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (a.thk == 4 || a.thk == 2) {
    const int bih = a.thk == 4, iflip = a.nstep % 2;
    const int nb = a.nb;
    e = launch_xctilr(a.dp + (long long)(a.n - 1) * a.kdm * a.slice, a.slice, a.kdm, a.ii, a.jj, nb, a.ld1, 6, 6,
                      a.nreg, s);
    if (e == cudaSuccess) e = launch_xctilr(a.p + a.slice, a.slice, a.kdm, a.ii, a.jj, nb, a.ld1, 6, 6, a.nreg, s);
    if (e != cudaSuccess) return e;
    nl += 2;
    cn_thk_init<<<grid_for(a, 6), b, 0, s>>>(a, bih, iflip);
    nl++;
    const int k0 = bih ? (iflip ? a.kdm : 2) : 2, k1 = bih ? (iflip ? 2 : a.kdm) : a.kdm, dk = k1 >= k0 ? 1 : -1;
    for (int k = k0;; k += dk) {
      if (bih) {
        cn_thk_util<<<grid_for(a, 5), b, 0, s>>>(a, k);
        nl++;
      }
      cn_thk_flux<<<grid_for(a, 4), b, 0, s>>>(a, k, bih, iflip);
      cn_thk_p<<<grid_for(a, 4), b, 0, s>>>(a, k);
      nl += 2;
      if (k == k1) break;
    }
    cn_thk_final<<<grid_for(a, 4), b, 0, s>>>(a);
    nl++;
  }
  if (a.uflxav && a.vflxav && a.dpav) {
    cn_cumul<<<grid_for(a, 0), b, 0, s>>>(a);
    nl++;
  }
  if (a.btrmas) {
    cn_btrmas<<<grid_for(a, 1), b, 0, s>>>(a);
    nl++;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_xctilr(a.dp + (long long)(a.n - 1) * a.kdm * a.slice, a.slice, a.kdm, a.ii, a.jj, a.nb, a.ld1, 6, 6,
                    a.nreg, s);
  if (e != cudaSuccess) return e;
  cn_ra<<<grid_for(a, 6), b, 0, s>>>(a);
  nl += 2;
  *launches += nl;
  return cudaGetLastError();
}

}  // namespace hyc
