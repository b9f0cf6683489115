// hyc_tile.cuh -- fused shared-memory tile kernel for advem's schemes (FP64).
//
// One CTA owns an output tile of TX x TY cells of one layer and stages a
// region of (TX+6) x (TY+6) cells in shared memory: every scheme here (PCM,
// MPDATA, FCT2, FCT4) needs inputs at most 3 cells from the cells it
// updates (fld_new(i) <- limiter ratios at i+-1 <- low-order bounds at i+-2
// <- 5-point extrema of fld at i+-3).  All stages of a scheme then run out
// of shared memory with a shrinking valid region, and only the updated
// field goes back to HBM.  The per-layer quantities (fluxes, thicknesses,
// reciprocal thickness, metrics, masks) are staged once and reused by every
// tracer of the layer.
//
// Stage-to-reference map (FCT2, mod_tsadvc.F90:645-997):
//   S1  upwind face fluxes                         :686-720 (+ :738-758)
//   S2  5-pt extrema, low-order fldlo, fmxlo/fmnlo :778-797
//   S3  high-order minus low-order flux fax/fay    :817-855
//   S4  Zalesak bounds, famax/famin, rp/rm         :863-909
//   S5  flux limiting                              :922-946
//   S6  corrected update, clip to [fqmin,fqmax]    :962-982
// Face fluxes are stored as zero on faces that are not between two sea
// cells; this is what the reference's section-edge zeroing
// (mod_tsadvc.F90:738-758) produces for every face its stencils read.
//
// Arithmetic keeps the reference's order of operations with no contraction
// (this file is compiled with -fmad=false); the only rewritten operation is
// division by the layer thickness, which uses div_rcp (bit-identical to
// IEEE division).
//
// The region is staged by TMA (one box per array, one mbarrier, bounded
// waits) when the launch carries tensor maps and the shape allows it
// (TileGeom::TMA), else by plain loads.
#pragma once
#include <cuda.h>

#include "hyc_args.h"
#include "hyc_device.cuh"
#include "hyc_tma.cuh"

namespace hyc {

// Loop over the rectangle [a0,a1) x [b0,b1) of the region, spread over the CTA.
template <int RX, class F>
__device__ __forceinline__ void for_rect(int a0, int a1, int b0, int b1, F f) {
  const int w = a1 - a0;
  const int n = w * (b1 - b0);
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    int bb = t / w;
    int aa = t - bb * w;
    f(a0 + aa, b0 + bb, (b0 + bb) * RX + a0 + aa);
  }
}

template <int SCHEME, int TX, int TY>
__global__ void __launch_bounds__(256, 1) advect_tile_kernel(const TileArgs A) {
  using G = TileGeom<TX, TY>;
  constexpr int RX = G::RX, RW = G::RW, RY = G::RY, N = G::N, NR = G::NR;
  extern __shared__ __align__(16) double sm[];
  __shared__ uint64_t bar;

  const int tile = blockIdx.x;
  const int k = blockIdx.y;  // 0-based layer
  const int tyi = tile / A.ntx, txi = tile - tyi * A.ntx;
  const int i0 = 1 + txi * TX, j0 = 1 + tyi * TY;  // first output cell (Fortran index)
  const int ib0 = i0 - 3, jb0 = j0 - 3;            // region origin
  const int nb = A.nbdy, ld1 = A.ld1;
  const int x0 = ib0 + nb - 1, y0 = jb0 + nb - 1;  // padded column / row of the region origin
  const int off = x0 & 1;                           // TMA boxes start at the even column x0 - off
  double *sal = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(sm) + 127) & ~uintptr_t(127));
  double *U = sal + off, *V = U + N, *FCO = V + N, *FCN = FCO + N, *HN = FCN + N, *RH = HN + N, *SCL = RH + N,
         *SCI = SCL + N;
  double *FLD = SCI + N, *FLDC = FLD + N, *FX = FLDC + N, *FY = FX + N, *FLO = FY + N, *FXL = FLO + N,
         *FNL = FXL + N, *RP = FNL + N, *RM = RP + N, *QX = RM + N, *QN = QX + N;
  uint8_t *MSK = reinterpret_cast<uint8_t *>(sal + G::NARR * N);
  const CUtensorMap *tm = G::TMA ? reinterpret_cast<const CUtensorMap *>(A.tmaps) : nullptr;
  const long long sl = A.slice;
  const double dt2 = A.dt2;
  uint32_t ph = 0;  // completed phases of bar
  if (tm && threadIdx.x == 0) {
    tma::bar_init(&bar, 1);
    tma::fence_bar_init();
  }
  // all threads wait for the mbarrier's next phase; if any gave up, the
  // copies in flight land (bounded) and the CTA stops
  auto landed = [&]() -> bool {
    const bool ok = tma::wait(&bar, ph & 1u, A.err);
    ph++;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) tma::wait(&bar, (ph - 1) & 1u, nullptr);
      return false;
    }
    return true;
  };

  // ---- stage per-layer inputs -------------------------------------------------
  const double *uk = A.mode == 0 ? A.uflx + k * sl : A.uflx;
  const double *vk = A.mode == 0 ? A.vflx + k * sl : A.vflx;
  if (tm) {
    __syncthreads();  // the mbarrier is initialised
    if (threadIdx.x == 0) {
      const int zk = A.mode == 0 ? k : 0;
      tma::expect_tx(&bar, (A.tm_has3 ? 6u : 5u) * G::BOX);
      tma::load3(U - off, tm + 0, &bar, x0 - off, y0, zk);
      tma::load3(V - off, tm + 1, &bar, x0 - off, y0, zk);
      tma::load3(FCN - off, tm + 2, &bar, x0 - off, y0, zk);
      if (A.tm_has3) tma::load3(FCO - off, tm + 3, &bar, x0 - off, y0, 0);
      tma::load3(SCL - off, tm + 4, &bar, x0 - off, y0, 0);
      tma::load3(SCI - off, tm + 5, &bar, x0 - off, y0, 0);
    }
    for (int t = threadIdx.x; t < NR; t += blockDim.x) {  // masks (bytes) by plain loads meanwhile
      int bb = t / RX, aa = t - bb * RX;
      int i = ib0 + aa, j = jb0 + bb;
      bool in = (i >= 1 - nb) && (i <= A.ii + nb) && (j >= 1 - nb) && (j <= A.jj + nb);
      MSK[t] = in ? A.msk[(long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1] : 0;
      if (!A.tm_has3) FCO[t] = 1.0;  // tsadvc without btrmas: onetamas = 1
    }
    if (!landed()) return;
  }
  for (int t = threadIdx.x; t < (tm ? 0 : NR); t += blockDim.x) {
    int bb = t / RX, aa = t - bb * RX;
    int i = ib0 + aa, j = jb0 + bb;
    bool in = (i >= 1 - nb) && (i <= A.ii + nb) && (j >= 1 - nb) && (j <= A.jj + nb);
    long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
    MSK[t] = in ? A.msk[o] : 0;
    U[t] = in ? uk[o] : 0.0;
    V[t] = in ? vk[o] : 0.0;
    SCL[t] = in ? A.scal[o] : 1.0;
    SCI[t] = in ? A.scali[o] : 1.0;
    if (A.mode == 0) {
      FCN[t] = in ? A.dpn[k * sl + o] : 0.0;  // dp(:,:,k,n) for now
      FCO[t] = (in && A.oneta_n) ? A.oneta_n[o] : 1.0;  // onetamas(:,:,m)
    } else {
      FCO[t] = in ? A.fco[o] : 0.0;
      FCN[t] = in ? A.fcn[o] : 0.0;
    }
  }
  __syncthreads();
  if (A.mode == 0) {
    // thickness prep, mod_tsadvc.F90:1905-1942 (in place; each cell reads
    // only its own FCO/FCN and the fluxes on its faces):
    //   util1 = max(onetamas*dp + flxdiv, 0), util2 = max(onetamas*dp, 0)
    // valid on [0,RX-1) x [0,RY-1) (the face at a+1, b+1 is needed).
    for (int t = threadIdx.x; t < NR; t += blockDim.x) {
      int bb = t / RX, aa = t - bb * RX;
      double o = FCO[t] * FCN[t];  // onetamas*dp
      double fdv = 0.0;
      if (aa < RX - 1 && bb < RY - 1) {
        if (A.ufco) {
          // the divergence of the smoothed layer-1 fluxes, read as the
          // staged ones would be (0 outside the array)
          const int i = ib0 + aa, j = jb0 + bb;
          auto at = [&](const double *f, int ic, int jc) -> double {
            const bool in = (ic >= 1 - nb) && (ic <= A.ii + nb) && (jc >= 1 - nb) && (jc <= A.jj + nb);
            return in ? f[(long long)(ic + nb - 1) + (long long)(jc + nb - 1) * ld1] : 0.0;
          };
          fdv = ((at(A.ufco, i + 1, j) - at(A.ufco, i, j)) + (at(A.vfco, i, j + 1) - at(A.vfco, i, j))) * dt2 *
                SCI[t];
        } else {
          fdv = ((U[t + 1] - U[t]) + (V[t + RX] - V[t])) * dt2 * SCI[t];
        }
      }
      FCO[t] = kmax(o + fdv, 0.0);
      FCN[t] = kmax(o, 0.0);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < NR; t += blockDim.x) {
    double hn = FCN[t] + kOnemu;
    HN[t] = hn;
    RH[t] = __drcp_rn(hn);
  }
  __syncthreads();

  // ---- loop over the fields advected in this layer ---------------------------
  for (int fi = 0; fi < A.nfld; fi++) {
    const FieldDesc fd = A.f[fi];
    if (k + 1 > fd.kmax || k + 1 < fd.kmin) continue;  // uniform across the CTA
    const double *fn = fd.nbase + (long long)(k + fd.k_off) * sl;
    const double *fm = fd.mbase + (long long)(k + fd.k_off) * sl;
    const double posdef = fd.posdef;
    constexpr bool CENTRE = SCHEME != kPCM && SCHEME != kMPDATA;
    if (tm) {  // the previous field's readers passed the barrier that ends its loop
      if (threadIdx.x == 0) {
        tma::fence_proxy_async();
        tma::expect_tx(&bar, (CENTRE ? 2u : 1u) * G::BOX);
        tma::load3(FLD - off, tm + 6 + 2 * fi, &bar, x0 - off, y0, k + fd.k_off);
        if (CENTRE) tma::load3(FLDC - off, tm + 7 + 2 * fi, &bar, x0 - off, y0, k + fd.k_off);
      }
    }
    for (int t = threadIdx.x; t < NR; t += blockDim.x) {
      if (!tm) {
        int bb = t / RX, aa = t - bb * RX;
        int i = ib0 + aa, j = jb0 + bb;
        bool in = (i >= 1 - nb) && (i <= A.ii + nb) && (j >= 1 - nb) && (j <= A.jj + nb);
        long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
        FLD[t] = in ? fn[o] : 0.0;
        if (CENTRE) FLDC[t] = in ? fm[o] : 0.0;
      }
      FX[t] = 0.0;
      FY[t] = 0.0;
    }
    if (tm && !landed()) return;
    __syncthreads();

    // S1: low-order (upwind) face fluxes on x-faces [1,RX-1] x rows [1,RY-1)
    // and y-faces cols [1,RX-1) x [1,RY-1]; MPDATA adds posdef and tx1/ty1.
    for_rect<RX>(1, RW, 1, RY - 1, [&](int a, int b, int e) {
      if (MSK[e] & kIU) {
        double uu = U[e];
        double q = ge0(uu) ? FLD[e - 1] : FLD[e];
        if (SCHEME == kMPDATA) {
          FXL[e] = .5 * fabs(uu) * (FLD[e] - FLD[e - 1]);  // tx1, :255
          FX[e] = uu * (q + posdef);                        // :261
        } else {
          FX[e] = uu * q;  // :698
        }
      } else if (SCHEME == kMPDATA) {
        FXL[e] = 0.0;
      }
    });
    for_rect<RX>(1, RW - 1, 1, RY, [&](int a, int b, int e) {
      if (MSK[e] & kIV) {
        double vv = V[e];
        double q = ge0(vv) ? FLD[e - RX] : FLD[e];
        if (SCHEME == kMPDATA) {
          FNL[e] = .5 * fabs(vv) * (FLD[e] - FLD[e - RX]);  // ty1, :264
          FY[e] = vv * (q + posdef);
        } else {
          FY[e] = vv * q;
        }
      } else if (SCHEME == kMPDATA) {
        FNL[e] = 0.0;
      }
    });
    __syncthreads();

    if (SCHEME == kPCM) {
      // mod_tsadvc.F90:610-630 on the output cells
      for_rect<RX>(3, RW - 3, 3, RY - 3, [&](int a, int b, int e) {
        int i = ib0 + a, j = jb0 + b;
        if (i > A.ii || j > A.jj) return;
        double c = FLD[e];
        double res = c;
        uint8_t m = MSK[e];
        if (m & kIP) {
          double w = (MSK[e - 1] & kIP) ? FLD[e - 1] : c;
          double ea = (MSK[e + 1] & kIP) ? FLD[e + 1] : c;
          double s = (MSK[e - RX] & kIP) ? FLD[e - RX] : c;
          double nn = (MSK[e + RX] & kIP) ? FLD[e + RX] : c;
          double fmx = kmax(kmax(kmax(kmax(c, w), ea), s), nn);
          double fmn = kmin(kmin(kmin(kmin(c, w), ea), s), nn);
          double fdv = ((FX[e + 1] - FX[e]) + (FY[e + RX] - FY[e])) * dt2 * SCI[e];
          double q = c * (FCO[e] + kOnemu) - fdv;
          res = kmax(fmn, kmin(fmx, div_rcp(q, HN[e], RH[e])));
        }
        A.out[((long long)fi * A.kdm + k) * sl + (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1] = res;
      });
      __syncthreads();
      continue;
    }

    // S2: on cells [1,RX-1) x [1,RY-1): 5-point extrema over sea neighbours
    // (ipim1/ipip1/ipjm1/ipjp1, bigrid.F90:316-333) and the low-order update.
    for_rect<RX>(1, RW - 1, 1, RY - 1, [&](int a, int b, int e) {
      if (!(MSK[e] & kIP)) return;
      double c = FLD[e];
      double w = (MSK[e - 1] & kIP) ? FLD[e - 1] : c;
      double ea = (MSK[e + 1] & kIP) ? FLD[e + 1] : c;
      double s = (MSK[e - RX] & kIP) ? FLD[e - RX] : c;
      double nn = (MSK[e + RX] & kIP) ? FLD[e + RX] : c;
      double fmx = kmax(kmax(kmax(kmax(c, w), ea), s), nn);
      double fmn = kmin(kmin(kmin(kmin(c, w), ea), s), nn);
      double fdv = ((FX[e + 1] - FX[e]) + (FY[e + RX] - FY[e])) * dt2 * SCI[e];
      if (SCHEME == kMPDATA) {
        fmx = fmx + posdef;  // :277-280
        fmn = fmn + posdef;
        double q = (c + posdef) * (FCO[e] + kOnemu) - fdv;  // :350
        FLO[e] = kmax(fmn, kmin(fmx, div_rcp(q, HN[e], RH[e])));
        FLDC[e] = fdv;  // flxdiv, read by neighbours in S3
        QX[e] = fmx;
        QN[e] = fmn;
      } else {
        double q = c * (FCO[e] + kOnemu) - fdv;  // :788
        double lo = kmax(fmn, kmin(fmx, div_rcp(q, HN[e], RH[e])));
        FLO[e] = lo;
        double cc = FLDC[e];
        FXL[e] = kmax(kmax(c, cc), lo);  // fmxlo, :792
        FNL[e] = kmin(kmin(c, cc), lo);  // fmnlo, :793
      }
    });
    __syncthreads();

    // S3: antidiffusive fluxes on x-faces [2,RX-2] x rows [2,RY-2) and
    // y-faces cols [2,RX-2) x [2,RY-2].
    for_rect<RX>(2, RW - 1, 2, RY - 2, [&](int a, int b, int e) {
      uint8_t m = MSK[e];
      if (!(m & kIU)) return;
      double uu = U[e];
      if (SCHEME == kMPDATA) {  // :377-381
        double fco2 = FCO[e] + FCO[e - 1];
        double fcn2 = FCN[e] + FCN[e - 1];
        FX[e] = FXL[e] - uu * (FLDC[e] + FLDC[e - 1]) / ((fco2 + fcn2) + kOnemu);
      } else if (SCHEME == kFCT4 && (MSK[e - 1] & kIU) && (MSK[e + 1] & kIU)) {  // :1540-1541
        const double ft14 = 7.0 / 12.0, ft24 = -1.0 / 12.0;
        double fhx = uu * (ft14 * (FLDC[e] + FLDC[e - 1]) + ft24 * (FLDC[e + 1] + FLDC[e - 2]));
        FX[e] = fhx - FX[e];
      } else {  // :824-825
        double fhx = uu * 0.5 * (FLDC[e] + FLDC[e - 1]);
        FX[e] = fhx - FX[e];
      }
    });
    for_rect<RX>(2, RW - 2, 2, RY - 1, [&](int a, int b, int e) {
      uint8_t m = MSK[e];
      if (!(m & kIV)) return;
      double vv = V[e];
      if (SCHEME == kMPDATA) {  // :383-387
        double fco2 = FCO[e] + FCO[e - RX];
        double fcn2 = FCN[e] + FCN[e - RX];
        FY[e] = FNL[e] - vv * (FLDC[e] + FLDC[e - RX]) / ((fco2 + fcn2) + kOnemu);
      } else if (SCHEME == kFCT4 && (MSK[e - RX] & kIV) && (MSK[e + RX] & kIV)) {  // :1551-1552
        const double ft14 = 7.0 / 12.0, ft24 = -1.0 / 12.0;
        double fhy = vv * (ft14 * (FLDC[e] + FLDC[e - RX]) + ft24 * (FLDC[e + RX] + FLDC[e - 2 * RX]));
        FY[e] = fhy - FY[e];
      } else {
        double fhy = vv * 0.5 * (FLDC[e] + FLDC[e - RX]);
        FY[e] = fhy - FY[e];
      }
    });
    __syncthreads();

    // S4: limiter ratios on cells [2,RX-2) x [2,RY-2)
    for_rect<RX>(2, RW - 2, 2, RY - 2, [&](int a, int b, int e) {
      uint8_t m = MSK[e];
      if (!(m & kIP)) return;
      if (SCHEME == kMPDATA) {  // :411-419
        double fx0 = FX[e], fx1 = FX[e + 1], fy0 = FY[e], fy1 = FY[e + RX];
        double flxdp = neg0(fx1) - pos0(fx0);
        double flxdn = pos0(fx1) - neg0(fx0);
        double flydp = neg0(fy1) - pos0(fy0);
        double flydn = pos0(fy1) - neg0(fy0);
        double lo = FLO[e];
        double fs = FCN[e] * SCL[e];
        RP[e] = (QX[e] - lo) * fs / ((kOnemu - (flxdp + flydp)) * dt2);
        RM[e] = (lo - QN[e]) * fs / ((kOnemu + (flxdn + flydn)) * dt2);
        return;
      }
      const bool mw = MSK[e - 1] & kIP, me = MSK[e + 1] & kIP, ms = MSK[e - RX] & kIP, mn = MSK[e + RX] & kIP;
      double fqmax = FXL[e], fqmin = FNL[e];
      // fqmax = max(fmxlo(i,j),fmxlo(ia,j),fmxlo(ib,j),fmxlo(i,ja),fmxlo(i,jb)), :876-879
      fqmax = kmax(fqmax, mw ? FXL[e - 1] : FXL[e]);
      fqmax = kmax(fqmax, me ? FXL[e + 1] : FXL[e]);
      fqmax = kmax(fqmax, ms ? FXL[e - RX] : FXL[e]);
      fqmax = kmax(fqmax, mn ? FXL[e + RX] : FXL[e]);
      fqmin = kmin(fqmin, mw ? FNL[e - 1] : FNL[e]);
      fqmin = kmin(fqmin, me ? FNL[e + 1] : FNL[e]);
      fqmin = kmin(fqmin, ms ? FNL[e - RX] : FNL[e]);
      fqmin = kmin(fqmin, mn ? FNL[e + RX] : FNL[e]);
      // ib=ipip1, jb=ipjp1: a sea cell with land to the E (N) reads its own
      // west (south) face twice, mod_tsadvc.F90:880-883.
      double fxa = FX[e], fxb = me ? FX[e + 1] : FX[e];
      double fya = FY[e], fyb = mn ? FY[e + RX] : FY[e];
      double famax = pos0(fxa) - neg0(fxb) + pos0(fya) - neg0(fyb);
      double famin = pos0(fxb) - neg0(fxa) + pos0(fyb) - neg0(fya);
      double lo = FLO[e];
      double qdt2 = 1.0 / dt2;
      double rp = 0.0, rm = 0.0;
      if (gt0(famax)) {
        double qp = (fqmax - lo) * FCN[e] * SCL[e] * qdt2;
        rp = klt(qp, famax) ? qp / famax : 1.0;
      }
      if (gt0(famin)) {
        double qm = (lo - fqmin) * FCN[e] * SCL[e] * qdt2;
        rm = klt(qm, famin) ? qm / famin : 1.0;
      }
      RP[e] = rp;
      RM[e] = rm;
      QX[e] = fqmax;
      QN[e] = fqmin;
    });
    __syncthreads();

    // S5: limit fluxes on x-faces [3,RX-3] x rows [3,RY-3) and y-faces
    for_rect<RX>(3, RW - 2, 3, RY - 3, [&](int a, int b, int e) {
      if (!(MSK[e] & kIU)) return;
      double f = FX[e];
      if (SCHEME == kMPDATA) {  // :440-441
        FX[e] = pos0(f) * kmin(kmin(1.0, RP[e]), RM[e - 1]) + neg0(f) * kmin(kmin(1.0, RP[e - 1]), RM[e]);
      } else {  // :929-934
        double fact = lt0(f) ? kmin(RP[e - 1], RM[e]) : kmin(RP[e], RM[e - 1]);
        FX[e] = fact * f;
      }
    });
    for_rect<RX>(3, RW - 3, 3, RY - 2, [&](int a, int b, int e) {
      if (!(MSK[e] & kIV)) return;
      double f = FY[e];
      if (SCHEME == kMPDATA) {
        FY[e] = pos0(f) * kmin(kmin(1.0, RP[e]), RM[e - RX]) + neg0(f) * kmin(kmin(1.0, RP[e - RX]), RM[e]);
      } else {
        double fact = lt0(f) ? kmin(RP[e - RX], RM[e]) : kmin(RP[e], RM[e - RX]);
        FY[e] = fact * f;
      }
    });
    __syncthreads();

    // S6: corrected update on the output cells, :962-982 (MPDATA :465-486)
    for_rect<RX>(3, RW - 3, 3, RY - 3, [&](int a, int b, int e) {
      int i = ib0 + a, j = jb0 + b;
      if (i > A.ii || j > A.jj) return;
      double res = FLD[e];
      if (MSK[e] & kIP) {
        double fdv = ((FX[e + 1] - FX[e]) + (FY[e + RX] - FY[e])) * dt2 * SCI[e];
        res = kmax(QN[e], kmin(QX[e], FLO[e] - div_rcp(fdv, HN[e], RH[e])));
        if (SCHEME == kMPDATA) res = res - posdef;
      }
      A.out[((long long)fi * A.kdm + k) * sl + (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1] = res;
    });
    __syncthreads();
  }
}

}  // namespace hyc
