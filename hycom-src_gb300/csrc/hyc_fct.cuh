// hyc_fct.cuh -- FP64 FCT2/FCT4 tile kernel tuned for GB300's FP64 pipe.
//
// Same stages and arithmetic as the generic tile kernel (hyc_tile.cuh; map to
// mod_tsadvc.F90:645-997 for FCT2 and :1370-1706 for FCT4), reorganised so
// that two CTAs fit on an SM (the FP64 pipe needs more resident warps to
// hide its latency than one 256-thread CTA gives):
//   * 15 shared arrays instead of 19: fmxlo/fmnlo overwrite fld/fldc in
//     place once fld and fldc are dead, and fqmax/fqmin live in registers of
//     the thread that later updates the same output cell;
//   * fco+onemu is formed once per cell (the reference forms it per field);
//   * the stage loops have compile-time bounds and are unrolled, so a
//     thread's cells interleave (more independent FP64 work in flight).
// The region is staged by TMA (cp.async.bulk.tensor, one box per array and
// one mbarrier, every wait bounded) when the launch carries tensor maps,
// else by plain loads.  Only sea cells of the interior are written to the
// output slice.
#pragma once
#include <cuda.h>

#include "hyc_args.h"
#include "hyc_device.cuh"
#include "hyc_tma.cuh"

namespace hyc {

// The region is RW x RY cells (the TX x TY output cells and a 3-cell ring).
// Its rows are stored RX = TX + 8 doubles apart, an even count, so that a
// TMA box row is a multiple of 16 bytes and the box can start on the even
// padded column at or before the region's first one (x coordinates of a
// box must be even for 8-byte elements); the region then sits at offset
// off = 0 or 1 in each array's slot.
template <int TX, int TY>
struct FctGeom {
  static constexpr int RW = TX + 6, RX = TX + 8, RY = TY + 6;
  static constexpr int NR = RX * RY;                     // cells of a staged box
  static constexpr int N = (NR + 1 + 15) / 16 * 16;      // one array's slot (128-byte multiple)
  static constexpr int NARR = 15;  // U V FCN HO HN RH SCL SCI | FLD FLDC FX FY FLO RP RM
  static constexpr unsigned BOX = NR * 8;                // bytes of one TMA box
  static constexpr size_t smem_bytes = 128 + (size_t)NARR * N * sizeof(double) + ((NR + 15) / 16) * 16;
};

// Compile-time rectangle [A0,A1) x [B0,B1) of a region of width RX, spread
// over 256 threads; f(a, b, e, it) with e = b*RX + a and it the iteration.
template <int RX, int A0, int A1, int B0, int B1, class F>
__device__ __forceinline__ void rect(F &&f) {
  constexpr int W = A1 - A0;
  constexpr int NN = W * (B1 - B0);
  constexpr int IT = (NN + 255) / 256;
#pragma unroll
  for (int it = 0; it < IT; it++) {
    const int t = threadIdx.x + it * 256;
    if (NN % 256 == 0 || t < NN) {
      const int bb = t / W;
      const int aa = t - bb * W;
      f(A0 + aa, B0 + bb, (B0 + bb) * RX + A0 + aa, it);
    }
  }
}

// One tile (tile index, 0-based layer k) of one basin; sm is the CTA's
// dynamic shared memory (FctGeom<TX,TY>::smem_bytes), bar its mbarrier and
// ph the count of the mbarrier's completed phases (uniform over the CTA).
// False when a TMA wait gave up (A.err is set; the CTA stops).
template <int SCHEME, int TX, int TY>
__device__ __forceinline__ bool fct_tile_body(const TileArgs &A, const int tile, const int k, double *sm,
                                              uint64_t *bar, uint32_t &ph) {
  using G = FctGeom<TX, TY>;
  constexpr int RX = G::RX, RW = G::RW, RY = G::RY, N = G::N, NR = G::NR;
  constexpr int NOUT_IT = (TX * TY + 255) / 256;
  const int tyi = tile / A.ntx, txi = tile - tyi * A.ntx;
  const int ib0 = 1 + txi * TX - 3, jb0 = 1 + tyi * TY - 3;  // region origin (Fortran index)
  const int nb = A.nbdy, ld1 = A.ld1, ii = A.ii, jj = A.jj;
  const int x0 = ib0 + nb - 1, y0 = jb0 + nb - 1;  // padded column / row of the region origin
  const int off = x0 & 1;                           // TMA boxes start at the even column x0 - off
  double *sal = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(sm) + 127) & ~uintptr_t(127));
  double *U = sal + off, *V = U + N, *FCN = V + N, *HO = FCN + N, *HN = HO + N, *RH = HN + N, *SCL = RH + N,
         *SCI = SCL + N;
  double *FLD = SCI + N, *FLDC = FLD + N, *FX = FLDC + N, *FY = FX + N, *FLO = FY + N, *RP = FLO + N,
         *RM = RP + N;
  uint8_t *MSK = reinterpret_cast<uint8_t *>(sal + G::NARR * N);
  const CUtensorMap *tm = reinterpret_cast<const CUtensorMap *>(A.tmaps);
  const long long sl = A.slice;
  const double dt2 = A.dt2;
  // all threads wait for the mbarrier's next phase; if any gave up, let the
  // copies in flight land (bounded) and report failure
  auto landed = [&]() -> bool {
    const bool ok = tma::wait(bar, ph & 1u, A.err);
    ph++;
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) tma::wait(bar, (ph - 1) & 1u, nullptr);
      return false;
    }
    return true;
  };

  // ---- per-layer inputs ------------------------------------------------------
  if (tm) {
    __syncthreads();  // the previous item's readers of these slots are done
    if (threadIdx.x == 0) {
      tma::fence_proxy_async();
      const int zk = A.mode == 0 ? k : 0;
      tma::expect_tx(bar, (A.tm_has3 ? 6u : 5u) * G::BOX);
      tma::load3(U - off, tm + 0, bar, x0 - off, y0, zk);
      tma::load3(V - off, tm + 1, bar, x0 - off, y0, zk);
      tma::load3(FCN - off, tm + 2, bar, x0 - off, y0, zk);
      if (A.tm_has3) tma::load3(HO - off, tm + 3, bar, x0 - off, y0, 0);
      tma::load3(SCL - off, tm + 4, bar, x0 - off, y0, 0);
      tma::load3(SCI - off, tm + 5, bar, x0 - off, y0, 0);
    }
    for (int t = threadIdx.x; t < NR; t += 256) {  // masks (bytes) by plain loads meanwhile
      const int bb = t / RX, aa = t - bb * RX;
      const int i = ib0 + aa, j = jb0 + bb;
      const bool in = (i >= 1 - nb) && (i <= ii + nb) && (j >= 1 - nb) && (j <= jj + nb);
      MSK[t] = in ? A.msk[(long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1] : 0;
      if (!A.tm_has3) HO[t] = 1.0;  // tsadvc without btrmas: onetamas = 1
    }
    if (!landed()) return false;
  } else {
    const double *uk = A.mode == 0 ? A.uflx + k * sl : A.uflx;
    const double *vk = A.mode == 0 ? A.vflx + k * sl : A.vflx;
    for (int t = threadIdx.x; t < NR; t += 256) {
      const int bb = t / RX, aa = t - bb * RX;
      const int i = ib0 + aa, j = jb0 + bb;
      const bool in = (i >= 1 - nb) && (i <= ii + nb) && (j >= 1 - nb) && (j <= jj + nb);
      const long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
      MSK[t] = in ? A.msk[o] : 0;
      U[t] = in ? uk[o] : 0.0;
      V[t] = in ? vk[o] : 0.0;
      SCL[t] = in ? A.scal[o] : 1.0;
      SCI[t] = in ? A.scali[o] : 1.0;
      if (A.mode == 0) {
        FCN[t] = in ? A.dpn[k * sl + o] : 0.0;            // dp(:,:,k,n)
        HO[t] = (in && A.oneta_n) ? A.oneta_n[o] : 1.0;   // onetamas(:,:,m)
      } else {
        HO[t] = in ? A.fco[o] : 0.0;
        FCN[t] = in ? A.fcn[o] : 0.0;
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < NR; t += 256) {
    const int bb = t / RX, aa = t - bb * RX;
    double fco, fcn;
    if (A.mode == 0) {  // mod_tsadvc.F90:1931-1938
      const double o = HO[t] * FCN[t];
      double fdv = 0.0;
      if (aa < RX - 1 && bb < RY - 1) {
        if (A.ufco) {
          // isopycnic layer 1: the divergence of the smoothed fluxes, read as
          // the staged ones would be (0 outside the array)
          const int i = ib0 + aa, j = jb0 + bb;
          auto at = [&](const double *f, int ic, int jc) -> double {
            const bool in = (ic >= 1 - nb) && (ic <= ii + nb) && (jc >= 1 - nb) && (jc <= jj + nb);
            return in ? f[(long long)(ic + nb - 1) + (long long)(jc + nb - 1) * ld1] : 0.0;
          };
          fdv = ((at(A.ufco, i + 1, j) - at(A.ufco, i, j)) + (at(A.vfco, i, j + 1) - at(A.vfco, i, j))) * dt2 *
                SCI[t];
        } else {
          fdv = ((U[t + 1] - U[t]) + (V[t + RX] - V[t])) * dt2 * SCI[t];
        }
      }
      fco = kmax(o + fdv, 0.0);
      fcn = kmax(o, 0.0);
    } else {
      fco = HO[t];
      fcn = FCN[t];
    }
    const double hn = fcn + kOnemu;
    FCN[t] = fcn;
    HO[t] = fco + kOnemu;
    HN[t] = hn;
    RH[t] = __drcp_rn(hn);
  }
  __syncthreads();

  const double qdt2 = 1.0 / dt2;  // mod_tsadvc.F90:865
  for (int fi = 0; fi < A.nfld; fi++) {
    const FieldDesc fd = A.f[fi];
    if (k + 1 > fd.kmax || k + 1 < fd.kmin) continue;
    const double *fn = fd.nbase + (long long)(k + fd.k_off) * sl;
    const double *fm = fd.mbase + (long long)(k + fd.k_off) * sl;
    double *out = A.out + ((long long)fi * A.kdm + k) * sl;
    if (tm) {  // the previous field's readers passed the barrier that ends its loop
      if (threadIdx.x == 0) {
        tma::fence_proxy_async();
        tma::expect_tx(bar, 2u * G::BOX);
        tma::load3(FLD - off, tm + 6 + 2 * fi, bar, x0 - off, y0, k + fd.k_off);
        tma::load3(FLDC - off, tm + 7 + 2 * fi, bar, x0 - off, y0, k + fd.k_off);
      }
      for (int t = threadIdx.x; t < NR; t += 256) {
        FX[t] = 0.0;
        FY[t] = 0.0;
      }
      if (!landed()) return false;
    } else {
      for (int t = threadIdx.x; t < NR; t += 256) {
        const int bb = t / RX, aa = t - bb * RX;
        const int i = ib0 + aa, j = jb0 + bb;
        const bool in = (i >= 1 - nb) && (i <= ii + nb) && (j >= 1 - nb) && (j <= jj + nb);
        const long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
        FLD[t] = in ? fn[o] : 0.0;
        FLDC[t] = in ? fm[o] : 0.0;
        FX[t] = 0.0;
        FY[t] = 0.0;
      }
      __syncthreads();
    }

    // S1: upwind fluxes, :686-720 (zero on faces that are not sea-sea)
    rect<RX, 1, RW, 1, RY - 1>([&](int a, int b, int e, int) {
      if (MSK[e] & kIU) {
        const double uu = U[e];
        FX[e] = uu * (ge0(uu) ? FLD[e - 1] : FLD[e]);
      }
    });
    rect<RX, 1, RW - 1, 1, RY>([&](int a, int b, int e, int) {
      if (MSK[e] & kIV) {
        const double vv = V[e];
        FY[e] = vv * (ge0(vv) ? FLD[e - RX] : FLD[e]);
      }
    });
    __syncthreads();

    // S2: low-order solution on [1,RX-1)^2, :778-791
    rect<RX, 1, RW - 1, 1, RY - 1>([&](int a, int b, int e, int) {
      const uint8_t m = MSK[e];
      if (!(m & kIP)) return;
      const double c = FLD[e];
      const double w = (MSK[e - 1] & kIP) ? FLD[e - 1] : c;
      const double ea = (MSK[e + 1] & kIP) ? FLD[e + 1] : c;
      const double s = (MSK[e - RX] & kIP) ? FLD[e - RX] : c;
      const double n = (MSK[e + RX] & kIP) ? FLD[e + RX] : c;
      const double fmx = kmax(kmax(kmax(kmax(c, w), ea), s), n);
      const double fmn = kmin(kmin(kmin(kmin(c, w), ea), s), n);
      const double fdv = ((FX[e + 1] - FX[e]) + (FY[e + RX] - FY[e])) * dt2 * SCI[e];
      const double q = c * HO[e] - fdv;
      FLO[e] = kmax(fmn, kmin(fmx, div_rcp(q, HN[e], RH[e])));
    });
    __syncthreads();

    // S3: antidiffusive fluxes, :817-855 (FCT4: :1528-1580)
    rect<RX, 2, RW - 1, 2, RY - 2>([&](int a, int b, int e, int) {
      if (!(MSK[e] & kIU)) return;
      const double uu = U[e];
      double fhx;
      if (SCHEME == kFCT4 && (MSK[e - 1] & kIU) && (MSK[e + 1] & kIU)) {
        const double ft14 = 7.0 / 12.0, ft24 = -1.0 / 12.0;
        fhx = uu * (ft14 * (FLDC[e] + FLDC[e - 1]) + ft24 * (FLDC[e + 1] + FLDC[e - 2]));
      } else {
        fhx = uu * 0.5 * (FLDC[e] + FLDC[e - 1]);
      }
      FX[e] = fhx - FX[e];
    });
    rect<RX, 2, RW - 2, 2, RY - 1>([&](int a, int b, int e, int) {
      if (!(MSK[e] & kIV)) return;
      const double vv = V[e];
      double fhy;
      if (SCHEME == kFCT4 && (MSK[e - RX] & kIV) && (MSK[e + RX] & kIV)) {
        const double ft14 = 7.0 / 12.0, ft24 = -1.0 / 12.0;
        fhy = vv * (ft14 * (FLDC[e] + FLDC[e - RX]) + ft24 * (FLDC[e + RX] + FLDC[e - 2 * RX]));
      } else {
        fhy = vv * 0.5 * (FLDC[e] + FLDC[e - RX]);
      }
      FY[e] = fhy - FY[e];
    });
    __syncthreads();

    // fmxlo/fmnlo (:792-793) in place over fld/fldc, now dead
    rect<RX, 1, RW - 1, 1, RY - 1>([&](int a, int b, int e, int) {
      if (!(MSK[e] & kIP)) return;
      const double c = FLD[e], cc = FLDC[e], lo = FLO[e];
      FLD[e] = kmax(kmax(c, cc), lo);
      FLDC[e] = kmin(kmin(c, cc), lo);
    });
    __syncthreads();

    // S4: Zalesak bounds and ratios, :863-909.  Output cells keep
    // fqmax/fqmin in registers for S6 (same thread-to-cell map).
    double qx[NOUT_IT], qn[NOUT_IT];
    auto zalesak = [&](int e, double &fqmax, double &fqmin) {
      const bool mw = MSK[e - 1] & kIP, me = MSK[e + 1] & kIP, ms = MSK[e - RX] & kIP, mn = MSK[e + RX] & kIP;
      fqmax = FLD[e];
      fqmin = FLDC[e];
      fqmax = kmax(fqmax, mw ? FLD[e - 1] : FLD[e]);
      fqmax = kmax(fqmax, me ? FLD[e + 1] : FLD[e]);
      fqmax = kmax(fqmax, ms ? FLD[e - RX] : FLD[e]);
      fqmax = kmax(fqmax, mn ? FLD[e + RX] : FLD[e]);
      fqmin = kmin(fqmin, mw ? FLDC[e - 1] : FLDC[e]);
      fqmin = kmin(fqmin, me ? FLDC[e + 1] : FLDC[e]);
      fqmin = kmin(fqmin, ms ? FLDC[e - RX] : FLDC[e]);
      fqmin = kmin(fqmin, mn ? FLDC[e + RX] : FLDC[e]);
      // ib=ipip1, jb=ipjp1 (:873-875): land to the E/N -> own face twice
      const double fxa = FX[e], fxb = me ? FX[e + 1] : FX[e];
      const double fya = FY[e], fyb = mn ? FY[e + RX] : FY[e];
      const double famax = pos0(fxa) - neg0(fxb) + pos0(fya) - neg0(fyb);
      const double famin = pos0(fxb) - neg0(fxa) + pos0(fyb) - neg0(fya);
      const double lo = FLO[e];
      double rp = 0.0, rm = 0.0;
      if (gt0(famax)) {
        const double qp = (fqmax - lo) * FCN[e] * SCL[e] * qdt2;
        rp = klt(qp, famax) ? qp / famax : 1.0;
      }
      if (gt0(famin)) {
        const double qm = (lo - fqmin) * FCN[e] * SCL[e] * qdt2;
        rm = klt(qm, famin) ? qm / famin : 1.0;
      }
      RP[e] = rp;
      RM[e] = rm;
    };
    rect<RX, 3, RW - 3, 3, RY - 3>([&](int a, int b, int e, int it) {
      if (MSK[e] & kIP) zalesak(e, qx[it], qn[it]);
    });
    {  // the ring [2,RW-2) x [2,RY-2) minus the output cells: ratios only
      constexpr int NRING = 2 * (RW - 4) + 2 * (RY - 6);
      static_assert(NRING <= 256, "ring larger than the CTA");
      const int t = threadIdx.x;
      if (t < NRING) {
        int a, b;
        if (t < RW - 4) { a = 2 + t; b = 2; }
        else if (t < 2 * (RW - 4)) { a = 2 + t - (RW - 4); b = RY - 3; }
        else if (t < 2 * (RW - 4) + (RY - 6)) { a = 2; b = 3 + t - 2 * (RW - 4); }
        else { a = RW - 3; b = 3 + t - 2 * (RW - 4) - (RY - 6); }
        const int e = b * RX + a;
        double dx, dn;
        if (MSK[e] & kIP) zalesak(e, dx, dn);
      }
    }
    __syncthreads();

    // S5: limit, :922-946
    rect<RX, 3, RW - 2, 3, RY - 3>([&](int a, int b, int e, int) {
      if (!(MSK[e] & kIU)) return;
      const double f = FX[e];
      const double fact = lt0(f) ? kmin(RP[e - 1], RM[e]) : kmin(RP[e], RM[e - 1]);
      FX[e] = fact * f;
    });
    rect<RX, 3, RW - 3, 3, RY - 2>([&](int a, int b, int e, int) {
      if (!(MSK[e] & kIV)) return;
      const double f = FY[e];
      const double fact = lt0(f) ? kmin(RP[e - RX], RM[e]) : kmin(RP[e], RM[e - RX]);
      FY[e] = fact * f;
    });
    __syncthreads();

    // S6: corrected update of the output cells, :962-982
    rect<RX, 3, RW - 3, 3, RY - 3>([&](int a, int b, int e, int it) {
      const int i = ib0 + a, j = jb0 + b;
      if (i > ii || j > jj || !(MSK[e] & kIP)) return;
      const double fdv = ((FX[e + 1] - FX[e]) + (FY[e + RX] - FY[e])) * dt2 * SCI[e];
      const double res = kmax(qn[it], kmin(qx[it], FLO[e] - div_rcp(fdv, HN[e], RH[e])));
      const long long o = (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1;
      out[o] = res;
      if (A.images) {  // periodic in x: the xctilr copy (mod_xc_sm.h:1415-1421) written here
        if (i <= A.images) out[o + ii] = res;
        if (i > ii - A.images) out[o - ii] = res;
      }
    });
    __syncthreads();
  }
  return true;
}

template <int SCHEME, int TX, int TY>
__global__ void __launch_bounds__(256, 2) fct_tile_kernel(const TileArgs A) {
  extern __shared__ __align__(16) double sm[];
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tma::bar_init(&bar, 1);
    tma::fence_bar_init();
  }
  __syncthreads();
  uint32_t ph = 0;
  fct_tile_body<SCHEME, TX, TY>(A, blockIdx.x, blockIdx.y, sm, &bar, ph);
}

// Persistent form for an ensemble of basins: CTAs take work items
// (basin, tile, layer) from a queue until it is empty.
template <int SCHEME, int TX, int TY>
__global__ void __launch_bounds__(256, 2)
    fct_queue_kernel(const TileArgs *__restrict__ basins, const int4 *__restrict__ items, int nitems, int *head) {
  extern __shared__ __align__(16) double sm[];
  __shared__ int cur;
  __shared__ int cur_basin;
  __shared__ __align__(16) TileArgs sa;  // the item's basin, staged once (read many times below)
  __shared__ uint64_t bar;
  uint32_t ph = 0;
  if (threadIdx.x == 0) {
    cur_basin = -1;
    tma::bar_init(&bar, 1);
    tma::fence_bar_init();
  }
  for (;;) {
    if (threadIdx.x == 0) cur = atomicAdd(head, 1);
    __syncthreads();
    const int it = cur;
    if (it >= nitems) break;
    const int4 w = items[it];
    if (w.x != cur_basin) {  // uniform: every thread read the same item
      __syncthreads();
      const int *src = reinterpret_cast<const int *>(basins + w.x);
      int *dst = reinterpret_cast<int *>(&sa);
      for (int q = threadIdx.x; q < (int)(sizeof(TileArgs) / 4); q += blockDim.x) dst[q] = src[q];
      __syncthreads();
      if (threadIdx.x == 0) cur_basin = w.x;
    }
    __syncthreads();
    if (!fct_tile_body<SCHEME, TX, TY>(sa, w.y, w.z, sm, &bar, ph)) break;
  }
}

}  // namespace hyc
