// hyc_mixed.cu -- FP32-mixed FCT2 for an ensemble of basins (persistent
// tile queue).
//
// Precision split (per update the FP32 pipe does the work; the FP64 pipe on
// GB300 issues at ~1/72 of the FP32 rate, so FP64 is kept to work per cell
// and layer, shared by all tracers of the layer):
//   FP64  thickness prep per cell and layer: the flux divergence of the
//         continuity step (from the FP32 mass fluxes, converted exactly),
//         fco = max(dp + div*delt1*scp2i, 0), fcn = max(dp, 0), and the
//         thickness-weighted division factors w = (fco+onemu)/(fcn+onemu)
//         and r = 1/(fcn+onemu) (mod_tsadvc.F90:1931-1938, :788-791);
//   FP32  fluxes, extrema, Zalesak limiter and the update of every tracer
//         (mod_tsadvc.F90:686-982), with the flux divergence summed with
//         two-sum error terms (compensated) before it is scaled.
// Tracer state, fluxes and the metric factors are FP32; dp is FP64.
//
// Work item = (basin, tile): the CTA walks all layers of the tile and all
// tracers of each layer, so masks and metrics are staged once per item and
// the per-layer factors once per layer.  The new time level is written to
// the third leapfrog buffer (no in-place update, no copy-back), with the
// periodic-x halo images written by the same store (xctilr fused in).
#include <cuda_runtime.h>

#include <cstdint>

#include "hyc_device.cuh"
#include "hyc_ens.h"

namespace hyc {

template <int TX, int TY>
struct MixGeom {
  static constexpr int RX = TX + 6, RY = TY + 6, N = RX * RY;
  // doubles: SCI | floats: DS QS U V W R QF FLD FLDC FX FY FLO RP RM | bytes: MSK
  static constexpr size_t smem_bytes = (size_t)N * 8 + (size_t)14 * N * 4 + ((N + 15) / 16) * 16;
  static_assert(N % 2 == 0, "FX/FY double as the 8-byte-aligned dp staging buffer");
};

template <int RX, int A0, int A1, int B0, int B1, int NT, class F>
__device__ __forceinline__ void rectf(F &&f) {
  constexpr int W = A1 - A0;
  constexpr int NN = W * (B1 - B0);
  constexpr int IT = (NN + NT - 1) / NT;
#pragma unroll
  for (int it = 0; it < IT; it++) {
    const int t = threadIdx.x + it * NT;
    if (NN % NT == 0 || t < NN) {
      const int bb = t / W;
      const int aa = t - bb * W;
      f(A0 + aa, B0 + bb, (B0 + bb) * RX + A0 + aa, it);
    }
  }
}

// a + b exactly as s + e (Knuth two-sum)
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}

// ((a - b) + (c - d)) with the rounding errors of the two differences added
// back (two-sum): the compensated flux divergence of four face fluxes.
__device__ __forceinline__ float comp_div(float a, float b, float c, float d) {
  float e1, e2;
  const float s1 = two_sum(a, -b, e1);
  const float s2 = two_sum(c, -d, e2);
  return (s1 + s2) + (e1 + e2);
}

template <int TX, int TY, int NT, bool PREP64>
__device__ __forceinline__ void mix_fct2_item(const MixBasin &B, const int tile, unsigned char *smraw) {
  using G = MixGeom<TX, TY>;
  constexpr int RX = G::RX, RY = G::RY, N = G::N;
  constexpr int NOUT_IT = (TX * TY + NT - 1) / NT;
  double *SCI = reinterpret_cast<double *>(smraw);
  float *DS = reinterpret_cast<float *>(SCI + N), *QS = DS + N, *U = QS + N, *V = U + N, *W = V + N, *R = W + N,
        *QF = R + N, *FLD = QF + N, *FLDC = FLD + N, *FX = FLDC + N, *FY = FX + N, *FLO = FY + N, *RP = FLO + N,
        *RM = RP + N;
  uint8_t *MSK = reinterpret_cast<uint8_t *>(RM + N);
  double *DPD = reinterpret_cast<double *>(FX);  // dp staging: FX and FY are free between layers

  const int tyi = tile / B.ntx, txi = tile - tyi * B.ntx;
  const int ib0 = 1 + txi * TX - 3, jb0 = 1 + tyi * TY - 3;
  const int nb = B.nbdy, ld1 = B.ld1, ii = B.ii, jj = B.jj;
  const long long sl = B.slice;
  const double dt2 = B.dt2;
  const float dt2f = (float)dt2;

  // ---- per item: masks and metric factors ---------------------------------
  for (int t = threadIdx.x; t < N; t += NT) {
    const int bb = t / RX, aa = t - bb * RX;
    const int i = ib0 + aa, j = jb0 + bb;
    const bool in = (i >= 1 - nb) && (i <= ii + nb) && (j >= 1 - nb) && (j <= jj + nb);
    const long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
    MSK[t] = in ? B.msk[o] : 0;
    const double si = in ? B.scp2i[o] : 1.0, sc = in ? B.scp2[o] : 1.0;
    SCI[t] = si;
    DS[t] = (float)(dt2 * si);  // flux -> tracer-content change per unit area over delt1
    QS[t] = (float)(sc / dt2);
  }
  for (int k = 0; k < B.kdm; k++) {
    __syncthreads();  // previous layer done with U/V/W/R/QF/FX/FY
    const float *uk = B.uflx + k * sl, *vk = B.vflx + k * sl;
    const double *dk = B.dp + k * sl;
    for (int t = threadIdx.x; t < N; t += NT) {
      const int bb = t / RX, aa = t - bb * RX;
      const int i = ib0 + aa, j = jb0 + bb;
      const bool in = (i >= 1 - nb) && (i <= ii + nb) && (j >= 1 - nb) && (j <= jj + nb);
      const long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
      U[t] = in ? uk[o] : 0.f;
      V[t] = in ? vk[o] : 0.f;
      DPD[t] = in ? dk[o] : 0.0;
    }
    __syncthreads();
    // thickness prep (mod_tsadvc.F90:1931-1938) -> FP32 factors
    //   W = (fco+onemu)/(fcn+onemu), R = 1/(fcn+onemu), QF = fcn*scal/delt1
    for (int t = threadIdx.x; t < N; t += NT) {
      const int bb = t / RX, aa = t - bb * RX;
      const bool face = aa < RX - 1 && bb < RY - 1;
      if (PREP64) {  // in FP64, as the reference
        double fdv = 0.0;
        if (face) fdv = (((double)U[t + 1] - (double)U[t]) + ((double)V[t + RX] - (double)V[t])) * dt2 * SCI[t];
        const double d = DPD[t];
        const double fco = kmax(d + fdv, 0.0), fcn = kmax(d, 0.0);
        const double r = 1.0 / (fcn + kOnemu);
        W[t] = (float)((fco + kOnemu) * r);
        R[t] = (float)r;
        QF[t] = (float)fcn * QS[t];
      } else {  // in FP32 on the FP32 pipe: compensated divergence, W = 1 + div*R
        const float onemu = (float)kOnemu;
        const float fdv = face ? comp_div(U[t + 1], U[t], V[t + RX], V[t]) * DS[t] : 0.f;
        const float d = (float)DPD[t];
        const float fcn = fmaxf(d, 0.f);
        const float r = __frcp_rn(fcn + onemu);
        W[t] = (d + fdv > 0.f) ? (d >= 0.f ? fmaf(fdv, r, 1.f) : (d + fdv + onemu) * r) : onemu * r;
        R[t] = r;
        QF[t] = fcn * QS[t];
      }
    }
    __syncthreads();

    for (int q = 0; q < B.ntr; q++) {
      const long long so = ((long long)q * B.kdm + k) * sl;
      const float *fo = B.fold + so, *fc = B.fcur + so;
      float *out = B.fnew + so;
      for (int t = threadIdx.x; t < N; t += NT) {
        const int bb = t / RX, aa = t - bb * RX;
        const int i = ib0 + aa, j = jb0 + bb;
        const bool in = (i >= 1 - nb) && (i <= ii + nb) && (j >= 1 - nb) && (j <= jj + nb);
        const long long o = in ? (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1 : 0;
        FLD[t] = in ? fo[o] : 0.f;
        FLDC[t] = in ? fc[o] : 0.f;
        FX[t] = 0.f;
        FY[t] = 0.f;
      }
      __syncthreads();
      // S1 upwind fluxes (:686-720)
      rectf<RX, 1, RX, 1, RY - 1, NT>([&](int, int, int e, int) {
        if (MSK[e] & kIU) {
          const float uu = U[e];
          FX[e] = uu * (uu >= 0.f ? FLD[e - 1] : FLD[e]);
        }
      });
      rectf<RX, 1, RX - 1, 1, RY, NT>([&](int, int, int e, int) {
        if (MSK[e] & kIV) {
          const float vv = V[e];
          FY[e] = vv * (vv >= 0.f ? FLD[e - RX] : FLD[e]);
        }
      });
      __syncthreads();
      // S2 low-order solution (:778-791): (fld*ho - div)/hn = fld*w - div*r
      rectf<RX, 1, RX - 1, 1, RY - 1, NT>([&](int, int, int e, int) {
        if (!(MSK[e] & kIP)) return;
        const float c = FLD[e];
        const float w = (MSK[e - 1] & kIP) ? FLD[e - 1] : c;
        const float ea = (MSK[e + 1] & kIP) ? FLD[e + 1] : c;
        const float s = (MSK[e - RX] & kIP) ? FLD[e - RX] : c;
        const float n = (MSK[e + RX] & kIP) ? FLD[e + RX] : c;
        const float fmx = fmaxf(fmaxf(fmaxf(fmaxf(c, w), ea), s), n);
        const float fmn = fminf(fminf(fminf(fminf(c, w), ea), s), n);
        const float fdv = comp_div(FX[e + 1], FX[e], FY[e + RX], FY[e]) * DS[e];
        FLO[e] = fmaxf(fmn, fminf(fmx, fmaf(c, W[e], -fdv * R[e])));
      });
      __syncthreads();
      // S3 antidiffusive fluxes (:817-833)
      rectf<RX, 2, RX - 1, 2, RY - 2, NT>([&](int, int, int e, int) {
        if (MSK[e] & kIU) FX[e] = U[e] * 0.5f * (FLDC[e] + FLDC[e - 1]) - FX[e];
      });
      rectf<RX, 2, RX - 2, 2, RY - 1, NT>([&](int, int, int e, int) {
        if (MSK[e] & kIV) FY[e] = V[e] * 0.5f * (FLDC[e] + FLDC[e - RX]) - FY[e];
      });
      __syncthreads();
      // fmxlo/fmnlo (:792-793) over fld/fldc in place
      rectf<RX, 1, RX - 1, 1, RY - 1, NT>([&](int, int, int e, int) {
        if (!(MSK[e] & kIP)) return;
        const float c = FLD[e], cc = FLDC[e], lo = FLO[e];
        FLD[e] = fmaxf(fmaxf(c, cc), lo);
        FLDC[e] = fminf(fminf(c, cc), lo);
      });
      __syncthreads();
      // S4 Zalesak (:863-909)
      float qx[NOUT_IT], qn[NOUT_IT];
      auto zalesak = [&](int e, float &fqmax, float &fqmin) {
        const bool mw = MSK[e - 1] & kIP, me = MSK[e + 1] & kIP, ms = MSK[e - RX] & kIP, mn = MSK[e + RX] & kIP;
        fqmax = FLD[e];
        fqmin = FLDC[e];
        fqmax = fmaxf(fqmax, mw ? FLD[e - 1] : FLD[e]);
        fqmax = fmaxf(fqmax, me ? FLD[e + 1] : FLD[e]);
        fqmax = fmaxf(fqmax, ms ? FLD[e - RX] : FLD[e]);
        fqmax = fmaxf(fqmax, mn ? FLD[e + RX] : FLD[e]);
        fqmin = fminf(fqmin, mw ? FLDC[e - 1] : FLDC[e]);
        fqmin = fminf(fqmin, me ? FLDC[e + 1] : FLDC[e]);
        fqmin = fminf(fqmin, ms ? FLDC[e - RX] : FLDC[e]);
        fqmin = fminf(fqmin, mn ? FLDC[e + RX] : FLDC[e]);
        const float fxa = FX[e], fxb = me ? FX[e + 1] : FX[e];  // ipip1 quirk (:873-883)
        const float fya = FY[e], fyb = mn ? FY[e + RX] : FY[e];
        const float famax = fmaxf(0.f, fxa) - fminf(0.f, fxb) + fmaxf(0.f, fya) - fminf(0.f, fyb);
        const float famin = fmaxf(0.f, fxb) - fminf(0.f, fxa) + fmaxf(0.f, fyb) - fminf(0.f, fya);
        const float lo = FLO[e];
        float rp = 0.f, rm = 0.f;
        if (famax > 0.f) {
          const float qp = (fqmax - lo) * QF[e];
          rp = qp < famax ? __fdiv_rn(qp, famax) : 1.f;
        }
        if (famin > 0.f) {
          const float qm = (lo - fqmin) * QF[e];
          rm = qm < famin ? __fdiv_rn(qm, famin) : 1.f;
        }
        RP[e] = rp;
        RM[e] = rm;
      };
      rectf<RX, 3, RX - 3, 3, RY - 3, NT>([&](int, int, int e, int it) {
        if (MSK[e] & kIP) zalesak(e, qx[it], qn[it]);
      });
      {
        constexpr int NR = 2 * (RX - 4) + 2 * (RY - 6);
        for (int t = threadIdx.x; t < NR; t += NT) {
          int a, b;
          if (t < RX - 4) { a = 2 + t; b = 2; }
          else if (t < 2 * (RX - 4)) { a = 2 + t - (RX - 4); b = RY - 3; }
          else if (t < 2 * (RX - 4) + (RY - 6)) { a = 2; b = 3 + t - 2 * (RX - 4); }
          else { a = RX - 3; b = 3 + t - 2 * (RX - 4) - (RY - 6); }
          const int e = b * RX + a;
          float dx, dn;
          if (MSK[e] & kIP) zalesak(e, dx, dn);
        }
      }
      __syncthreads();
      // S5 limit (:922-946)
      rectf<RX, 3, RX - 2, 3, RY - 3, NT>([&](int, int, int e, int) {
        if (!(MSK[e] & kIU)) return;
        const float f = FX[e];
        FX[e] = (f < 0.f ? fminf(RP[e - 1], RM[e]) : fminf(RP[e], RM[e - 1])) * f;
      });
      rectf<RX, 3, RX - 3, 3, RY - 2, NT>([&](int, int, int e, int) {
        if (!(MSK[e] & kIV)) return;
        const float f = FY[e];
        FY[e] = (f < 0.f ? fminf(RP[e - RX], RM[e]) : fminf(RP[e], RM[e - RX])) * f;
      });
      __syncthreads();
      // S6 update (:962-982), new level + periodic halo images
      rectf<RX, 3, RX - 3, 3, RY - 3, NT>([&](int a, int b, int e, int it) {
        const int i = ib0 + a, j = jb0 + b;
        if (i > ii || j > jj || !(MSK[e] & kIP)) return;
        const float fdv = comp_div(FX[e + 1], FX[e], FY[e + RX], FY[e]) * DS[e];
        const float res = fmaxf(qn[it], fminf(qx[it], FLO[e] - fdv * R[e]));
        const long long o = (long long)(i + nb - 1) + (long long)(j + nb - 1) * ld1;
        out[o] = res;
        if (B.images) {
          if (i <= B.images) out[o + ii] = res;
          if (i > ii - B.images) out[o - ii] = res;
        }
      });
      __syncthreads();
    }
  }
  (void)dt2f;
}

template <int TX, int TY, int NT, bool PREP64>
__global__ void __launch_bounds__(NT, 2) mix_fct2_queue_kernel(const MixBasin *__restrict__ basins,
                                                           const int4 *__restrict__ items, int nitems, int *head) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int cur;
  for (;;) {
    if (threadIdx.x == 0) cur = atomicAdd(head, 1);
    __syncthreads();
    const int it = cur;
    __syncthreads();
    if (it >= nitems) break;
    const int4 w = items[it];
    mix_fct2_item<TX, TY, NT, PREP64>(basins[w.x], w.y, smraw);
    __syncthreads();
  }
}

template <int TX, int TY, int NT>
static cudaError_t launch_mix(const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm,
                              bool prep64, cudaStream_t s) {
  constexpr size_t smem = MixGeom<TX, TY>::smem_bytes;
  static_assert(smem <= 227 * 1024, "tile does not fit");
  auto kern = prep64 ? mix_fct2_queue_kernel<TX, TY, NT, true> : mix_fct2_queue_kernel<TX, TY, NT, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  kern<<<nsm * per_sm, NT, smem, s>>>(basins, items, nitems, head);
  return cudaGetLastError();
}

bool mix_shape_ok(TileShape t) {
  return (t.tx == 32 && t.ty == 16) || (t.tx == 64 && t.ty == 16) || (t.tx == 32 && t.ty == 32) ||
         (t.tx == 64 && t.ty == 8) || (t.tx == 128 && t.ty == 8);
}

cudaError_t launch_mix_fct2(TileShape t, const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm,
                            bool prep64, cudaStream_t s) {
  if (t.tx == 32 && t.ty == 16) return launch_mix<32, 16, 256>(basins, items, nitems, head, nsm, prep64, s);
  if (t.tx == 64 && t.ty == 16) return launch_mix<64, 16, 256>(basins, items, nitems, head, nsm, prep64, s);
  if (t.tx == 32 && t.ty == 32) return launch_mix<32, 32, 256>(basins, items, nitems, head, nsm, prep64, s);
  if (t.tx == 64 && t.ty == 8) return launch_mix<64, 8, 256>(basins, items, nitems, head, nsm, prep64, s);
  if (t.tx == 128 && t.ty == 8) return launch_mix<128, 8, 256>(basins, items, nitems, head, nsm, prep64, s);
  return cudaErrorInvalidValue;
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
