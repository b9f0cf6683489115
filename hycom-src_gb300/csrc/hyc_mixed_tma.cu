// hyc_mixed_tma.cu -- FP32-mixed FCT2 ensemble kernel with TMA staging.
//
// Same arithmetic as hyc_mixed.cu (stage map to mod_tsadvc.F90:645-997,
// thickness prep :1931-1938), but every region a CTA works on is moved into
// shared memory by the Tensor Memory Accelerator (cp.async.bulk.tensor)
// and the loads run ahead of the compute:
//   * tracer regions (old and center level) are double-buffered: while the
//     stages of tracer q run, the regions of the next (layer, tracer) pair
//     are in flight;
//   * the per-layer mass fluxes are double-buffered and dp single-buffered,
//     so layer k+1's inputs arrive during layer k's tracers.
// Each load is one mbarrier transaction; the issuing thread fences the
// generic-proxy accesses of the buffer's previous use before re-filling it.
//
// TMA rules observed: the box's x start (in elements) is a multiple of 4
// (16 bytes for FP32, 32 for FP64), row strides are multiples of 16 bytes
// (the ensemble pitch is a multiple of 4 elements), shared destinations are
// 128-byte aligned, loads only (out-of-range cells read as zero).
// The halo is HYCOM's nbdy = 6: region cell (a,b) of tile (tx,ty) sits at
// array column tx*TX + a + 3 and row ty*TY + b + 3, so the box starts at
// column tx*TX (aligned) with a lead of 3 columns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "hyc_device.cuh"
#include "hyc_ens.h"

namespace hyc {

namespace {

constexpr int kLead = 3;

__device__ __forceinline__ uint32_t sa(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sa(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t gtimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait: gives up after 2 s of wall time and records the failure.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtimer_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (gtimer_ns() - t0 > 2000000000ull) break;
  }
  if (err) atomicExch(err, 1);
  return false;
}
__device__ __forceinline__ void tma3(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(sa(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(sa(bar))
      : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ float two_sum(float a, float b, float &e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}
__device__ __forceinline__ float comp_div(float a, float b, float c, float d) {
  float e1, e2;
  const float s1 = two_sum(a, -b, e1);
  const float s2 = two_sum(c, -d, e2);
  return (s1 + s2) + (e1 + e2);
}

constexpr size_t al128(size_t b) { return (b + 127) / 128 * 128; }

}  // namespace

template <int TX, int TY>
struct TmaGeom {
  static constexpr int RX = TX + 6, RY = TY + 6;
  static constexpr int P = (TX + 9 + 3) / 4 * 4;  // box width (elements), multiple of 4
  static constexpr int NP = P * RY;
  static constexpr size_t F = al128((size_t)NP * 4), D = al128((size_t)NP * 8), B = al128((size_t)NP);
  // FLD[2] FLDC[2] U[2] V[2] | W R QF DS QS FX FY FLO RP RM | DP(double) SCI(double) | MSK | mbarriers
  static constexpr size_t off_bar = 18 * F + 2 * D + B;
  static constexpr size_t smem_bytes = off_bar + 64 + 128;  // +128: alignment slack of the dynamic base
  static_assert(TX % 4 == 0, "tile width must be a multiple of 4");
};

template <int TX, int TY, int NT, bool PREP64>
__global__ void __launch_bounds__(NT, 2)
    mix_fct2_tma_kernel(const MixBasin *__restrict__ basins, const int4 *__restrict__ items, int nitems, int *head,
                        int *err) {
  using G = TmaGeom<TX, TY>;
  constexpr int RX = G::RX, RY = G::RY, P = G::P, NP = G::NP;
  constexpr int NOUT_IT = (TX * TY + NT - 1) / NT;
  extern __shared__ unsigned char smraw_[];
  unsigned char *smraw = (unsigned char *)(((uintptr_t)smraw_ + 127) & ~(uintptr_t)127);
  // double buffers: buffer s of FLD/FLDC/U/V at smraw + (base + s) * F
  auto FLDb = [&](int s) { return (float *)(smraw + (0 + s) * G::F); };
  auto FLDCb = [&](int s) { return (float *)(smraw + (2 + s) * G::F); };
  auto Ub = [&](int s) { return (float *)(smraw + (4 + s) * G::F); };
  auto Vb = [&](int s) { return (float *)(smraw + (6 + s) * G::F); };
  float *W = (float *)(smraw + 8 * G::F), *R = (float *)(smraw + 9 * G::F), *QF = (float *)(smraw + 10 * G::F),
        *DS = (float *)(smraw + 11 * G::F), *QS = (float *)(smraw + 12 * G::F), *FX = (float *)(smraw + 13 * G::F),
        *FY = (float *)(smraw + 14 * G::F), *FLO = (float *)(smraw + 15 * G::F), *RP = (float *)(smraw + 16 * G::F),
        *RM = (float *)(smraw + 17 * G::F);
  double *DP = (double *)(smraw + 18 * G::F), *SCI = (double *)(smraw + 18 * G::F + G::D);
  uint8_t *MSK = (uint8_t *)(smraw + 18 * G::F + 2 * G::D);
  uint64_t *barF = (uint64_t *)(smraw + G::off_bar);  // [2] tracer regions
  uint64_t *barL = barF + 2;                           // [2] layer inputs
  __shared__ int cur;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 4; s++) mbar_init(barF + s, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t nF = 0, nL = 0;  // completed uses of the two buffer pairs (phase tracking)
  bool ok = true;

  for (;;) {
    if (threadIdx.x == 0) cur = atomicAdd(head, 1);
    __syncthreads();
    const int item = cur;
    __syncthreads();
    if (item >= nitems || !ok) break;
    const int4 wi = items[item];
    const MixBasin &B = basins[wi.x];
    const int tile = wi.y;
    const int tyi = tile / B.ntx, txi = tile - tyi * B.ntx;
    const int X0 = txi * TX, Y0 = tyi * TY + 3;  // box origin (array column/row)
    const int ii = B.ii, jj = B.jj, ld1 = B.ld1, ld2 = B.ld2, kdm = B.kdm, ntr = B.ntr;
    const long long sl = B.slice;
    const double dt2 = B.dt2;
    const CUtensorMap *tmo = B.tm_old, *tmc = B.tm_cur, *tmu = B.tm_u, *tmv = B.tm_v, *tmd = B.tm_dp;
    const uint32_t fbytes = (uint32_t)NP * 4 * 2, lbytes = (uint32_t)NP * (4 + 4 + 8);

    // first loads of the item: layer 0 inputs, (layer 0, tracer 0) regions
    if (threadIdx.x == 0) {
      fence_async_smem();
      const int sL = nL & 1, sF = nF & 1;
      mbar_expect_tx(barL + sL, lbytes);
      tma3(Ub(sL), tmu, barL + sL, X0, Y0, 0);
      tma3(Vb(sL), tmv, barL + sL, X0, Y0, 0);
      tma3(DP, tmd, barL + sL, X0, Y0, 0);
      mbar_expect_tx(barF + sF, fbytes);
      tma3(FLDb(sF), tmo, barF + sF, X0, Y0, 0);
      tma3(FLDCb(sF), tmc, barF + sF, X0, Y0, 0);
    }
    // per item: masks and metric factors (plain loads, bounds-checked)
    for (int t = threadIdx.x; t < NP; t += NT) {
      const int b = t / P, c = t - b * P;
      const int ax = X0 + c, ay = Y0 + b;
      const bool in = ax < ld1 && ay < ld2;
      const long long o = in ? (long long)ax + (long long)ay * ld1 : 0;
      MSK[t] = in ? B.msk[o] : 0;
      const double si = in ? B.scp2i[o] : 1.0, sc = in ? B.scp2[o] : 1.0;
      SCI[t] = si;
      DS[t] = (float)(dt2 * si);
      QS[t] = (float)(sc / dt2);
    }
    __syncthreads();

    for (int k = 0; k < kdm && ok; k++) {
      const int sL = nL & 1;
      ok = __syncthreads_and(mbar_wait(barL + sL, (nL >> 1) & 1, err));  // uniform across the CTA
      nL++;
      if (!ok) break;
      float *U = Ub(sL), *V = Vb(sL);
      // thickness prep for layer k (region [0,RX-1) x [0,RY-1) is what is used)
      for (int t = threadIdx.x; t < NP; t += NT) {
        const int b = t / P, c = t - b * P;
        const bool face = c + 1 < P && b + 1 < RY;
        if (PREP64) {
          double fdv = 0.0;
          if (face) fdv = (((double)U[t + 1] - (double)U[t]) + ((double)V[t + P] - (double)V[t])) * dt2 * SCI[t];
          const double d = DP[t];
          const double fco = kmax(d + fdv, 0.0), fcn = kmax(d, 0.0);
          const double r = 1.0 / (fcn + kOnemu);
          W[t] = (float)((fco + kOnemu) * r);
          R[t] = (float)r;
          QF[t] = (float)fcn * QS[t];
        } else {
          const float onemu = (float)kOnemu;
          const float fdv = face ? comp_div(U[t + 1], U[t], V[t + P], V[t]) * DS[t] : 0.f;
          const float d = (float)DP[t];
          const float fcn = fmaxf(d, 0.f);
          const float r = __frcp_rn(fcn + onemu);
          W[t] = (d + fdv > 0.f) ? (d >= 0.f ? fmaf(fdv, r, 1.f) : (d + fdv + onemu) * r) : onemu * r;
          R[t] = r;
          QF[t] = fcn * QS[t];
        }
      }
      __syncthreads();  // DP consumed; W/R/QF ready
      if (threadIdx.x == 0 && k + 1 < kdm) {  // layer k+1 inputs into the other U/V buffer
        fence_async_smem();
        const int s2 = nL & 1;
        mbar_expect_tx(barL + s2, lbytes);
        tma3(Ub(s2), tmu, barL + s2, X0, Y0, k + 1);
        tma3(Vb(s2), tmv, barL + s2, X0, Y0, k + 1);
        tma3(DP, tmd, barL + s2, X0, Y0, k + 1);
      }

      for (int q = 0; q < ntr; q++) {
        const int sF = nF & 1;
        // prefetch the next (layer, tracer) pair of this item into the other buffer
        if (threadIdx.x == 0) {
          int nk = k, nq = q + 1;
          if (nq == ntr) {
            nq = 0;
            nk = k + 1;
          }
          if (nk < kdm) {
            fence_async_smem();
            const int s2 = (nF + 1) & 1;
            mbar_expect_tx(barF + s2, fbytes);
            tma3(FLDb(s2), tmo, barF + s2, X0, Y0, nq * kdm + nk);
            tma3(FLDCb(s2), tmc, barF + s2, X0, Y0, nq * kdm + nk);
          }
        }
        ok = __syncthreads_and(mbar_wait(barF + sF, (nF >> 1) & 1, err));
        nF++;
        if (!ok) break;
        float *FLD = FLDb(sF), *FLDC = FLDCb(sF);
        float *out = B.fnew + ((long long)q * kdm + k) * sl;
        for (int t = threadIdx.x; t < NP; t += NT) {
          FX[t] = 0.f;
          FY[t] = 0.f;
        }
        __syncthreads();
        // region cell (a, b) -> e = b*P + a + kLead
        auto rect = [&](auto A0c, auto A1c, auto B0c, auto B1c, auto &&f) {
          constexpr int A0 = decltype(A0c)::value, A1 = decltype(A1c)::value, B0 = decltype(B0c)::value,
                        B1 = decltype(B1c)::value;
          constexpr int Wd = A1 - A0, NN = Wd * (B1 - B0), IT = (NN + NT - 1) / NT;
#pragma unroll
          for (int it = 0; it < IT; it++) {
            const int t = threadIdx.x + it * NT;
            if (NN % NT == 0 || t < NN) {
              const int bb = t / Wd, aa = t - bb * Wd;
              f(A0 + aa, B0 + bb, (B0 + bb) * P + A0 + aa + kLead, it);
            }
          }
        };
        using I1 = std::integral_constant<int, 1>;
        using I2 = std::integral_constant<int, 2>;
        using I3 = std::integral_constant<int, 3>;
        using RX0 = std::integral_constant<int, RX>;
        using RX1 = std::integral_constant<int, RX - 1>;
        using RX2 = std::integral_constant<int, RX - 2>;
        using RX3 = std::integral_constant<int, RX - 3>;
        using RY0 = std::integral_constant<int, RY>;
        using RY1 = std::integral_constant<int, RY - 1>;
        using RY2 = std::integral_constant<int, RY - 2>;
        using RY3 = std::integral_constant<int, RY - 3>;
        // S1 upwind fluxes (:686-720)
        rect(I1{}, RX0{}, I1{}, RY1{}, [&](int, int, int e, int) {
          if (MSK[e] & kIU) {
            const float uu = U[e];
            FX[e] = uu * (uu >= 0.f ? FLD[e - 1] : FLD[e]);
          }
        });
        rect(I1{}, RX1{}, I1{}, RY0{}, [&](int, int, int e, int) {
          if (MSK[e] & kIV) {
            const float vv = V[e];
            FY[e] = vv * (vv >= 0.f ? FLD[e - P] : FLD[e]);
          }
        });
        __syncthreads();
        // S2 low-order solution (:778-791)
        rect(I1{}, RX1{}, I1{}, RY1{}, [&](int, int, int e, int) {
          if (!(MSK[e] & kIP)) return;
          const float c = FLD[e];
          const float w = (MSK[e - 1] & kIP) ? FLD[e - 1] : c;
          const float ea = (MSK[e + 1] & kIP) ? FLD[e + 1] : c;
          const float s = (MSK[e - P] & kIP) ? FLD[e - P] : c;
          const float n = (MSK[e + P] & kIP) ? FLD[e + P] : c;
          const float fmx = fmaxf(fmaxf(fmaxf(fmaxf(c, w), ea), s), n);
          const float fmn = fminf(fminf(fminf(fminf(c, w), ea), s), n);
          const float fdv = comp_div(FX[e + 1], FX[e], FY[e + P], FY[e]) * DS[e];
          FLO[e] = fmaxf(fmn, fminf(fmx, fmaf(c, W[e], -fdv * R[e])));
        });
        __syncthreads();
        // S3 antidiffusive fluxes (:817-833)
        rect(I2{}, RX1{}, I2{}, RY2{}, [&](int, int, int e, int) {
          if (MSK[e] & kIU) FX[e] = U[e] * 0.5f * (FLDC[e] + FLDC[e - 1]) - FX[e];
        });
        rect(I2{}, RX2{}, I2{}, RY1{}, [&](int, int, int e, int) {
          if (MSK[e] & kIV) FY[e] = V[e] * 0.5f * (FLDC[e] + FLDC[e - P]) - FY[e];
        });
        __syncthreads();
        // fmxlo/fmnlo (:792-793) in place
        rect(I1{}, RX1{}, I1{}, RY1{}, [&](int, int, int e, int) {
          if (!(MSK[e] & kIP)) return;
          const float c = FLD[e], cc = FLDC[e], lo = FLO[e];
          FLD[e] = fmaxf(fmaxf(c, cc), lo);
          FLDC[e] = fminf(fminf(c, cc), lo);
        });
        __syncthreads();
        // S4 Zalesak (:863-909)
        float qx[NOUT_IT], qn[NOUT_IT];
        auto zalesak = [&](int e, float &fqmax, float &fqmin) {
          const bool mw = MSK[e - 1] & kIP, me = MSK[e + 1] & kIP, ms = MSK[e - P] & kIP, mn = MSK[e + P] & kIP;
          fqmax = FLD[e];
          fqmin = FLDC[e];
          fqmax = fmaxf(fqmax, mw ? FLD[e - 1] : FLD[e]);
          fqmax = fmaxf(fqmax, me ? FLD[e + 1] : FLD[e]);
          fqmax = fmaxf(fqmax, ms ? FLD[e - P] : FLD[e]);
          fqmax = fmaxf(fqmax, mn ? FLD[e + P] : FLD[e]);
          fqmin = fminf(fqmin, mw ? FLDC[e - 1] : FLDC[e]);
          fqmin = fminf(fqmin, me ? FLDC[e + 1] : FLDC[e]);
          fqmin = fminf(fqmin, ms ? FLDC[e - P] : FLDC[e]);
          fqmin = fminf(fqmin, mn ? FLDC[e + P] : FLDC[e]);
          const float fxa = FX[e], fxb = me ? FX[e + 1] : FX[e];  // ipip1 quirk (:873-883)
          const float fya = FY[e], fyb = mn ? FY[e + P] : FY[e];
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
        rect(I3{}, RX3{}, I3{}, RY3{}, [&](int, int, int e, int it) {
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
            const int e = b * P + a + kLead;
            float dx, dn;
            if (MSK[e] & kIP) zalesak(e, dx, dn);
          }
        }
        __syncthreads();
        // S5 limit (:922-946)
        rect(I3{}, RX2{}, I3{}, RY3{}, [&](int, int, int e, int) {
          if (!(MSK[e] & kIU)) return;
          const float f = FX[e];
          FX[e] = (f < 0.f ? fminf(RP[e - 1], RM[e]) : fminf(RP[e], RM[e - 1])) * f;
        });
        rect(I3{}, RX3{}, I3{}, RY2{}, [&](int, int, int e, int) {
          if (!(MSK[e] & kIV)) return;
          const float f = FY[e];
          FY[e] = (f < 0.f ? fminf(RP[e - P], RM[e]) : fminf(RP[e], RM[e - P])) * f;
        });
        __syncthreads();
        // S6 update (:962-982) -> new level, plus periodic halo images
        rect(I3{}, RX3{}, I3{}, RY3{}, [&](int a, int b, int e, int it) {
          const int i = X0 + a + kLead - 5, j = Y0 + b - 5;  // Fortran indices (nbdy = 6)
          if (i > ii || j > jj || !(MSK[e] & kIP)) return;
          const float fdv = comp_div(FX[e + 1], FX[e], FY[e + P], FY[e]) * DS[e];
          const float res = fmaxf(qn[it], fminf(qx[it], FLO[e] - fdv * R[e]));
          const long long o = (long long)(X0 + a + kLead) + (long long)(Y0 + b) * ld1;
          out[o] = res;
          if (B.images) {
            if (i <= B.images) out[o + ii] = res;
            if (i > ii - B.images) out[o - ii] = res;
          }
        });
        __syncthreads();
      }
    }
  }
}

template <int TX, int TY>
static cudaError_t launch_tma(const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm, bool prep64,
                              int *err, cudaStream_t s) {
  constexpr size_t smem = TmaGeom<TX, TY>::smem_bytes;
  static_assert(smem <= 227 * 1024, "tile does not fit");
  auto kern = prep64 ? mix_fct2_tma_kernel<TX, TY, 256, true> : mix_fct2_tma_kernel<TX, TY, 256, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  kern<<<nsm * per_sm, 256, smem, s>>>(basins, items, nitems, head, err);
  return cudaGetLastError();
}

bool mix_tma_shape_ok(TileShape t) {
  return (t.tx == 32 && t.ty == 16) || (t.tx == 64 && t.ty == 8) || (t.tx == 32 && t.ty == 8) ||
         (t.tx == 64 && t.ty == 16);
}

cudaError_t launch_mix_fct2_tma(TileShape t, const MixBasin *basins, const int4 *items, int nitems, int *head,
                                int nsm, bool prep64, int *err, cudaStream_t s) {
  if (t.tx == 32 && t.ty == 16) return launch_tma<32, 16>(basins, items, nitems, head, nsm, prep64, err, s);
  if (t.tx == 64 && t.ty == 8) return launch_tma<64, 8>(basins, items, nitems, head, nsm, prep64, err, s);
  if (t.tx == 32 && t.ty == 8) return launch_tma<32, 8>(basins, items, nitems, head, nsm, prep64, err, s);
  if (t.tx == 64 && t.ty == 16) return launch_tma<64, 16>(basins, items, nitems, head, nsm, prep64, err, s);
  return cudaErrorInvalidValue;
}

}  // namespace hyc
