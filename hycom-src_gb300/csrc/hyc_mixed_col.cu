// hyc_mixed_col.cu -- FP32-mixed FCT2 ensemble kernel, one warp per column
// strip marching north through the rows.
//
// The shared-memory tile kernels spend most of their instructions on index
// arithmetic, shared-memory round trips between stages and the recomputed
// tile halo.  Here each lane owns one column i and carries every stage of
// mod_tsadvc.F90:645-997 in registers as a row pipeline: at step J the lane
// loads row J, computes the fluxes of row J, the low-order solution and
// antidiffusive fluxes of row J-1, the Zalesak ratios of row J-2 and the
// limited update of row J-3.  East/west neighbours come from warp shuffles,
// north/south neighbours are the registers of the previous rows.  A warp
// covers 32 columns and updates the 26 in the middle (the scheme reaches 3
// cells); a work item is (basin, strip, segment of rows) with all layers and
// tracers, taken from a queue by whole warps (no CTA-wide barriers).
//
// Arithmetic per cell is that of hyc_mixed.cu: FP32 fluxes, extrema,
// limiter and update, two-sum compensated flux divergence; the thickness
// factors W = (fco+onemu)/(fcn+onemu), R = 1/(fcn+onemu), QF = fcn*scal/dt2
// from the continuity divergence per cell and layer, in FP64 (PREP64) or in
// compensated FP32.
#include <cuda_runtime.h>

#include <cstdint>

#include "hyc_device.cuh"
#include "hyc_ens.h"

namespace hyc {

namespace {

__device__ __forceinline__ float two_sum(float a, float b, float &e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}
// ((a - b) + (c - d)) with the rounding errors of the two differences added
// back (two-sum): the cancellation between the large, nearly equal fluxes
// through opposite faces is exact; the last addition rounds relative to the
// divergence itself.
__device__ __forceinline__ float comp_div(float a, float b, float c, float d) {
  float e1, e2;
  const float s1 = two_sum(a, -b, e1);
  const float s2 = two_sum(c, -d, e2);
  return (s1 + s2) + (e1 + e2);
}
__device__ __forceinline__ float up(float x) { return __shfl_up_sync(0xffffffffu, x, 1); }
__device__ __forceinline__ float dn(float x) { return __shfl_down_sync(0xffffffffu, x, 1); }
__device__ __forceinline__ unsigned upu(unsigned x) { return __shfl_up_sync(0xffffffffu, x, 1); }
__device__ __forceinline__ unsigned dnu(unsigned x) { return __shfl_down_sync(0xffffffffu, x, 1); }

// pipeline registers of one tracer (row offsets relative to the step's row J)
struct TrState {
  float f1, f2, f1w, f1e;   // fld at J-1, J-2; fld(J-1) of the west/east lanes
  float c1, c1w;            // fldc at J-1 and its west lane
  float fx1, fx1e, fy1;     // low-order x-flux (west face) and y-flux (south face) of row J-1
  float lo2, lo3;           // fldlo at J-2, J-3
  float mx2, mn2, mx2w, mx2e, mn2w, mn2e, mx3, mn3;  // fmxlo/fmnlo at J-2 (+ neighbours), J-3
  float ax2, ax2e;          // antidiffusive x-flux (west face) of row J-2 and its east lane
  float ay1, ay2;           // antidiffusive y-flux (south face) of rows J-1, J-2
  float rp3, rm3;           // ratios at J-3
  float lx3, lx3e, ly3;     // limited fluxes of row J-3 (x: west face, + east lane; y: south face)
  float qx3, qn3;           // fqmax/fqmin at J-3
};

}  // namespace

template <int NQ, bool PREP64>
__global__ void __launch_bounds__(128)
    mix_fct2_col_kernel(const MixBasin *__restrict__ basins, const int4 *__restrict__ items, int nitems, int *head,
                        int rows_max) {
  const int lane = threadIdx.x & 31;
  // per warp: the masks and metric factors of its item's rows, read once per
  // item instead of once per layer
  extern __shared__ __align__(16) unsigned char csm[];
  const int wid = threadIdx.x >> 5;
  float2 *sdq = reinterpret_cast<float2 *>(csm) + (size_t)wid * rows_max * 32;
  uint8_t *smk = csm + (size_t)(blockDim.x >> 5) * rows_max * 32 * sizeof(float2) + (size_t)wid * rows_max * 32;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(head, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const int4 w = items[it];
    const MixBasin &B = basins[w.x];
    const int ii = B.ii, jj = B.jj, nb = B.nbdy, ld1 = B.ld1, kdm = B.kdm;
    const long long sl = B.slice;
    const int i = 1 + 26 * w.y - 3 + lane;  // this lane's column (Fortran index)
    const int j0 = 1 + w.z * B.seg, j1 = min(j0 + B.seg, jj + 1);
    const bool colin = i >= 1 - nb && i <= ii + nb;
    const bool colout = lane >= 3 && lane < 29 && i <= ii;
    const double dt2 = B.dt2;
    const float onemu = (float)kOnemu;
    const long long cbase = colin ? (long long)(i + nb - 1) : 0;
    const int jr0 = j0 - 3, nrows = j1 + 2 - jr0 + 1;  // rows j0-3 .. j1+2
    __syncwarp();
    for (int r = 0; r < nrows; r++) {
      const int J = jr0 + r;
      const bool in = colin && J >= 1 - nb && J <= jj + nb;
      const long long o = cbase + (long long)(J + nb - 1) * ld1;
      smk[r * 32 + lane] = in ? B.msk[o] : 0;
      sdq[r * 32 + lane] = in ? B.dsqs[o] : make_float2(0.f, 0.f);
    }
    __syncwarp();

    for (int q0 = 0; q0 < B.ntr; q0 += NQ) {
      const int nq = min(NQ, B.ntr - q0);
      for (int k = 0; k < kdm; k++) {
        const float *uk = B.uflx + k * sl, *vk = B.vflx + k * sl;
        const double *dk = B.dp + k * sl;
        const float *fo[NQ], *fc[NQ];
        float *fn[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++) {
          const long long so = ((long long)(q0 + (q < nq ? q : 0)) * kdm + k) * sl;
          fo[q] = B.fold + so;
          fc[q] = B.fcur + so;
          fn[q] = B.fnew + so;
        }
        TrState S[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++) S[q] = TrState{};
        unsigned m1 = 0, m2 = 0, m3 = 0, mw1 = 0, me1 = 0, mw2 = 0, me2 = 0;
        float u1 = 0.f, v1 = 0.f, W1 = 1.f, R1 = 0.f, R2 = 0.f, R3 = 0.f, QF1 = 0.f, QF2 = 0.f;
        float DS1 = 0.f, DS2 = 0.f, DS3 = 0.f, QS1 = 0.f;
        double d1 = 0.0;
        double sci1 = 0.0;
        // row J inputs (loaded one row ahead)
        auto load_row = [&](int J, unsigned &m, float (&f)[NQ], float (&c)[NQ], float &u, float &v, double &d,
                            float2 &dq, double &sci) {
          const bool in = colin && J >= 1 - nb && J <= jj + nb;
          const long long o = cbase + (long long)(J + nb - 1) * ld1;
          m = smk[(J - jr0) * 32 + lane];
          u = in ? uk[o] : 0.f;
          v = in ? vk[o] : 0.f;
          d = in ? dk[o] : 0.0;
          dq = sdq[(J - jr0) * 32 + lane];
          sci = (PREP64 && in) ? B.scp2i[o] : 0.0;
#pragma unroll
          for (int q = 0; q < NQ; q++) {
            f[q] = (in && q < nq) ? fo[q][o] : 0.f;
            c[q] = (in && q < nq) ? fc[q][o] : 0.f;
          }
        };
        unsigned mN;
        float fN[NQ], cN[NQ], uN, vN;
        double dN, sciN;
        float2 dqN;
        load_row(j0 - 3, mN, fN, cN, uN, vN, dN, dqN, sciN);
#pragma unroll 2
        for (int J = j0 - 3; J <= j1 + 2; J++) {
          const unsigned m0 = mN;
          float f0[NQ], c0[NQ];
#pragma unroll
          for (int q = 0; q < NQ; q++) {
            f0[q] = fN[q];
            c0[q] = cN[q];
          }
          const float u0 = uN, v0 = vN;
          const double d0 = dN, sci0 = sciN;
          const float2 dq0 = dqN;
          if (J < j1 + 2) load_row(J + 1, mN, fN, cN, uN, vN, dN, dqN, sciN);  // prefetch

          // thickness factors of row J-1 (mod_tsadvc.F90:1931-1938)
          const float u1e = dn(u1);
          if (PREP64) {
            const double fdv = (((double)u1e - (double)u1) + ((double)v0 - (double)v1)) * dt2 * sci1;
            const double fco = kmax(d1 + fdv, 0.0), fcn = kmax(d1, 0.0);
            const double r = 1.0 / (fcn + kOnemu);
            W1 = (float)((fco + kOnemu) * r);
            R1 = (float)r;
            QF1 = (float)fcn * QS1;
          } else {
            const float fdv = comp_div(u1e, u1, v0, v1) * DS1;
            const float d = (float)d1;
            const float fcn = fmaxf(d, 0.f);
            const float r = __frcp_rn(fcn + onemu);
            W1 = (d + fdv > 0.f) ? (d >= 0.f ? fmaf(fdv, r, 1.f) : (d + fdv + onemu) * r) : onemu * r;
            R1 = r;
            QF1 = fcn * QS1;
          }
          const unsigned mw0 = upu(m0), me0 = dnu(m0);

#pragma unroll
          for (int q = 0; q < NQ; q++) {
            TrState &s = S[q];
            const float f0w = up(f0[q]), f0e = dn(f0[q]);
            // S1: low-order fluxes of row J (:686-720)
            const float fx0 = (m0 & kIU) ? u0 * (u0 >= 0.f ? f0w : f0[q]) : 0.f;
            const float fy0 = (m0 & kIV) ? v0 * (v0 >= 0.f ? s.f1 : f0[q]) : 0.f;
            // S2: low-order solution of row J-1 (:778-791)
            const float c = s.f1;
            const float fw = (mw1 & kIP) ? s.f1w : c, fe = (me1 & kIP) ? s.f1e : c;
            const float fs = (m2 & kIP) ? s.f2 : c, fnn = (m0 & kIP) ? f0[q] : c;
            const float fmx = fmaxf(fmaxf(fmaxf(fmaxf(c, fw), fe), fs), fnn);
            const float fmn = fminf(fminf(fminf(fminf(c, fw), fe), fs), fnn);
            const float fdv = comp_div(s.fx1e, s.fx1, fy0, s.fy1) * DS1;
            const float lo1 = fmaxf(fmn, fminf(fmx, fmaf(c, W1, -fdv * R1)));
            // S3: antidiffusive fluxes, x of row J-1 and y of row J (:817-833)
            const float ax1 = (m1 & kIU) ? u1 * 0.5f * (s.c1 + s.c1w) - s.fx1 : 0.f;
            const float ay0 = (m0 & kIV) ? v0 * 0.5f * (c0[q] + s.c1) - fy0 : 0.f;
            const float mx1 = fmaxf(fmaxf(c, s.c1), lo1), mn1 = fminf(fminf(c, s.c1), lo1);  // :792-793
            // S4: Zalesak ratios of row J-2 (:863-909)
            const float x2 = s.mx2, n2 = s.mn2;
            float fqmax = x2, fqmin = n2;
            fqmax = fmaxf(fqmax, (mw2 & kIP) ? s.mx2w : x2);
            fqmax = fmaxf(fqmax, (me2 & kIP) ? s.mx2e : x2);
            fqmax = fmaxf(fqmax, (m3 & kIP) ? s.mx3 : x2);
            fqmax = fmaxf(fqmax, (m1 & kIP) ? mx1 : x2);
            fqmin = fminf(fqmin, (mw2 & kIP) ? s.mn2w : n2);
            fqmin = fminf(fqmin, (me2 & kIP) ? s.mn2e : n2);
            fqmin = fminf(fqmin, (m3 & kIP) ? s.mn3 : n2);
            fqmin = fminf(fqmin, (m1 & kIP) ? mn1 : n2);
            const float fxa = s.ax2, fxb = (me2 & kIP) ? s.ax2e : s.ax2;  // ipip1 quirk (:873-883)
            const float fya = s.ay2, fyb = (m1 & kIP) ? s.ay1 : s.ay2;
            const float famax = fmaxf(0.f, fxa) - fminf(0.f, fxb) + fmaxf(0.f, fya) - fminf(0.f, fyb);
            const float famin = fmaxf(0.f, fxb) - fminf(0.f, fxa) + fmaxf(0.f, fyb) - fminf(0.f, fya);
            float rp2 = 0.f, rm2 = 0.f;
            if (famax > 0.f) {
              const float qp = (fqmax - s.lo2) * QF2;
              rp2 = qp < famax ? __fdiv_rn(qp, famax) : 1.f;
            }
            if (famin > 0.f) {
              const float qm = (s.lo2 - fqmin) * QF2;
              rm2 = qm < famin ? __fdiv_rn(qm, famin) : 1.f;
            }
            // S5: limited fluxes of row J-2 (:922-946)
            const float rp2w = up(rp2), rm2w = up(rm2);
            const float lx2 = (m2 & kIU) ? (s.ax2 < 0.f ? fminf(rp2w, rm2) : fminf(rp2, rm2w)) * s.ax2 : 0.f;
            const float ly2 = (m2 & kIV) ? (s.ay2 < 0.f ? fminf(s.rp3, rm2) : fminf(rp2, s.rm3)) * s.ay2 : 0.f;
            // S6: update of row J-3 (:962-982)
            const int jo = J - 3;
            if (colout && jo >= j0 && jo < j1 && (m3 & kIP) && q < nq) {
              const float fd3 = comp_div(s.lx3e, s.lx3, ly2, s.ly3) * DS3;
              const float res = fmaxf(s.qn3, fminf(s.qx3, s.lo3 - fd3 * R3));
              const long long o = cbase + (long long)(jo + nb - 1) * ld1;
              fn[q][o] = res;
              if (B.images) {
                if (i <= B.images) fn[q][o + ii] = res;
                if (i > ii - B.images) fn[q][o - ii] = res;
              }
            }
            // shift the pipeline one row
            const float lx2e = dn(lx2), ax1e = dn(ax1), fx0e = dn(fx0);
            const float mx1w = up(mx1), mx1e = dn(mx1), mn1w = up(mn1), mn1e = dn(mn1);
            const float c0w = up(c0[q]);
            s.lx3 = lx2;
            s.lx3e = lx2e;
            s.ly3 = ly2;
            s.qx3 = fqmax;
            s.qn3 = fqmin;
            s.rp3 = rp2;
            s.rm3 = rm2;
            s.ax2 = ax1;
            s.ax2e = ax1e;
            s.ay2 = s.ay1;
            s.ay1 = ay0;
            s.mx3 = s.mx2;
            s.mn3 = s.mn2;
            s.mx2 = mx1;
            s.mn2 = mn1;
            s.mx2w = mx1w;
            s.mx2e = mx1e;
            s.mn2w = mn1w;
            s.mn2e = mn1e;
            s.lo3 = s.lo2;
            s.lo2 = lo1;
            s.fx1 = fx0;
            s.fx1e = fx0e;
            s.fy1 = fy0;
            s.c1 = c0[q];
            s.c1w = c0w;
            s.f2 = s.f1;
            s.f1 = f0[q];
            s.f1w = f0w;
            s.f1e = f0e;
          }
          // shared per-row state
          m3 = m2;
          m2 = m1;
          m1 = m0;
          mw2 = mw1;
          me2 = me1;
          mw1 = mw0;
          me1 = me0;
          R3 = R2;
          R2 = R1;
          QF2 = QF1;
          DS3 = DS2;
          DS2 = DS1;
          DS1 = dq0.x;
          QS1 = dq0.y;
          u1 = u0;
          v1 = v0;
          d1 = d0;
          sci1 = sci0;
        }
      }
    }
  }
}

// per-cell metric factors for the column kernel: (dt2*scp2i, scp2/dt2) in FP32
__global__ void dsqs_kernel(const double *scp2, const double *scp2i, double dt2, long long n, float2 *out) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    out[t] = make_float2((float)(dt2 * scp2i[t]), (float)(scp2[t] / dt2));
}

cudaError_t launch_dsqs(const double *scp2, const double *scp2i, double dt2, long long n, float2 *out, cudaStream_t s) {
  int bx = (int)((n + 255) / 256);
  if (bx > 2048) bx = 2048;
  dsqs_kernel<<<bx, 256, 0, s>>>(scp2, scp2i, dt2, n, out);
  return cudaGetLastError();
}

cudaError_t launch_mix_fct2_col(const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm, int nq,
                                bool prep64, int seg, cudaStream_t s) {
  const int rows_max = seg + 6;
  const size_t smem = (size_t)4 * rows_max * 32 * (sizeof(float2) + 1);
  auto pick = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    kern<<<nsm * per_sm, 128, smem, s>>>(basins, items, nitems, head, rows_max);
    return cudaGetLastError();
  };
  if (nq >= 2) return prep64 ? pick(mix_fct2_col_kernel<2, true>) : pick(mix_fct2_col_kernel<2, false>);
  return prep64 ? pick(mix_fct2_col_kernel<1, true>) : pick(mix_fct2_col_kernel<1, false>);
}

}  // namespace hyc
