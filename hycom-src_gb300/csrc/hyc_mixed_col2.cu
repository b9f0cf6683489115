// hyc_mixed_col2.cu -- FP32-mixed FCT2, FCT4 and MPDATA ensemble kernel: a warp marches a
// 64-column strip north through the rows, two columns per lane, with the
// rows streamed into a per-warp shared-memory ring by TMA.
//
// Work item: (basin, strip, segment of rows, chunk of layers), all the
// launch's tracers of the basin (its table entry's q0 .. q0+ntr-1).  The
// strip starts at padded column s = 56*w (a multiple of 4, so every TMA box
// starts on a 16-byte boundary), lane l owns columns s+2l and s+2l+1, and
// the 56 columns s+4 .. s+59 are updated (the scheme reaches 3 cells).
//
// Memory: lane 0 of each warp keeps kNS blocks of kRB rows in flight.  A
// block holds, per row, the old and centre levels of the pass's tracers,
// uflx, vflx (FP32), dp (FP64) and the per-cell word (dt2*scp2i in FP64
// with ip, iu, iv in its three lowest mantissa bits) -- one
// cp.async.bulk.tensor per array, one mbarrier per slot.  Out-of-range rows
// and columns arrive as zeros (TMA fill), so the kernel has no bounds tests
// on loads.
//
// Compute: the stage pipeline of mod_tsadvc.F90:645-997 runs in registers --
// at row J the lane forms the low-order fluxes of row J (:686-720), the
// low-order solution and antidiffusive fluxes of row J-1 (:778-855), the
// Zalesak ratios and limited fluxes of row J-2 (:863-946) and the update of
// row J-3 (:962-982).  With two columns per lane, one shuffle moves a value
// across the lane boundary for both columns, and adds, multiplies and FMAs
// run as packed FP32x2 operations.  The flux divergences use two-sum
// compensation.
//
// Thickness factors of mod_tsadvc.F90:1905-1942, once per cell and layer
// and shared by the pass's tracers:  W = (fco+onemu)/(fcn+onemu),
// R = 1/(fcn+onemu), QF = fcn*scp2/dt2.  PREP64 (the precision form): the
// continuity update fco+onemu = (dp+onemu) + div*dt2*scp2i (one FP64 FMA),
// fcn+onemu (one FP64 add), the reciprocal R (hardware FP64 seed, one
// Newton step: two FP64 FMAs, relative error < 2^-40) and W = (fco+onemu)*R
// (one FP64 multiply) are FP64 -- five FP64-pipe operations per cell and
// layer (MPDATA, which also needs W-1 without cancellation: seven).  The
// conversions between FP32 and FP64 run on the integer pipes: on GB300 an
// F2F conversion issues on the FP64 pipe, at about 1/60 of the FP32 rate.
// Without PREP64 the factors are formed in compensated FP32.
//
// DIFF: tsadvc's lateral diffusion (mod_tsadvc.F90:2138-2230) runs on the
// new values before they are stored -- at row J the epilogue diffuses row
// J-4 against the new rows J-5 (its south-face flux, kept) and J-3 -- with
// the face factors from a per-cell grid table streamed like the cell words
// (row r of the table holds the u-factors of row r-4 and the v-factors of
// row r-3).  Advection and diffusion are then one pass over the fields.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "hyc_device.cuh"
#include "hyc_ens.h"
#include "hyc_tma.cuh"

namespace hyc {

namespace {

constexpr int kW = kCol2Box;  // staged columns per warp, two per lane
constexpr int kRB = kCol2Rows;  // rows per TMA block (the box height of the host's maps)
constexpr int kNS = 2;      // ring slots per warp
constexpr int kWarps = 4;   // warps per CTA
constexpr unsigned kFull = 0xffffffffu;

template <int SCHEME, int NQ, bool DIFF>
struct Ring {
  static constexpr int NC = SCHEME == kMPDATA ? 0 : NQ;  // centre-level rows (leapfrog schemes)
  static constexpr int FROW = kW * 4;  // one FP32 row
  static constexpr int DROW = kW * 8;  // one FP64 row
  static constexpr int OFF_FO = 0;
  static constexpr int OFF_FC = OFF_FO + NQ * kRB * FROW;
  static constexpr int OFF_U = OFF_FC + NC * kRB * FROW;
  static constexpr int OFF_V = OFF_U + kRB * FROW;
  static constexpr int OFF_DP = OFF_V + kRB * FROW;   // dp, FP64
  static constexpr int OFF_CG = OFF_DP + kRB * DROW;  // per-cell word, FP64
  static constexpr int OFF_GD = OFF_CG + kRB * DROW;  // DIFF: diffusion face factors (FP32 pairs)
  static constexpr int TX_BYTES = OFF_GD + (DIFF ? kRB * DROW : 0);
  static constexpr int SLOT = (TX_BYTES + 127) / 128 * 128;
  static constexpr int WARP = kNS * SLOT;
  static constexpr size_t SMEM = (size_t)kWarps * WARP + kWarps * kNS * 8 + 128;
};

// packed FP32x2 arithmetic (sm_100 family)
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
  unsigned long long r, x, y;
  asm("mov.b64 %0, {%1,%2};" : "=l"(x) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1,%2};" : "=l"(y) : "f"(b.x), "f"(b.y));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(x), "l"(y));
  float2 o;
  asm("mov.b64 {%0,%1}, %2;" : "=f"(o.x), "=f"(o.y) : "l"(r));
  return o;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// hardware FP64 reciprocal seed (multi-function unit; about 9x the FP64 FMA rate here)
__device__ __forceinline__ double rcp_seed64(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
}
// FP32 -> FP64 on the integer pipes: exact for normal values, +-0 for zeros
// and denormals.  The exponent is rebased by 1023-127 and the mantissa
// widened; the sign stays in bit 31 of the high word.
__device__ __forceinline__ double f2d_i(float f) {
  const unsigned b = __float_as_uint(f);
  unsigned hi = ((unsigned)((int)b >> 3) & 0x8FFFFFFFu) + 0x38000000u;
  unsigned lo = b << 29;
  if ((b & 0x7F800000u) == 0u) {
    hi = b & 0x80000000u;
    lo = 0u;
  }
  return __hiloint2double((int)hi, (int)lo);
}
// FP64 -> FP32 on the integer pipes for positive values in the FP32 normal
// range, rounded to nearest (ties away from zero): the top 32 bits after
// dropping the sign and the two high exponent bits, exponent rebased by
// 1023-127 (mod 2^32), plus the first dropped bit
__device__ __forceinline__ float d2f_pos(double x) {
  const unsigned lo = (unsigned)__double2loint(x), hi = (unsigned)__double2hiint(x);
  return __uint_as_float(__funnelshift_l(lo, hi, 3) + 0x40000000u + ((lo >> 28) & 1u));
}
// as d2f_pos for either sign; magnitudes below the FP32 normal range give +-0
__device__ __forceinline__ float d2f_i(double x) {
  const unsigned lo = (unsigned)__double2loint(x), hi = (unsigned)__double2hiint(x);
  const unsigned t = __funnelshift_l(lo, hi, 3) + 0x40000000u + ((lo >> 28) & 1u);
  const unsigned m = ((hi >> 20) & 0x7FFu) > 0x380u ? (t & 0x7FFFFFFFu) : 0u;
  return __uint_as_float(m | (hi & 0x80000000u));
}
// max(x, onemu) by one signed comparison of the bit patterns: for positive
// operands their integer order is the numeric order, and a negative x
// (sign bit set) compares below onemu
__device__ __forceinline__ double max_onemu(double x) {
  return __double_as_longlong(x) < __double_as_longlong(kOnemu) ? kOnemu : x;
}
// 1/h: hardware seed and one Newton step in FP64 (h >= onemu > 0)
__device__ __forceinline__ double rcp64(double h) {
  const double r = rcp_seed64(h);
  return __fma_rn(r, __fma_rn(-h, r, 1.0), r);
}
// ((a - b) + (c - d)) with the rounding errors of the two differences added
// back (two-sum), both columns at once
__device__ __forceinline__ float2 comp_div2(float2 a, float2 b, float2 c, float2 d) {
  const float2 s1 = sub2(a, b), t1 = sub2(s1, a);
  const float2 e1 = sub2(sub2(a, sub2(s1, t1)), add2(b, t1));
  const float2 s2 = sub2(c, d), t2 = sub2(s2, c);
  const float2 e2 = sub2(sub2(c, sub2(s2, t2)), add2(d, t2));
  return add2(add2(s1, s2), add2(e1, e2));
}
// the column west / east of each of this lane's two columns
__device__ __forceinline__ float2 west(float2 x) { return make_float2(__shfl_up_sync(kFull, x.y, 1), x.x); }
__device__ __forceinline__ float2 east(float2 x) { return make_float2(x.y, __shfl_down_sync(kFull, x.x, 1)); }
__device__ __forceinline__ float2 sel(bool pa, bool pb, float2 a, float2 b) {
  return make_float2(pa ? a.x : b.x, pb ? a.y : b.y);
}
__device__ __forceinline__ float2 min2(float2 a, float2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }
// harmonc of mod_tsadvc.F90:1770-1771 on the clipped thicknesses, both
// columns: 2ab/max(a+b, 2*eps_har)
__device__ __forceinline__ float2 harmonic2(float2 a, float2 b) {
  const float2 t = add2(a, b);
  const float2 r = make_float2(rcp_approx(fmaxf(t.x, 2.0e-20f)), rcp_approx(fmaxf(t.y, 2.0e-20f)));
  return mul2(mul2(mul2(a, make_float2(2.f, 2.f)), b), r);
}
__device__ __forceinline__ float2 pos2(float2 a) { return make_float2(fmaxf(a.x, 0.f), fmaxf(a.y, 0.f)); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(fminf(a.x, 0.f), fminf(a.y, 0.f)); }


// pipeline registers of one tracer, both columns.  Land neighbours drop
// out of the 5-point extrema of the field by carrying a copy of it that is
// NaN where ip = 0: max.f32 and min.f32 return the other operand when one
// is NaN, so one copy serves the maxima and the minima (the centre operand
// is the unmasked field, so no extremum is NaN).  The extrema of fmxlo and
// fmnlo carry -BIG (maxima) or +BIG (minima) masked copies, and so does
// MPDATA's field (measured faster there).
struct St2 {
  float2 f1;                 // fld at J-1
  float2 fN1, fN2;           // fld at J-1, J-2, NaN at land cells
  float2 c1, c2, c3;         // fldc at J-1 (J-2, J-3: FCT4's y stencil)
  float2 fx1, fy1;           // low-order x (west face) / y (south face) fluxes of row J-1
  float2 lo2, lo3;           // fldlo at J-2, J-3
  float2 mxA2, mnB2, mxA3, mnB3;  // fmxlo/fmnlo at J-2, J-3, masked
  float2 ax2, ay1, ay2;      // antidiffusive x-flux of row J-2; y-fluxes of the south faces of
                             // rows J-1, J-2 (FCT4: ay1 = face J-2, its face J-1 formed at row J)
  float2 rp3, rm3;           // Zalesak ratios at J-3
  float2 lx3, ly3;           // limited fluxes of row J-3
  float2 qx3, qn3;           // fqmax/fqmin at J-3
};
// MPDATA pipeline registers of one tracer, both columns (f-space: the
// posdef offset enters through the mass-flux divergence only)
struct StM {
  float2 f1;                  // fld at J-1
  float2 fA1, fB1, fA2, fB2;  // fld at J-1, J-2 masked for maxima (A) / minima (B)
  float2 fx1, fy1;            // low-order x (west face) / y (south face) fluxes of row J-1, f part
  float2 tx1, ty1;            // .5|u|(f-f_w) of row J-1 (x), .5|v|(f-f_s) of the south face of J-1
  float2 fg2;                 // flxdiv (with posdef) of row J-2
  float2 lo2, lo3;            // fldlo - posdef at J-2, J-3
  float2 mx2, mn2, mx3, mn3;  // fmx/fmn - posdef at J-2, J-3
  float2 ax2, ay2;            // antidiffusive x-flux of row J-2, y-flux of the south face of J-2
  float2 rp3, rm3;            // ratios at J-3
  float2 lx3, ly3;            // limited fluxes of row J-3
};
constexpr float kBig = 1.0e30f;   // land sentinel of the masked extrema (finite: no inf*0)
// Store a row's results after every tracer of the pass is computed: the
// tracer loop is then one branch-free block whose independent chains the
// compiler can interleave (stores inside it split it at each tracer).
constexpr bool kLateStore = true;

}  // namespace

template <int SCHEME, int NQ, bool PREP64, bool DIFF>
__global__ void __launch_bounds__(kWarps * 32, NQ == 1 ? 3 : 2)
    mix_col2_kernel(const MixBasin *__restrict__ basins, const int4 *__restrict__ items, int nitems, int *head,
                    int *err) {
  using RG = Ring<SCHEME, NQ, DIFF>;
  // rows fed before the first stored row: the scheme reaches 3 rows; the
  // diffusion epilogue stores row J-4 and needs the new values of J-5..J-3
  constexpr int kLead = DIFF ? 4 : 3;
  constexpr bool MP = SCHEME == kMPDATA;
  constexpr bool F4 = SCHEME == kFCT4;
  using St = typename std::conditional<MP, StM, St2>::type;
  extern __shared__ unsigned char c2raw_[];
  unsigned char *sm = (unsigned char *)(((uintptr_t)c2raw_ + 127) & ~(uintptr_t)127);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned char *ring = sm + wid * RG::WARP;
  uint64_t *bar = (uint64_t *)(sm + kWarps * RG::WARP) + wid * kNS;  // full[kNS]
  if (lane == 0) {
    for (int s = 0; s < kNS; s++) tma::bar_init(bar + s, 1);
    tma::fence_bar_init();
  }
  __syncwarp();
  uint32_t tg = 0;  // blocks this warp has consumed (slot and phase of the next one)
  const float onemu = (float)kOnemu;
  const float2 onemu2 = make_float2(onemu, onemu);

  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(head, 1);
    it = __shfl_sync(kFull, it, 0);
    if (it >= nitems) break;
    const int4 w = items[it];
    const MixBasin &B = basins[w.x];
    const int ii = B.ii, jj = B.jj, nb = B.nbdy, ld1 = B.ld1, kdm = B.kdm, images = B.images;
    const int q0 = B.q0, ntr = B.ntr;  // this launch's tracers: q0 .. q0+ntr-1
    float *const fnew = B.fnew;
    const long long sl = B.slice;
    const int s0 = 56 * w.y;  // strip start (padded column)
    const int j0 = 1 + w.z * B.seg, j1 = min(j0 + B.seg, jj + 1);
    const int nblk = (j1 - j0 + 2 * kLead + kRB - 1) / kRB;
    const int nqp = (ntr + NQ - 1) / NQ;
    const int ka = w.w * B.kchunk, kb = min(kdm, ka + B.kchunk);  // this item's layers
    const int T = (kb - ka) * nqp * nblk;
    // this lane's columns: padded a0 = s0 + 2*lane (A) and a0 + 1 (B)
    const int a0 = s0 + 2 * lane;
    const int iA = a0 - nb + 1, iB = iA + 1;  // Fortran indices
    const bool outA = lane >= 2 && lane < 30 && iA >= 1 && iA <= ii;
    const bool outB = lane >= 2 && lane < 30 && iB >= 1 && iB <= ii;

    auto issue = [&](int t) {  // lane 0: block t of this item into its slot
      const int kk = t / (nqp * nblk);
      const int rem = t - kk * nqp * nblk;
      const int k = ka + kk;
      const int qp = rem / nblk, blk = rem - qp * nblk;
      const int y = j0 - kLead + blk * kRB + nb - 1;
      const uint32_t g = tg + t;
      unsigned char *slot = ring + (g % kNS) * RG::SLOT;
      uint64_t *b = bar + (g % kNS);
      tma::expect_tx(b, RG::TX_BYTES);
#pragma unroll
      for (int q = 0; q < NQ; q++) {
        const int qq = q0 + min(qp * NQ + q, ntr - 1);
        tma::load3(slot + RG::OFF_FO + q * kRB * RG::FROW, B.c2_old, b, s0, y, qq * kdm + k);
        if (!MP) tma::load3(slot + RG::OFF_FC + q * kRB * RG::FROW, B.c2_cur, b, s0, y, qq * kdm + k);
      }
      tma::load3(slot + RG::OFF_U, B.c2_u, b, s0, y, k);
      tma::load3(slot + RG::OFF_V, B.c2_v, b, s0, y, k);
      tma::load3(slot + RG::OFF_DP, B.c2_dp, b, s0, y, k);
      tma::load3(slot + RG::OFF_CG, B.c2_cg, b, s0, y, 0);
      if (DIFF) {
        tma::load3(slot + RG::OFF_GD, B.c2_gd, b, s0, y, 0);
      }
    };
    if (lane == 0)
      for (int d = 0; d < kNS && d < T; d++) issue(d);

    int t = 0;
    bool ok = true;
    for (int k = ka; k < kb && ok; k++) {
      for (int qp = 0; qp < nqp && ok; qp++) {
        const int qb = qp * NQ;  // this pass's tracers: qb .. qb+nq-1
        const int nq = min(NQ, ntr - qb);
        float *fn[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++)
          fn[q] = fnew + ((long long)(q0 + min(qb + (q < nq ? q : 0), ntr - 1)) * kdm + k) * sl;
        St S[NQ];
        float P[NQ];  // posdef of each tracer of the pass (MPDATA)
#pragma unroll
        for (int q = 0; q < NQ; q++) {
          S[q] = St{};
          P[q] = B.posdef[q0 + min(qb + q, ntr - 1)];
        }
        const float2 z2 = make_float2(0.f, 0.f);
        float2 u1 = z2, u1m = z2, v1 = z2, R2 = z2, nR3 = z2, QF2 = z2, DS1 = z2, DS2 = z2, DS3 = z2, QS1 = z2;
        float2 v1m = z2, H2 = z2;  // MPDATA, FCT4: masked v of row J-1; MPDATA: fco+fcn of row J-2
        float2 IU1 = z2, IV1 = z2, IV2 = z2;  // FCT4: iu of row J-1, iv of rows J-1, J-2 (0/1)
        float2 L1 = z2, L2 = z2, L3 = z2;  // land flags (1 = land) of rows J-1, J-2, J-3
        float L2e = 0.f;                   // land flag east of column B, row J-2
        double dA1 = 0.0, dB1 = 0.0;       // dp of row J-1
        double sA1 = 0.0, sB1 = 0.0;       // dt2*scp2i of row J-1 (FP64 prep)
        // DIFF: new values of row J-4 and the diffusive flux through its south face, per tracer;
        // max(dp,0), dt2*scp2i and the land flags of row J-4
        float2 D1[NQ], VF1[NQ];
#pragma unroll
        for (int q = 0; q < NQ; q++) D1[q] = VF1[q] = z2;
        float2 h4 = z2, DS4 = z2, L4 = z2;
        float2 hq1 = z2, hq2 = z2;  // DIFF: max(dp,0) of rows J-2, J-3 (FP32, from the thickness prep)
        for (int blk = 0; blk < nblk; blk++, t++) {
          const uint32_t g = tg + t;
          if (!__all_sync(kFull, tma::wait(bar + (g % kNS), (g / kNS) & 1u, err))) {
            // give the other copies in flight a bounded chance to land, then stop
            for (int d = 1; d < kNS && t + d < T; d++) tma::wait(bar + ((g + d) % kNS), ((g + d) / kNS) & 1u, nullptr);
            ok = false;
            break;
          }
          const unsigned char *slot = ring + (g % kNS) * RG::SLOT;
#pragma unroll(PREP64 ? 2 : kRB)
          for (int rr = 0; rr < kRB; rr++) {
            const int J = j0 - kLead + blk * kRB + rr;
            // ---- inputs of row J
            const float2 u0 = ((const float2 *)(slot + RG::OFF_U + rr * RG::FROW))[lane];
            const float2 v0 = ((const float2 *)(slot + RG::OFF_V + rr * RG::FROW))[lane];
            const double2 d0 = ((const double2 *)(slot + RG::OFF_DP + rr * RG::DROW))[lane];
            const double2 cg = ((const double2 *)(slot + RG::OFF_CG + rr * RG::DROW))[lane];
            // per-cell word: dt2*scp2i with ip, iu, iv in the three lowest mantissa bits
            const unsigned mA = (unsigned)__double2loint(cg.x), mB = (unsigned)__double2loint(cg.y);
            const float2 ds0 = make_float2(d2f_pos(cg.x), d2f_pos(cg.y));  // FP32 dt2*scp2i (2.0 off the arrays)
            const float2 giu = make_float2((mA & kIU) ? 1.f : 0.f, (mB & kIU) ? 1.f : 0.f);
            const float2 giv = make_float2((mA & kIV) ? 1.f : 0.f, (mB & kIV) ? 1.f : 0.f);
            // scp2/dt2 = 1/(dt2*scp2i) at sea cells (scp2i = 1/scp2, geopar.F90:320), 0 on land
            const float2 qs0 = make_float2((mA & kIP) ? rcp_approx(ds0.x) : 0.f, (mB & kIP) ? rcp_approx(ds0.y) : 0.f);
            float2 f0[NQ], c0[NQ];
#pragma unroll
            for (int q = 0; q < NQ; q++) {
              f0[q] = ((const float2 *)(slot + RG::OFF_FO + (q * kRB + rr) * RG::FROW))[lane];
              c0[q] = MP ? z2 : ((const float2 *)(slot + RG::OFF_FC + (q * kRB + rr) * RG::FROW))[lane];
            }

            // ---- thickness factors of row J-1 (mod_tsadvc.F90:1905-1942)
            float2 W1, R1, QF1, Wm1, H1;  // Wm1 = W-1 and H1 = fco+fcn (MPDATA only)
            float2 hc1 = z2;              // DIFF: max(dp,0) of row J-1
            float2 dv;                    // FP64 prep: the divergence of the face fluxes of row J-1
            bool unA = false, unB = false;  // FP64 prep, MPDATA: fco = dp + div*dt2*scp2i (no clip)
            if (PREP64) {
              // continuity (:1931-1936): the face-flux differences and their sum by
              // two-sum in FP32, scaled by dt2*scp2i and added to dp in FP64
              dv = comp_div2(east(u1), u1, v0, v1);
              const double bA = dA1 + kOnemu, bB = dB1 + kOnemu;       // dp + onemu
              // fcn + onemu = max(dp, 0) + onemu (dp = -0 gives onemu either way)
              const double hA = __double2hiint(dA1) >= 0 ? bA : kOnemu, hB = __double2hiint(dB1) >= 0 ? bB : kOnemu;
              const double rA = rcp64(hA), rB = rcp64(hB);
              const float2 hf = make_float2(d2f_pos(hA), d2f_pos(hB));
              if (!MP) {
                // fco + onemu = max(dp + div*dt2*scp2i, 0) + onemu
                const double cA = max_onemu(__fma_rn(f2d_i(dv.x), sA1, bA));
                const double cB = max_onemu(__fma_rn(f2d_i(dv.y), sB1, bB));
                W1 = make_float2(d2f_pos(cA * rA), d2f_pos(cB * rB));
              } else {
                const double fA = f2d_i(dv.x) * sA1, fB = f2d_i(dv.y) * sB1;
                const double cA = kmax(bA + fA, kOnemu), cB = kmax(bB + fB, kOnemu);
                unA = ge0(dA1) && !klt(bA + fA, kOnemu);
                unB = ge0(dB1) && !klt(bB + fB, kOnemu);
                Wm1 = make_float2(d2f_i((cA - hA) * rA), d2f_i((cB - hB) * rB));
                W1 = add2(Wm1, make_float2(1.f, 1.f));
                H1 = add2(sub2(make_float2(d2f_pos(cA), d2f_pos(cB)), onemu2), sub2(hf, onemu2));
              }
              R1 = make_float2(d2f_pos(rA), d2f_pos(rB));
              QF1 = mul2(sub2(hf, onemu2), QS1);  // fcn*scp2/dt2
              if (DIFF) hc1 = sub2(hf, onemu2);
            } else {
              const float2 fdv = mul2(comp_div2(east(u1), u1, v0, v1), DS1);
              const float2 d = make_float2(d2f_i(dA1), d2f_i(dB1));
              const float2 fcn = pos2(d);
              const float2 r = make_float2(rcp_approx(fcn.x + onemu), rcp_approx(fcn.y + onemu));
              const float2 w1 = fma2(fdv, r, make_float2(1.f, 1.f));
              W1.x = (d.x + fdv.x > 0.f) ? (d.x >= 0.f ? w1.x : (d.x + fdv.x + onemu) * r.x) : onemu * r.x;
              W1.y = (d.y + fdv.y > 0.f) ? (d.y >= 0.f ? w1.y : (d.y + fdv.y + onemu) * r.y) : onemu * r.y;
              R1 = r;
              QF1 = mul2(fcn, QS1);
              if (MP) {
                const float2 wm = mul2(fdv, r);  // W-1 without the rounding of W
                Wm1.x = (d.x + fdv.x > 0.f && d.x >= 0.f) ? wm.x : W1.x - 1.f;
                Wm1.y = (d.y + fdv.y > 0.f && d.y >= 0.f) ? wm.y : W1.y - 1.f;
                H1 = add2(pos2(add2(d, fdv)), fcn);
              }
            }
            const float2 nR1 = make_float2(-R1.x, -R1.y);
            // face fluxes with the face masks applied (iu/iv = 0 faces carry no
            // advective or antidiffusive flux, mod_tsadvc.F90:738-758), split for the
            // upwind choice: u*f_upwind = max(u,0)*f_west + min(u,0)*f (one of the two
            // products is zero, so the rounding is that of u*f)
            const float2 u0m = mul2(u0, giu), v0m = mul2(v0, giv);
            const float2 un0 = neg2(u0m), vn0 = neg2(v0m);
            const float2 up0 = sub2(u0m, un0), vp0 = sub2(v0m, vn0);  // max(x,0) = x - min(x,0), exact
            const float2 half = make_float2(0.5f, 0.5f);
            const float2 u1h = mul2(u1m, half), v0h = mul2(v0m, half), v1h = mul2(v1m, half);
            const float2 F14 = make_float2(7.f / 12.f, 7.f / 12.f), F24 = make_float2(-1.f / 12.f, -1.f / 12.f);
            // land flags (1 = land)
            const float2 L0 = make_float2((mA & kIP) ? 0.f : 1.f, (mB & kIP) ? 0.f : 1.f);
            const float qnan = __int_as_float(0x7fc00000);
            const float2 M0 = make_float2((mA & kIP) ? 0.f : qnan, (mB & kIP) ? 0.f : qnan);  // NaN on land
            const bool ip1A = L1.x == 0.f, ip1B = L1.y == 0.f;
            const bool ip2B = L2.y == 0.f, ip2E = L2e == 0.f;  // column B and its east neighbour, row J-2
            const bool ip3A = L3.x == 0.f, ip3B = L3.y == 0.f;
            const int jo = J - kLead;  // the row stored at this step
            const bool rowout = jo >= j0 && jo < j1;
            const bool stA = rowout && outA && (DIFF ? L4.x == 0.f : ip3A), stB = rowout && outB && (DIFF ? L4.y == 0.f : ip3B);
            const float2 nbig = make_float2(-kBig, -kBig), pbig = make_float2(kBig, kBig);
            // MPDATA (mod_tsadvc.F90:207-493), shared by the tracers:
            //  du1  divergence of the masked mass fluxes of row J-1 (the posdef part of
            //       flxdiv is posdef*du1);
            //  Z1   (W-1) - du1*R: lo = f*W - fdiv*R + posdef*Z1 is the low-order
            //       solution with posdef taken out (Z1 = 0 when the mass fluxes at
            //       closed faces are zero);
            //  uD1, vD1  u/((fco2+fcn2)+onemu) of the west and south faces of row J-1
            //       (:377-387);  ua0, va0  .5|u|, .5|v| of row J (:255, :264)
            float2 du1, Z1, uD1, vD1, ua0, va0;
            if (MP) {
              const float2 dvm = comp_div2(east(u1m), u1m, v0m, v1m);  // of the masked mass fluxes
              du1 = mul2(dvm, DS1);
              Z1 = fma2(du1, nR1, Wm1);
              if (PREP64) {
                // unclipped, W-1 - du*R = (div - div_masked)*dt2*scp2i*R: formed from the
                // difference of the two divergences, which is exactly 0 wherever no
                // closed face carries a flux, instead of from W-1 (FP64) and du*R (FP32)
                const float2 zd = mul2(mul2(sub2(dv, dvm), DS1), R1);
                Z1 = sel(unA, unB, zd, Z1);
              }
              const float2 Hw = west(H1);
              uD1 = make_float2(u1m.x * rcp_approx((H1.x + Hw.x) + onemu), u1m.y * rcp_approx((H1.y + Hw.y) + onemu));
              vD1 = make_float2(v1m.x * rcp_approx((H1.x + H2.x) + onemu), v1m.y * rcp_approx((H1.y + H2.y) + onemu));
              ua0 = mul2(make_float2(fabsf(u0m.x), fabsf(u0m.y)), half);
              va0 = mul2(make_float2(fabsf(v0m.x), fabsf(v0m.y)), half);
            }

            // FCT4 (mod_tsadvc.F90:1534-1555): 4th-order antidiffusive fluxes where
            // both neighbouring faces are open, else 2nd order -- x faces of row J-1
            // (iu(i-1), iu(i+1) of row J-1), the y face J-1 (iv of rows J-2 and J)
            bool x4A = false, x4B = false, y4A = false, y4B = false;
            if (F4) {
              const float iuwB = __shfl_up_sync(kFull, IU1.y, 1), iueA = __shfl_down_sync(kFull, IU1.x, 1);
              x4A = iuwB != 0.f && IU1.y != 0.f;
              x4B = IU1.x != 0.f && iueA != 0.f;
              y4A = IV2.x != 0.f && giv.x != 0.f;
              y4B = IV2.y != 0.f && giv.y != 0.f;
            }
            float2 res[NQ];
            auto store_row = [&](int q, float resA, float resB) {
              float *p = fn[q] + (long long)a0 + (long long)(jo + nb - 1) * ld1;
              if (stA && stB) {
                __stcs((float2 *)p, make_float2(resA, resB));  // a0 is even, ld1 a multiple of 4: 8-byte aligned
              } else {
                if (stA) __stcs(p, resA);
                if (stB) __stcs(p + 1, resB);
              }
              if (images) {
                if (stA && iA <= images) p[ii] = resA;
                if (stA && iA > ii - images) p[-ii] = resA;
                if (stB && iB <= images) p[1 + ii] = resB;
                if (stB && iB > ii - images) p[1 - ii] = resB;
              }
            };
            if constexpr (!MP) {
#pragma unroll
            for (int q = 0; q < NQ; q++) {
              St &s = S[q];
              // S1: low-order fluxes of row J (:686-720)
              const float2 fx0 = fma2(up0, west(f0[q]), mul2(un0, f0[q]));
              const float2 fy0 = fma2(vp0, s.f1, mul2(vn0, f0[q]));
              const float2 fN0 = add2(f0[q], M0);  // exact at sea cells, NaN on land
              // S2: low-order solution of row J-1 (:778-791), extrema over sea neighbours
              const float2 c = s.f1;
              const float2 fw = west(s.fN1), fe = east(s.fN1);
              const float fmxA = max3f(max3f(c.x, fw.x, fe.x), s.fN2.x, fN0.x);
              const float fmxB = max3f(max3f(c.y, fw.y, fe.y), s.fN2.y, fN0.y);
              const float fmnA = min3f(min3f(c.x, fw.x, fe.x), s.fN2.x, fN0.x);
              const float fmnB = min3f(min3f(c.y, fw.y, fe.y), s.fN2.y, fN0.y);
              const float2 fdv = mul2(comp_div2(east(s.fx1), s.fx1, fy0, s.fy1), DS1);
              const float2 t1 = fma2(c, W1, mul2(fdv, nR1));
              const float2 lo1 = make_float2(fmaxf(fmnA, fminf(fmxA, t1.x)), fmaxf(fmnB, fminf(fmxB, t1.y)));
              // S3: antidiffusive fluxes, x of row J-1 and y of row J (:817-833); FCT4:
              // x of row J-1 and y of the face J-1 (:1534-1555), whose stencil
              // reaches row J
              float2 ax1, ayn;
              if constexpr (!F4) {
                ax1 = sub2(mul2(u1h, add2(s.c1, west(s.c1))), s.fx1);
                ayn = sub2(mul2(v0h, add2(c0[q], s.c1)), fy0);
              } else {
                const float cwB = __shfl_up_sync(kFull, s.c1.y, 1), cwA = __shfl_up_sync(kFull, s.c1.x, 1);
                const float ceA = __shfl_down_sync(kFull, s.c1.x, 1);
                const float2 inx = add2(s.c1, make_float2(cwB, s.c1.x));                    // c(i) + c(i-1)
                const float2 outx = add2(make_float2(s.c1.y, ceA), make_float2(cwA, cwB));  // c(i+1) + c(i-2)
                const float2 hx4 = mul2(u1m, fma2(F14, inx, mul2(F24, outx)));
                ax1 = sub2(sel(x4A, x4B, hx4, mul2(u1h, inx)), s.fx1);
                const float2 iny = add2(s.c1, s.c2), outy = add2(c0[q], s.c3);  // rows J-1 + J-2, J + J-3
                const float2 hy4 = mul2(v1m, fma2(F14, iny, mul2(F24, outy)));
                ayn = sub2(sel(y4A, y4B, hy4, mul2(v1h, iny)), s.fy1);
              }
              const float2 mx1 = make_float2(max3f(c.x, s.c1.x, lo1.x), max3f(c.y, s.c1.y, lo1.y));  // :792-793
              const float2 mn1 = make_float2(min3f(c.x, s.c1.x, lo1.x), min3f(c.y, s.c1.y, lo1.y));
              const float2 mxA1 = fma2(L1, nbig, mx1), mnB1 = fma2(L1, pbig, mn1);
              // S4: Zalesak ratios of row J-2 (:863-909)
              const float2 xw = west(s.mxA2), xe = east(s.mxA2), nw = west(s.mnB2), ne = east(s.mnB2);
              const float2 fqmax = make_float2(max3f(max3f(s.mxA2.x, xw.x, xe.x), s.mxA3.x, mxA1.x),
                                               max3f(max3f(s.mxA2.y, xw.y, xe.y), s.mxA3.y, mxA1.y));
              const float2 fqmin = make_float2(min3f(min3f(s.mnB2.x, nw.x, ne.x), s.mnB3.x, mnB1.x),
                                               min3f(min3f(s.mnB2.y, nw.y, ne.y), s.mnB3.y, mnB1.y));
              const float2 fxa = s.ax2, fxb = sel(ip2B, ip2E, east(s.ax2), s.ax2);  // ipip1 quirk (:873-883)
              // the south face of row J-2 and, with the ipjp1 quirk, its north face
              const float2 fya = F4 ? s.ay1 : s.ay2, fyb = F4 ? sel(ip1A, ip1B, ayn, s.ay1) : sel(ip1A, ip1B, s.ay1, s.ay2);
              const float2 nxa = neg2(fxa), nxb = neg2(fxb), nya = neg2(fya), nyb = neg2(fyb);
              const float2 pxa = sub2(fxa, nxa), pxb = sub2(fxb, nxb), pya = sub2(fya, nya), pyb = sub2(fyb, nyb);
              const float2 famax = sub2(add2(sub2(pxa, nxb), pya), nyb);
              const float2 famin = sub2(add2(sub2(pxb, nxa), pyb), nya);
              // rp = (qp < famax) ? qp/famax : 1, and 0 when famax <= 0 (:884-903), written
              // as min(1, qp*(1/famax)).  famax >= 0; where it is 0 the product is inf or
              // NaN and fminf returns 1, which only ever multiplies zero fluxes (no
              // antidiffusive inflow).  qp >= 0 at sea cells and 0 at land cells (scp2/dt2
              // is stored as 0 there), so every ratio is finite.
              const float2 qpv = mul2(sub2(fqmax, s.lo2), QF2), qmv = mul2(sub2(s.lo2, fqmin), QF2);
              const float2 rp2 = make_float2(fminf(1.f, qpv.x * rcp_approx(famax.x)),
                                             fminf(1.f, qpv.y * rcp_approx(famax.y)));
              const float2 rm2 = make_float2(fminf(1.f, qmv.x * rcp_approx(famin.x)),
                                             fminf(1.f, qmv.y * rcp_approx(famin.y)));
              // S5: limited fluxes of row J-2 (:922-946)
              const float2 rp2w = west(rp2), rm2w = west(rm2);
              // lx = max(ax,0)*min(rp,rm_w) + min(ax,0)*min(rp_w,rm): one product is
              // zero, so the rounding is that of the reference's single product
              const float2 nax = neg2(s.ax2), pax = sub2(s.ax2, nax);
              const float2 nay = neg2(fya), pay = sub2(fya, nay);
              const float2 lx2 = fma2(pax, min2(rp2, rm2w), mul2(nax, min2(rp2w, rm2)));
              const float2 ly2 = fma2(pay, min2(rp2, s.rm3), mul2(nay, min2(s.rp3, rm2)));
              // S6: update of row J-3 (:962-982)
              const float2 fd3 = mul2(comp_div2(east(s.lx3), s.lx3, ly2, s.ly3), DS3);
              const float2 t3 = fma2(fd3, nR3, s.lo3);
              const float resA = fmaxf(s.qn3.x, fminf(s.qx3.x, t3.x));
              const float resB = fmaxf(s.qn3.y, fminf(s.qx3.y, t3.y));
              res[q] = make_float2(resA, resB);
              if (!kLateStore && (stA || stB) && q < nq) store_row(q, resA, resB);
              // shift the pipeline one row
              s.lx3 = lx2;
              s.ly3 = ly2;
              s.qx3 = fqmax;
              s.qn3 = fqmin;
              s.rp3 = rp2;
              s.rm3 = rm2;
              s.ax2 = ax1;
              s.ay2 = s.ay1;
              s.ay1 = ayn;
              s.mxA3 = s.mxA2;
              s.mnB3 = s.mnB2;
              s.mxA2 = mxA1;
              s.mnB2 = mnB1;
              s.lo3 = s.lo2;
              s.lo2 = lo1;
              s.fx1 = fx0;
              s.fy1 = fy0;
              s.c3 = s.c2;
              s.c2 = s.c1;
              s.c1 = c0[q];
              s.fN2 = s.fN1;
              s.fN1 = fN0;
              s.f1 = f0[q];
            }
            } else {
#pragma unroll
            for (int q = 0; q < NQ; q++) {
              St &s = S[q];
              // P1: low-order fluxes (f part) of row J, tx/ty (:249-271), masked copies
              const float2 f0w = west(f0[q]);
              const float2 fx0 = fma2(up0, f0w, mul2(un0, f0[q]));
              const float2 fy0 = fma2(vp0, s.f1, mul2(vn0, f0[q]));
              const float2 tx0 = mul2(ua0, sub2(f0[q], f0w));
              const float2 ty0 = mul2(va0, sub2(f0[q], s.f1));
              const float2 fA0 = fma2(L0, nbig, f0[q]), fB0 = fma2(L0, pbig, f0[q]);
              // P1/P2: extrema of row J-1 (:272-281) and its low-order solution (:345-353)
              const float2 c = s.f1;
              const float2 aw = west(s.fA1), ae = east(s.fA1), bw = west(s.fB1), be = east(s.fB1);
              const float2 mx1 = make_float2(max3f(max3f(c.x, aw.x, ae.x), s.fA2.x, fA0.x),
                                             max3f(max3f(c.y, aw.y, ae.y), s.fA2.y, fA0.y));
              const float2 mn1 = make_float2(min3f(min3f(c.x, bw.x, be.x), s.fB2.x, fB0.x),
                                             min3f(min3f(c.y, bw.y, be.y), s.fB2.y, fB0.y));
              const float2 fdf = mul2(comp_div2(east(s.fx1), s.fx1, fy0, s.fy1), DS1);
              const float2 Pq = make_float2(P[q], P[q]);
              const float2 t1 = fma2(Pq, Z1, fma2(c, W1, mul2(fdf, nR1)));
              const float2 lo1 = make_float2(fmaxf(mn1.x, fminf(mx1.x, t1.x)), fmaxf(mn1.y, fminf(mx1.y, t1.y)));
              const float2 fg1 = fma2(Pq, du1, fdf);  // flxdiv with posdef
              // P3: antidiffusive fluxes of the west and south faces of row J-1 (:369-392)
              const float2 ax1 = sub2(s.tx1, mul2(uD1, add2(fg1, west(fg1))));
              const float2 ay1 = sub2(s.ty1, mul2(vD1, add2(fg1, s.fg2)));
              // P4: ratios of row J-2 (:405-423); ay1 is the north face of row J-2
              const float2 axe = east(s.ax2);
              const float2 nxw = neg2(s.ax2), nxe = neg2(axe), nys = neg2(s.ay2), nyn = neg2(ay1);
              const float2 pxw = sub2(s.ax2, nxw), pxe = sub2(axe, nxe), pys = sub2(s.ay2, nys), pyn = sub2(ay1, nyn);
              const float2 dp_ = add2(sub2(nxe, pxw), sub2(nyn, pys));   // flxdp + flydp
              const float2 dn_ = add2(sub2(pxe, nxw), sub2(pyn, nys));   // flxdn + flydn
              const float2 qpv = mul2(sub2(s.mx2, s.lo2), QF2), qmv = mul2(sub2(s.lo2, s.mn2), QF2);
              const float2 rp2 = make_float2(qpv.x * rcp_approx(onemu - dp_.x), qpv.y * rcp_approx(onemu - dp_.y));
              const float2 rm2 = make_float2(qmv.x * rcp_approx(onemu + dn_.x), qmv.y * rcp_approx(onemu + dn_.y));
              // P5: limited fluxes of row J-2 (:433-449)
              const float2 rp2w = west(rp2), rm2w = west(rm2);
              const float2 lx2 = fma2(pxw, make_float2(min3f(1.f, rp2.x, rm2w.x), min3f(1.f, rp2.y, rm2w.y)),
                                      mul2(nxw, make_float2(min3f(1.f, rp2w.x, rm2.x), min3f(1.f, rp2w.y, rm2.y))));
              const float2 ly2 = fma2(pys, make_float2(min3f(1.f, rp2.x, s.rm3.x), min3f(1.f, rp2.y, s.rm3.y)),
                                      mul2(nys, make_float2(min3f(1.f, s.rp3.x, rm2.x), min3f(1.f, s.rp3.y, rm2.y))));
              // P6: update of row J-3 (:465-486), posdef already out
              const float2 fd3 = mul2(comp_div2(east(s.lx3), s.lx3, ly2, s.ly3), DS3);
              const float2 t3 = fma2(fd3, nR3, s.lo3);
              const float resA = fmaxf(s.mn3.x, fminf(s.mx3.x, t3.x));
              const float resB = fmaxf(s.mn3.y, fminf(s.mx3.y, t3.y));
              res[q] = make_float2(resA, resB);
              if (!kLateStore && (stA || stB) && q < nq) store_row(q, resA, resB);
              // shift the pipeline one row
              s.lx3 = lx2;
              s.ly3 = ly2;
              s.rp3 = rp2;
              s.rm3 = rm2;
              s.ax2 = ax1;
              s.ay2 = ay1;
              s.mx3 = s.mx2;
              s.mn3 = s.mn2;
              s.mx2 = mx1;
              s.mn2 = mn1;
              s.lo3 = s.lo2;
              s.lo2 = lo1;
              s.fg2 = fg1;
              s.tx1 = tx0;
              s.ty1 = ty0;
              s.fx1 = fx0;
              s.fy1 = fy0;
              s.fA2 = s.fA1;
              s.fB2 = s.fB1;
              s.fA1 = fA0;
              s.fB1 = fB0;
              s.f1 = f0[q];
            }
            }
            if constexpr (DIFF) {
              // Laplacian diffusion of row J-4 (tsdff_2x/tsdff_1x, mod_tsadvc.F90:2262-2492) on the
              // new values: face factors temdf2*aspux*scuy (0 where iu = 0) of row J-4 and
              // temdf2*aspvy*scvx (0 where iv = 0) of row J-3 come from the grid table (its row J
              // holds them), times the harmonic mean of max(dp,0) on either side (kept in FP32
              // from the thickness prep of rows J-3 and J-4); the update is
              // -delt1/(scp2*max(dp,eps_har)) times the flux divergence, at sea cells only
              const float4 g4 = ((const float4 *)(slot + RG::OFF_GD + rr * RG::DROW))[lane];
              const float2 h3 = hq2;
              const float2 FU = mul2(make_float2(g4.x, g4.z), harmonic2(west(h4), h4));
              const float2 FV = mul2(make_float2(g4.y, g4.w), harmonic2(h4, h3));
              // delt1 is tsadvc's dt2, so delt1/scp2 = dt2*scp2i
              const float2 FP = make_float2(L4.x == 0.f ? -DS4.x * rcp_approx(fmaxf(h4.x, 1.0e-20f)) : 0.f,
                                            L4.y == 0.f ? -DS4.y * rcp_approx(fmaxf(h4.y, 1.0e-20f)) : 0.f);
#pragma unroll
              for (int q = 0; q < NQ; q++) {
                const float2 dN = D1[q];
                const float2 uw = mul2(FU, sub2(west(dN), dN));  // through the west face
                const float2 vn = mul2(FV, sub2(dN, res[q]));    // through the north face
                const float2 dvg = add2(sub2(east(uw), uw), sub2(vn, VF1[q]));
                const float2 o = fma2(dvg, FP, dN);
                if ((stA || stB) && q < nq) store_row(q, o.x, o.y);
                VF1[q] = vn;
                D1[q] = res[q];
              }
              h4 = h3;
              hq2 = hq1;
              hq1 = hc1;
              DS4 = DS3;
              L4 = L3;
            } else if (kLateStore && (stA || stB)) {
#pragma unroll
              for (int q = 0; q < NQ; q++)
                if (q < nq) store_row(q, res[q].x, res[q].y);
            }
            // shared per-row state
            L3 = L2;
            L2 = L1;
            L2e = __shfl_down_sync(kFull, L1.x, 1);  // the column east of B
            nR3 = make_float2(-R2.x, -R2.y);
            R2 = R1;
            QF2 = QF1;
            DS3 = DS2;
            DS2 = DS1;
            DS1 = ds0;
            QS1 = qs0;
            L1 = L0;
            u1 = u0;
            u1m = u0m;
            if (MP || F4) v1m = v0m;
            if (MP) H2 = H1;
            if (F4) {
              IU1 = giu;
              IV2 = IV1;
              IV1 = giv;
            }
            v1 = v0;
            dA1 = d0.x;
            dB1 = d0.y;
            if (PREP64) {  // FP64 dt2*scp2i without the mask bits
              sA1 = __hiloint2double(__double2hiint(cg.x), (int)(mA & ~7u));
              sB1 = __hiloint2double(__double2hiint(cg.y), (int)(mB & ~7u));
            }
          }
          __syncwarp();  // every lane is done with the slot before it is refilled
          if (lane == 0 && t + kNS < T) issue(t + kNS);
        }
      }
    }
    if (!ok) return;
    tg += T;
  }
}

// Failure path of the streaming kernels, exercised without a fault: one
// thread waits on an mbarrier through the same bounded wait the strip kernel
// uses for its TMA blocks.  arrive = 0: nothing completes the phase, the wait
// gives up after its limit, records the failure in *err and the kernel
// returns; arrive = 1: the phase completes first and *err is left alone.
__global__ void wait_probe_kernel(int arrive, int *err) {
  __shared__ uint64_t probe_bar;
  if (threadIdx.x == 0) {
    tma::bar_init(&probe_bar, 1);
    tma::fence_bar_init();
    if (arrive) tma::arrive(&probe_bar);
    tma::wait(&probe_bar, 0, err);
  }
}

cudaError_t launch_wait_probe(int arrive, int *err, cudaStream_t s) {
  wait_probe_kernel<<<1, 32, 0, s>>>(arrive, err);
  return cudaGetLastError();
}

// per-cell word of the strip kernel: dt2*scp2i (FP64) with ip, iu, iv in
// its three lowest mantissa bits (a relative change below 2^-49)
__global__ void cell_word_kernel(const double *scp2i, const uint8_t *msk, double dt2, long long n, double *out) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const long long b = __double_as_longlong(dt2 * scp2i[t]);
    out[t] = __longlong_as_double((b & ~7LL) | (long long)(msk[t] & (kIP | kIU | kIV)));
  }
}

cudaError_t launch_cell_words(const double *scp2i, const uint8_t *msk, double dt2, long long n, double *out,
                              cudaStream_t s) {
  int bx = (int)((n + 255) / 256);
  if (bx > 2048) bx = 2048;
  cell_word_kernel<<<bx, 256, 0, s>>>(scp2i, msk, dt2, n, out);
  return cudaGetLastError();
}

cudaError_t launch_mix_col2(int scheme, const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm,
                            int nq, bool prep64, bool diff, int *err, cudaStream_t s) {
  auto pick = [&](auto kern, size_t smem) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    kern<<<nsm * per_sm, kWarps * 32, smem, s>>>(basins, items, nitems, head, err);
    return cudaGetLastError();
  };
  if (diff && !prep64) return cudaErrorInvalidValue;  // the diffusion epilogue exists with the FP64 prep only
#define HYC_COL2(S, Q)                                                                     \
  (diff ? pick(mix_col2_kernel<S, Q, true, true>, Ring<S, Q, true>::SMEM)                  \
        : prep64 ? pick(mix_col2_kernel<S, Q, true, false>, Ring<S, Q, false>::SMEM)        \
                 : pick(mix_col2_kernel<S, Q, false, false>, Ring<S, Q, false>::SMEM))
  if (scheme == kFCT2) return nq >= 2 ? HYC_COL2(kFCT2, 2) : HYC_COL2(kFCT2, 1);
  if (scheme == kMPDATA) return nq >= 2 ? HYC_COL2(kMPDATA, 2) : HYC_COL2(kMPDATA, 1);
  if (scheme == kFCT4) return nq >= 2 ? HYC_COL2(kFCT4, 2) : HYC_COL2(kFCT4, 1);
#undef HYC_COL2
  return cudaErrorInvalidValue;
}

}  // namespace hyc
