// hyc_tsdff.cu -- lateral diffusion at the end of tsadvc (mod_tsadvc.F90:
// 2138-2230; tsdff_2x :2262-2350, tsdff_1x :2352-2440) and the density
// update of the diffused layers through the 17-term equation of state
// (stmt_fns.h:183-218, :249-263, :496-505; EOS_17T with EOS_SIG2).
//
// The reference diffuses field after field, layer after layer: the
// face fluxes of the whole slice first (margin 1), then the in-place update
// of the sea cells (margin 0).  Every (field, layer) is independent, so one
// launch covers all of them: a CTA owns a 32x32 tile of one layer, computes
// the face factors temdf2*aspux*scuy*harmonc(h(i-1),h(i)) once for all the
// layer's fields, and writes each field's new values into a scratch slice
// (a neighbouring tile still reads the old values as its halo).  A second
// launch copies the new values into level n and recomputes th3d from the
// new temperature and salinity.
//
// FP64, built without FMA contraction, in the reference's operation order:
// the results equal the oracle's bit for bit.  The path is bound by the FP64
// pipe (three correctly rounded divisions per cell and layer for the
// fluxes, a division and a square root for the density), not by HBM.
#include <cuda_runtime.h>

#include <cstdint>

#include "hyc_args.h"
#include "hyc_device.cuh"
#include "hyc_eos.cuh"
#include "hyc_internal.h"

namespace hyc {

namespace {

constexpr int kTX = 32, kTY = 32;        // tile (cells)
constexpr int kBX = kTX + 2, kBY = kTY + 2;  // tile plus a one-cell ring
constexpr int kThreads = 256;            // 32 x 8; a thread owns 4 rows of one column
constexpr double kEpsHar = 1.0e-20;      // eps_har, mod_tsadvc.F90:1762-1763

// harmonic means, mod_tsadvc.F90:1770-1771 (max on the integer pipes,
// kmax/pos0 of hyc_device.cuh)
__device__ __forceinline__ double harmonz(double a, double b) { return 2.0 * a * b / kmax((a + b), 2.0 * kEpsHar); }
__device__ __forceinline__ double harmonc(double aa, double bb) { return harmonz(pos0(aa), pos0(bb)); }

__device__ __forceinline__ long long cell(const TsdffArgs &A, int i, int j) {
  return (long long)(i + A.nb - 1) + (long long)(j + A.nb - 1) * A.ld1;
}

// One (32x32 tile, layer) per CTA; every field of the layer.
__global__ void __launch_bounds__(kThreads) tsdff_tile_kernel(const TsdffArgs A, int ntx) {
  __shared__ double sh[kBY][kBX];      // dp(k,n)*onetamas(n) on the tile and its ring
  __shared__ double sf[kBY][kBX];      // the field being diffused (old values)
  __shared__ double fu[kTY][kTX + 1];  // u-face factors of faces i0..i0+32 (0 where iu = 0)
  __shared__ double fv[kTY + 1][kTX];  // v-face factors of faces j0..j0+32
  __shared__ uint8_t sm[kBY][kBX];     // masks
  const int k = blockIdx.y;
  const int i0 = 1 + (int)(blockIdx.x % ntx) * kTX, j0 = 1 + (int)(blockIdx.x / ntx) * kTY;
  const int tid = threadIdx.x;
  const long long lk = (long long)k * A.slice;
  // box cells i0-1..i0+32, j0-1..j0+32 that any needed face touches: i <= ii+1, j <= jj+1
  const int bi1 = min(kBX, A.ii + 2 - (i0 - 1)), bj1 = min(kBY, A.jj + 2 - (j0 - 1));
  for (int t = tid; t < kBX * kBY; t += kThreads) {
    const int bj = t / kBX, bi = t - bj * kBX;
    if (bi < bi1 && bj < bj1) {
      const long long c = cell(A, i0 - 1 + bi, j0 - 1 + bj);
      sh[bj][bi] = A.dpn[lk + c] * A.oneta[c];
      sm[bj][bi] = A.msk[c];
    } else {
      sh[bj][bi] = 0.0;
      sm[bj][bi] = 0;
    }
  }
  __syncthreads();
  // face factors (tsdff_2x :2274-2287): u-faces i in i0..min(i0+32, ii+1), rows j0..min(j0+31, jj)
  for (int t = tid; t < kTY * (kTX + 1); t += kThreads) {
    const int b = t / (kTX + 1), a = t - b * (kTX + 1);
    double f = 0.0;
    if (a < bi1 - 1 && b < bj1 - 2 && (sm[b + 1][a + 1] & kIU)) {
      const long long c = cell(A, i0 + a, j0 + b);
      f = A.temdf2 * A.aspux[c] * A.scuy[c] * harmonc(sh[b + 1][a], sh[b + 1][a + 1]);
    }
    fu[b][a] = f;
  }
  for (int t = tid; t < (kTY + 1) * kTX; t += kThreads) {
    const int b = t / kTX, a = t - b * kTX;
    double f = 0.0;
    if (a < bi1 - 2 && b < bj1 - 1 && (sm[b + 1][a + 1] & kIV)) {
      const long long c = cell(A, i0 + a, j0 + b);
      f = A.temdf2 * A.aspvy[c] * A.scvx[c] * harmonc(sh[b][a + 1], sh[b + 1][a + 1]);
    }
    fv[b][a] = f;
  }
  // update factors of this thread's cells (:2335-2336)
  const int a = tid & 31, b0 = tid >> 5;
  const int i = i0 + a;
  double fac[4];
  bool sea[4];
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int b = b0 + 8 * r, j = j0 + b;
    sea[r] = i <= A.ii && j <= A.jj && (sm[b + 1][a + 1] & kIP);
    fac[r] = sea[r] ? -A.delt1 / (A.scp2[cell(A, i, j)] * kmax(sh[b + 1][a + 1], kEpsHar)) : 0.0;
  }
  for (int q = 0; q < A.nfld; q++) {
    const double *f = A.fld[q] + lk;
    __syncthreads();  // sf free, fu/fv written
    for (int t = tid; t < kBX * kBY; t += kThreads) {
      const int bj = t / kBX, bi = t - bj * kBX;
      sf[bj][bi] = (bi < bi1 && bj < bj1) ? f[cell(A, i0 - 1 + bi, j0 - 1 + bj)] : 0.0;
    }
    __syncthreads();
    double *out = A.out + ((long long)q * A.kdm + k) * A.slice;
#pragma unroll
    for (int r = 0; r < 4; r++) {
      if (!sea[r]) continue;
      const int b = b0 + 8 * r, j = j0 + b;
      const double fc = sf[b + 1][a + 1];
      const double uw = (sm[b + 1][a + 1] & kIU) ? fu[b][a] * (sf[b + 1][a] - fc) : 0.0;
      const double ue = (sm[b + 1][a + 2] & kIU) ? fu[b][a + 1] * (fc - sf[b + 1][a + 2]) : 0.0;
      const double vs = (sm[b + 1][a + 1] & kIV) ? fv[b][a] * (sf[b][a + 1] - fc) : 0.0;
      const double vn = (sm[b + 2][a + 1] & kIV) ? fv[b + 1][a] * (fc - sf[b + 2][a + 1]) : 0.0;
      const double util = ((ue - uw) + (vn - vs)) * fac[r];
      out[cell(A, i, j)] = fc + util;
    }
  }
}

// New values into level n at the sea cells of the interior; th3d from the
// new temperature and salinity (:2199-2229, the ldtemp branch).
__global__ void tsdff_store_kernel(const TsdffArgs A) {
  const int k = blockIdx.y;
  const long long lk = (long long)k * A.slice;
  const long long n = (long long)A.ii * A.jj;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int j = 1 + (int)(t / A.ii), i = 1 + (int)(t - (long long)(j - 1) * A.ii);
    const long long c = cell(A, i, j);
    if (!(A.msk[c] & kIP)) continue;
    double tn = 0.0, sn = 0.0;
    for (int q = 0; q < A.nfld; q++) {
      const double v = A.out[((long long)q * A.kdm + k) * A.slice + c];
      A.fld[q][lk + c] = v;
      if (q == A.eos_t) tn = v;
      if (q == A.eos_s) sn = v;
    }
    if (A.eos_t >= 0) A.th3d[lk + c] = sig17(tn, sn) - A.thbase;
  }
}

}  // namespace

cudaError_t launch_tsdff(const TsdffArgs &a, cudaStream_t s) {
  if (a.nfld < 1 || a.nfld > kMaxFields || a.kdm < 1 || a.kdm > 65535) return cudaErrorInvalidValue;
  const int ntx = (a.ii + kTX - 1) / kTX, nty = (a.jj + kTY - 1) / kTY;
  tsdff_tile_kernel<<<dim3((unsigned)(ntx * nty), (unsigned)a.kdm), kThreads, 0, s>>>(a, ntx);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const long long n = (long long)a.ii * a.jj;
  long long bx = (n + 255) / 256;
  if (bx > 4096) bx = 4096;
  tsdff_store_kernel<<<dim3((unsigned)bx, (unsigned)a.kdm), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace hyc
