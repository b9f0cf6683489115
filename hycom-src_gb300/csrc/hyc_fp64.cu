// hyc_fp64.cu -- FP64 kernels of the tracer-advection path and their launchers.
// Compiled with -fmad=false so that every product and sum rounds separately,
// as in the reference's REAL*8 build with no FMA contraction.
#include <climits>
#include <cstdio>
#include <cstring>

#include "hyc_ens.h"
#include "hyc_internal.h"
#include "hyc_fct.cuh"
#include "hyc_tile.cuh"

namespace hyc {

// ---------------------------------------------------------------------------
// fused tile kernels
// ---------------------------------------------------------------------------
template <class K>
static cudaError_t launch_kernel(K kern, size_t smem, const TileArgs &a, int nlayers, cudaStream_t s,
                                 unsigned long long &attr_done) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 64 || !(attr_done >> dev & 1ULL)) {  // one bit per device ordinal < 64
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // ask for the largest shared-memory carveout so that two CTAs fit per SM
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    if (dev < 64) attr_done |= 1ULL << dev;
  }
  dim3 grid((unsigned)(a.ntx * a.nty), (unsigned)nlayers);
  kern<<<grid, 256, smem, s>>>(a);
  return cudaGetLastError();
}

template <int S, int TX, int TY>
static cudaError_t launch_one(const TileArgs &a, int nlayers, cudaStream_t s) {
  static unsigned long long attr_done = 0;
  if constexpr (S == kFCT2 || S == kFCT4) {
    static_assert(FctGeom<TX, TY>::smem_bytes <= 227 * 1024, "tile does not fit in shared memory");
    return launch_kernel(fct_tile_kernel<S, TX, TY>, FctGeom<TX, TY>::smem_bytes, a, nlayers, s, attr_done);
  } else {
    static_assert(TileGeom<TX, TY>::smem_bytes <= 227 * 1024, "tile does not fit in shared memory");
    return launch_kernel(advect_tile_kernel<S, TX, TY>, TileGeom<TX, TY>::smem_bytes, a, nlayers, s, attr_done);
  }
}

template <int TX, int TY>
static cudaError_t launch_shape(int scheme, const TileArgs &a, int nlayers, cudaStream_t s) {
  switch (scheme) {
    case kPCM: return launch_one<kPCM, TX, TY>(a, nlayers, s);
    case kMPDATA: return launch_one<kMPDATA, TX, TY>(a, nlayers, s);
    case kFCT2: return launch_one<kFCT2, TX, TY>(a, nlayers, s);
    case kFCT4: return launch_one<kFCT4, TX, TY>(a, nlayers, s);
  }
  return cudaErrorInvalidValue;
}

bool advect_tile_shape_ok(TileShape t) {
  return (t.tx == 32 && t.ty == 16) || (t.tx == 32 && t.ty == 32) ||
         (t.tx == 16 && t.ty == 16);
}

bool advect_tiles_tma(int scheme, TileShape t) {
  if (!advect_tile_shape_ok(t)) return false;
  if (scheme == kFCT2 || scheme == kFCT4) return true;  // fct_tile_kernel: every shape
  if (t.tx == 32 && t.ty == 16) return TileGeom<32, 16>::TMA;
  if (t.tx == 32 && t.ty == 32) return TileGeom<32, 32>::TMA;
  return TileGeom<16, 16>::TMA;
}

size_t advect_tiles_smem(TileShape t) {
  if (t.tx == 32 && t.ty == 16) return TileGeom<32, 16>::smem_bytes;
  if (t.tx == 32 && t.ty == 32) return TileGeom<32, 32>::smem_bytes;
  if (t.tx == 16 && t.ty == 16) return TileGeom<16, 16>::smem_bytes;
  return 0;
}

cudaError_t launch_advect_tiles(int scheme, const TileArgs &a, int nlayers, TileShape t, cudaStream_t s) {
  if (t.tx == 32 && t.ty == 16) return launch_shape<32, 16>(scheme, a, nlayers, s);
  if (t.tx == 32 && t.ty == 32) return launch_shape<32, 32>(scheme, a, nlayers, s);
  if (t.tx == 16 && t.ty == 16) return launch_shape<16, 16>(scheme, a, nlayers, s);
  return cudaErrorInvalidValue;
}

// persistent FCT kernels for the FP64 ensemble
template <int S, int TX, int TY>
static cudaError_t launch_queue_one(const TileArgs *basins, const int4 *items, int nitems, int *head, int nsm,
                                    cudaStream_t s) {
  constexpr size_t smem = FctGeom<TX, TY>::smem_bytes;
  auto kern = fct_queue_kernel<S, TX, TY>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  kern<<<nsm * per_sm, 256, smem, s>>>(basins, items, nitems, head);
  return cudaGetLastError();
}

cudaError_t launch_fct_queue(int scheme, TileShape t, const TileArgs *basins, const int4 *items, int nitems,
                             int *head, int nsm, cudaStream_t s) {
  if (t.tx == 32 && t.ty == 16) {
    if (scheme == kFCT2) return launch_queue_one<kFCT2, 32, 16>(basins, items, nitems, head, nsm, s);
    if (scheme == kFCT4) return launch_queue_one<kFCT4, 32, 16>(basins, items, nitems, head, nsm, s);
  }
  if (t.tx == 16 && t.ty == 16) {
    if (scheme == kFCT2) return launch_queue_one<kFCT2, 16, 16>(basins, items, nitems, head, nsm, s);
    if (scheme == kFCT4) return launch_queue_one<kFCT4, 16, 16>(basins, items, nitems, head, nsm, s);
  }
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// copy the interior of the output slices back into field level n
// grid: (blocks over interior, nlayers, nfld)
// ---------------------------------------------------------------------------
__global__ void copy_back_kernel(const TileArgs A) {
  const int k = blockIdx.y, fi = blockIdx.z;
  const FieldDesc fd = A.f[fi];
  if (k + 1 > fd.kmax || k + 1 < fd.kmin) return;
  const long long sl = A.slice;
  double *dst = fd.nbase + (long long)(k + fd.k_off) * sl;
  const double *src = A.out + ((long long)fi * A.kdm + k) * sl;
  const long long n = (long long)A.ii * A.jj;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int j = (int)(t / A.ii), i = (int)(t - (long long)j * A.ii);
    long long o = (long long)(i + A.nbdy) + (long long)(j + A.nbdy) * A.ld1;
    if (A.msk[o] & kIP) dst[o] = A.cfac ? src[o] * A.cfac[fi * A.kdm + k] : src[o];  // sea points only
  }
}

// ---------------------------------------------------------------------------
// advem's explicit conservation (mod_tsadvc.F90:168-203, lconserve): for
// every (field, layer) of a tile launch, the contents before and after,
// sum(fld_old*fco*scal) and sum(fld_new*fcn*scal) over interior sea points,
// each summed in xcsum's order (mod_xc_sm.h:900-963: a row in strips of
// 2*nbdy+1 columns, each strip from 0 in column order, the strips in order,
// then the rows in order), then the factor 1 + (old-new)/new that the copy
// back applies.  fco/fcn are formed as the tile kernel forms them (tsadvc
// mode) or taken as given (advem mode).
// rows: [(fi*kdm + k)*2 + (0 old, 1 new)][jj]
// grid: (ceil(jj/8), nlayers, nfld), 8 warps per block, one row per warp
// ---------------------------------------------------------------------------
__global__ void conserve_rows_kernel(const TileArgs A, double *rows) {
  const int k = blockIdx.y, fi = blockIdx.z;
  const FieldDesc fd = A.f[fi];
  if (k + 1 > fd.kmax || k + 1 < fd.kmin) return;
  const int lane = threadIdx.x & 31, jr = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (jr >= A.jj) return;  // whole warps
  const long long sl = A.slice, ld = A.ld1;
  const int nb = A.nbdy, w = 2 * nb + 1, nstrip = (A.ii + w - 1) / w;
  const double *fo = fd.nbase + (long long)(k + fd.k_off) * sl;  // level n before the copy back
  const double *fnw = A.out + ((long long)fi * A.kdm + k) * sl;
  const double *uk = A.mode == 0 ? (A.ufco ? A.ufco : A.uflx + k * sl) : nullptr;
  const double *vk = A.mode == 0 ? (A.vfco ? A.vfco : A.vflx + k * sl) : nullptr;
  const long long row = (long long)(jr + nb) * ld;
  double so = 0.0, sn = 0.0;  // row sums (lane 0)
  for (int r0 = 0; r0 < nstrip; r0 += 32) {
    const int st = r0 + lane;
    double po = 0.0, pn = 0.0;  // strip sums
    if (st < nstrip) {
      const int i1 = st * w, i2 = min(A.ii, i1 + w);
      for (int i = i1; i < i2; i++) {
        const long long c = row + i + nb;
        if (!(A.msk[c] & kIP)) continue;
        double fco, fcn;
        if (A.mode == 0) {
          const double o = (A.oneta_n ? A.oneta_n[c] : 1.0) * A.dpn[k * sl + c];
          const double fdv = ((uk[c + 1] - uk[c]) + (vk[c + ld] - vk[c])) * A.dt2 * A.scali[c];
          fco = kmax(o + fdv, 0.0);
          fcn = kmax(o, 0.0);
        } else {
          fco = A.fco[c];
          fcn = A.fcn[c];
        }
        po = po + fo[c] * fco * A.scal[c];
        pn = pn + fnw[c] * fcn * A.scal[c];
      }
    }
    const int nr = min(32, nstrip - r0);
    for (int l = 0; l < nr; l++) {
      const double a = __shfl_sync(0xffffffffu, po, l), b = __shfl_sync(0xffffffffu, pn, l);
      so = so + a;
      sn = sn + b;
    }
  }
  if (lane == 0) {
    double *rp = rows + ((long long)fi * A.kdm + k) * 2 * A.jj;
    rp[jr] = so;
    rp[A.jj + jr] = sn;
  }
}

// one thread per (field, layer): the rows in order, then 1 + offset (:176-181)
__global__ void conserve_factor_kernel(const TileArgs A, int nlayers, const double *rows, double *fac) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= A.nfld * nlayers) return;
  const int fi = t / nlayers, k = t - fi * nlayers;
  const double *rp = rows + ((long long)fi * A.kdm + k) * 2 * A.jj;
  double sumold = rp[0], sumnew = rp[A.jj];
  for (int j = 1; j < A.jj; j++) {
    sumold = sumold + rp[j];
    sumnew = sumnew + rp[A.jj + j];
  }
  const double offset = sumnew != 0.0 ? (sumold - sumnew) / sumnew : 0.0;
  fac[fi * A.kdm + k] = 1.0 + offset;
}

size_t conserve_rows_elems(int nfld, int kdm, int jj) { return (size_t)nfld * kdm * 2 * jj; }

cudaError_t launch_conserve(const TileArgs &a, int nlayers, double *rows, double *fac, cudaStream_t s) {
  dim3 grid((a.jj + 7) / 8, nlayers, a.nfld);
  conserve_rows_kernel<<<grid, 256, 0, s>>>(a, rows);
  conserve_factor_kernel<<<(a.nfld * nlayers + 127) / 128, 128, 0, s>>>(a, nlayers, rows, fac);
  return cudaGetLastError();
}

cudaError_t launch_copy_back(const TileArgs &a, int nlayers, cudaStream_t s) {
  long long n = (long long)a.ii * a.jj;
  int bx = (int)((n + 255) / 256);
  if (bx > 1216) bx = 1216;
  dim3 grid(bx, nlayers, a.nfld);
  copy_back_kernel<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Isopycnic mixed-layer flux smoothing, mod_tsadvc.F90:1860-1897: at the
// open faces within `margin` of the interior, half the layer-1 flux plus a
// quarter of each along-face neighbour's (the face's own flux where that
// neighbour face is closed); every other face of the two output slices is
// 0, as the reference's uflux/vflux are zeroed on entry (:1812-1813)
// ---------------------------------------------------------------------------
__global__ void iso_smooth_kernel(const double *uk, const double *vk, const uint8_t *msk, long long slice, int ii,
                                  int jj, int nb, int ld1, int margin, double *us, double *vs) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < slice;
       t += (long long)gridDim.x * blockDim.x) {
    const int jr = (int)(t / ld1), ia = (int)(t - (long long)jr * ld1);
    const int i = ia - nb + 1, j = jr - nb + 1;
    double uo = 0.0, vo = 0.0;
    if (i >= 1 - margin && i <= ii + margin && j >= 1 - margin && j <= jj + margin) {
      const uint8_t m = msk[t];
      if (m & kIV) {
        const double vfa = (msk[t - 1] & kIV) ? vk[t - 1] : vk[t];
        const double vfb = (msk[t + 1] & kIV) ? vk[t + 1] : vk[t];
        vo = .5 * vk[t] + .25 * (vfa + vfb);
      }
      if (m & kIU) {
        const double ufa = (msk[t - ld1] & kIU) ? uk[t - ld1] : uk[t];
        const double ufb = (msk[t + ld1] & kIU) ? uk[t + ld1] : uk[t];
        uo = .5 * uk[t] + .25 * (ufa + ufb);
      }
    }
    us[t] = uo;
    vs[t] = vo;
  }
}

cudaError_t launch_iso_smooth(const double *uk, const double *vk, const uint8_t *msk, long long slice, int ii, int jj,
                              int nb, int ld1, int margin, double *us, double *vs, cudaStream_t s) {
  int bx = (int)((slice + 255) / 256);
  if (bx > 2048) bx = 2048;
  iso_smooth_kernel<<<bx, 256, 0, s>>>(uk, vk, msk, slice, ii, jj, nb, ld1, margin, us, vs);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// xctilr, mod_xc_sm.h:1337-1428.  Every halo cell is computed directly from
// interior cells (the reference's N/S pass followed by the E/W pass over
// rows 1-nhl..jj+nhl gives the same values), so one launch has no ordering
// hazard.  grid: (blocks, nlev)
// ---------------------------------------------------------------------------
__global__ void xctilr_kernel(double *a, long long slice, int ii, int jj, int nb, int ld1, int mhl, int nhl,
                              int nreg) {
  double *s = a + (long long)blockIdx.y * slice;
  const bool closed_y = nreg <= 2, closed_x = (nreg == 0 || nreg == 4);
  const long long W = (long long)ii + 2 * mhl;
  const long long nns = 2LL * nhl * W, new_ = 2LL * mhl * jj;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nns + new_;
       t += (long long)gridDim.x * blockDim.x) {
    int i, j;
    if (t < nns) {
      long long band = t / ((long long)nhl * W), r = t - band * nhl * W;
      int jr = (int)(r / W), ic = (int)(r - (long long)jr * W);
      i = 1 - mhl + ic;
      j = band == 0 ? 1 - nhl + jr : jj + 1 + jr;
    } else {
      long long t2 = t - nns;
      long long band = t2 / ((long long)mhl * jj), r = t2 - band * mhl * jj;
      int jr = (int)(r / mhl), c = (int)(r - (long long)jr * mhl);
      j = 1 + jr;
      i = band == 0 ? 1 - mhl + c : ii + 1 + c;
    }
    const bool inI = i >= 1 && i <= ii, inJ = j >= 1 && j <= jj;
    int si = i < 1 ? i + ii : (i > ii ? i - ii : i);
    int sj = j < 1 ? j + jj : (j > jj ? j - jj : j);
    double v;
    if (!inJ) {
      if (inI) v = closed_y ? 0.0 : s[(si + nb - 1) + (long long)(sj + nb - 1) * ld1];
      else v = (closed_x || closed_y) ? 0.0 : s[(si + nb - 1) + (long long)(sj + nb - 1) * ld1];
    } else {
      v = closed_x ? 0.0 : s[(si + nb - 1) + (long long)(j + nb - 1) * ld1];
    }
    s[(i + nb - 1) + (long long)(j + nb - 1) * ld1] = v;
  }
}

cudaError_t launch_xctilr(double *a, long long slice, int nlev, int ii, int jj, int nbdy, int ld1, int mh, int nh,
                          int nreg, cudaStream_t s) {
  if (nreg < 0) return cudaSuccess;  // HYC_NREG_EXTERNAL: the caller exchanges the halos
  int mhl = mh < nbdy ? mh : nbdy;
  if (mhl < 0) mhl = 0;
  int nhl = nh < nbdy ? nh : nbdy;
  if (nhl < 0) nhl = 0;
  if (nlev <= 0 || (mhl == 0 && nhl == 0)) return cudaSuccess;
  long long n = 2LL * nhl * (ii + 2LL * mhl) + 2LL * mhl * jj;
  int bx = (int)((n + 255) / 256);
  if (bx > 512) bx = 512;
  for (int l0 = 0; l0 < nlev; l0 += 65535) {
    int nl = nlev - l0 < 65535 ? nlev - l0 : 65535;
    xctilr_kernel<<<dim3(bx, nl), 256, 0, s>>>(a + (long long)l0 * slice, slice, ii, jj, nbdy, ld1, mhl, nhl, nreg);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// salinity range diagnostic
// ---------------------------------------------------------------------------
long long double_to_key(double x) {
  long long b;
  memcpy(&b, &x, 8);
  return b ^ (long long)((unsigned long long)(b >> 63) >> 1);
}
double key_to_double(long long k) {
  long long b = k ^ (long long)((unsigned long long)(k >> 63) >> 1);
  double x;
  memcpy(&x, &b, 8);
  return x;
}

__global__ void saln_range_kernel(const double *saln_n, const double *dp_n, const uint8_t *msk, long long slice,
                                  int ii, int jj, int nb, int ld1, long long *keys, int kdm) {
  const int k = blockIdx.y;
  // onemm = onem*0.001 with onem = g/svref = 9.806/(1/1000) folded in double
  // (9805.999999999998 Pa), mod_cb_arrays.F90:843-851
  const double onemm = (9.806 / (1.0 / 1000.0)) * 0.001;
  const double *s = saln_n + (long long)k * slice, *d = dp_n + (long long)k * slice;
  long long kmn = LLONG_MAX, kmx = LLONG_MIN;
  const long long n = (long long)ii * jj;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int j = (int)(t / ii), i = (int)(t - (long long)j * ii);
    long long o = (long long)(i + nb) + (long long)(j + nb) * ld1;
    if ((msk[o] & kIP) && d[o] > onemm) {
      long long kk = dkey(s[o]);
      kmn = kk < kmn ? kk : kmn;
      kmx = kk > kmx ? kk : kmx;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    long long a = __shfl_down_sync(0xffffffffu, kmn, off), b = __shfl_down_sync(0xffffffffu, kmx, off);
    kmn = a < kmn ? a : kmn;
    kmx = b > kmx ? b : kmx;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(reinterpret_cast<long long *>(&keys[k]), kmn);
    atomicMax(reinterpret_cast<long long *>(&keys[kdm + k]), kmx);
  }
}

cudaError_t launch_saln_range(const double *saln_n, const double *dp_n, const uint8_t *msk, long long slice, int kdm,
                              int ii, int jj, int nbdy, int ld1, long long *keys, cudaStream_t s) {
  long long n = (long long)ii * jj;
  int bx = (int)((n + 255) / 256);
  if (bx > 304) bx = 304;
  saln_range_kernel<<<dim3(bx, kdm), 256, 0, s>>>(saln_n, dp_n, msk, slice, ii, jj, nbdy, ld1, keys, kdm);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// compensated FP64 content sum.  A fixed grid (kSumBlocks x 256) walks the
// interior in a fixed order; each thread keeps a (sum, error) pair with
// two-sum, the CTA combines pairs in a fixed tree, and one CTA combines the
// CTA results in block order.  Same inputs give the same bits every run.
// ---------------------------------------------------------------------------
constexpr int kSumBlocks = 608;
int mass_sum_partials() { return kSumBlocks; }

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
  s = __dadd_rn(a, b);
  double bb = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
}
__device__ __forceinline__ void acc(double &hi, double &lo, double x) {
  double s, e;
  two_sum(hi, x, s, e);
  hi = s;
  lo = __dadd_rn(lo, e);
}

__global__ void mass_sum_kernel(const double *fld, const double *fc, const double *scal, const uint8_t *msk, int ii,
                                int jj, int nb, int ld1, double *partial) {
  double hi = 0.0, lo = 0.0;
  const long long n = (long long)ii * jj;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    int j = (int)(t / ii), i = (int)(t - (long long)j * ii);
    long long o = (long long)(i + nb) + (long long)(j + nb) * ld1;
    if (msk[o] & kIP) acc(hi, lo, __dmul_rn(__dmul_rn(fld[o], __dadd_rn(fc[o], kOnemu)), scal[o]));
  }
  __shared__ double sh[256], sl[256];
  sh[threadIdx.x] = hi;
  sl[threadIdx.x] = lo;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double s, e;
      two_sum(sh[threadIdx.x], sh[threadIdx.x + w], s, e);
      sh[threadIdx.x] = s;
      sl[threadIdx.x] = __dadd_rn(__dadd_rn(sl[threadIdx.x], sl[threadIdx.x + w]), e);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = sh[0];
    partial[2 * blockIdx.x + 1] = sl[0];
  }
}

__global__ void mass_sum_final(const double *partial, int nblk, double *res) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double hi = 0.0, lo = 0.0;
  for (int b = 0; b < nblk; b++) {
    acc(hi, lo, partial[2 * b]);
    lo = __dadd_rn(lo, partial[2 * b + 1]);
  }
  res[0] = __dadd_rn(hi, lo);
}

cudaError_t launch_mass_sum(const double *fld, const double *fc, const double *scal, const uint8_t *msk, int ii,
                            int jj, int nbdy, int ld1, double *partial, double *dres, cudaStream_t s) {
  mass_sum_kernel<<<kSumBlocks, 256, 0, s>>>(fld, fc, scal, msk, ii, jj, nbdy, ld1, partial);
  mass_sum_final<<<1, 32, 0, s>>>(partial, kSumBlocks, dres);
  return cudaGetLastError();
}

}  // namespace hyc
