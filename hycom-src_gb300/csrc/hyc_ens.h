// hyc_ens.h -- device-visible descriptors and launchers of the ensemble
// (batched) form.  Not part of the public C ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "hyc_args.h"
#include "hyc_internal.h"

namespace hyc {

// One basin of an FP32-mixed ensemble for one leapfrog rotation.  Slices
// use the ensemble pitch ld1 (>= idm+2*nbdy, a multiple of 4).
struct MixBasin {
  int ii, jj, nbdy, ld1, ld2;
  long long slice;
  int ntx, nty, kdm, ntr;
  int images;  // periodic-x halo images to write (0 when closed)
  int pad;
  double dt2;
  const uint8_t *msk;
  const double *scp2, *scp2i;
  const float *uflx, *vflx;   // kdm slices
  const double *dp;           // kdm slices, dp(:,:,k,n)
  const float *fold, *fcur;   // ntr*kdm slices, levels t-1 and t
  float *fnew;                // ntr*kdm slices, level t+1
  // TMA descriptors (device memory) for the current tile shape: levels t-1
  // and t (3-D: ld1 x ld2 x ntr*kdm, FP32), uflx, vflx (FP32) and dp (FP64)
  const CUtensorMap *tm_old, *tm_cur, *tm_u, *tm_v, *tm_dp;
  // column kernel: (dt2*scp2i, scp2/dt2) per cell, rows per segment
  const float2 *dsqs;
  int seg;
  int kchunk;  // two-column strip kernel: layers per work item
  float posdef[kMaxFields];  // MPDATA offset of each tracer (mod_tsadvc.F90:1755-1763)
  // two-column strip kernel: TMA maps (box 64 x 4 rows) of the old and
  // centre levels, uflx, vflx, dp, the per-cell factors (float4 as 4*ld1
  // floats per row) and dt2*scp2i (FP64)
  const CUtensorMap *c2_old, *c2_cur, *c2_u, *c2_v, *c2_dp, *c2_ge, *c2_si, *c2_dp32;
};

bool mix_shape_ok(TileShape t);
cudaError_t launch_mix_fct2(TileShape t, const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm,
                            bool prep64, cudaStream_t s);

bool mix_tma_shape_ok(TileShape t);
cudaError_t launch_mix_fct2_tma(TileShape t, const MixBasin *basins, const int4 *items, int nitems, int *head,
                                int nsm, bool prep64, int *err, cudaStream_t s);
// one warp per 32-column strip (26 updated), segments of `seg` rows
constexpr int kColStrip = 26;
cudaError_t launch_mix_fct2_col(const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm, int nq,
                                bool prep64, int seg, cudaStream_t s);
// two columns per lane, 64-column strips (56 updated) streamed by TMA
constexpr int kCol2Strip = 56;
constexpr int kCol2Box = 64, kCol2Rows = 4;
cudaError_t launch_mix_col2(int scheme, const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm,
                            int nq, bool prep64, int *err, cudaStream_t s);
cudaError_t launch_geo4(const double *scp2, const double *scp2i, const uint8_t *msk, double dt2, long long n,
                        float4 *out, cudaStream_t s);
cudaError_t launch_wait_probe(int arrive, int *err, cudaStream_t s);
cudaError_t launch_dtsi(const double *scp2i, double dt2, long long n, double *out, cudaStream_t s);
cudaError_t launch_dsqs(const double *scp2, const double *scp2i, double dt2, long long n, float2 *out,
                        cudaStream_t s);

// TMA box width (elements) of a tile shape: TX + 12 for the nbdy = 6 halo
inline int tma_box_x(TileShape t) { return (t.tx + 9 + 3) / 4 * 4; }
inline int tma_box_y(TileShape t) { return t.ty + 6; }

// FP64 ensemble: the FCT tile body over a queue of (basin, tile, layer)
cudaError_t launch_fct_queue(int scheme, TileShape t, const TileArgs *basins, const int4 *items, int nitems,
                             int *head, int nsm, cudaStream_t s);

cudaError_t launch_repitch(const void *src, int src_fp32, long long spitch, long long sslice, void *dst, int dst_fp32,
                           long long dpitch, long long dslice, int w, int h, int nslices, cudaStream_t s);

cudaError_t launch_content(const void *fld, int fld_fp32, const void *uflx, const void *vflx, int flx_fp32,
                           const double *dp, const double *scp2, const double *scp2i, const uint8_t *msk, int ii,
                           int jj, int nb, int ld1, long long slice, int kdm, int use_fco, double dt2,
                           double *partial, cudaStream_t s);

}  // namespace hyc
