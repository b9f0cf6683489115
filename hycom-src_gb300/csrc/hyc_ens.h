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
  int kdm, ntr;  // ntr: tracers this table's launch advances, from q0 on
  int images;  // periodic-x halo images to write (0 when closed)
  int seg;     // rows per strip segment
  int kchunk;  // layers per work item
  int q0;      // first tracer of this table's launch
  float *fnew;  // ntr*kdm slices, level t+1
  float posdef[kMaxFields];  // MPDATA offset of each tracer (mod_tsadvc.F90:1755-1763)
  // TMA maps (box 64 x 4 rows, device memory): levels t-1 and t (3-D, ld1 x
  // ld2 x ntr*kdm, FP32), uflx, vflx (FP32), dp (FP64), the per-cell
  // words (one slice, FP64) and, with the diffusion epilogue, the grid
  // table of diffusion face factors (one slice of FP32 pairs: row r holds
  // temdf2*aspux*scuy of row r-4 and temdf2*aspvy*scvx of row r-3)
  const CUtensorMap *c2_old, *c2_cur, *c2_u, *c2_v, *c2_dp, *c2_cg, *c2_gd;
};

// two columns per lane, 64-column strips (56 updated) streamed by TMA
constexpr int kCol2Strip = 56;
constexpr int kCol2Box = 64, kCol2Rows = 4;
cudaError_t launch_mix_col2(int scheme, const MixBasin *basins, const int4 *items, int nitems, int *head, int nsm,
                            int nq, bool prep64, bool diff, int *err, cudaStream_t s);
// grid table of the diffusion epilogue (see MixBasin::c2_gd) from reference-layout FP64
// arrays (pitch ld1r); out has the ensemble pitch ld1
cudaError_t launch_diff_table(const double *aspux, const double *aspvy, const double *scuy, const double *scvx,
                              const uint8_t *msk, double temdf2, int ld1r, int ld1, int ld2, float2 *out,
                              cudaStream_t s);
// per-cell words: dt2*scp2i with the ip, iu, iv bits of msk in the three lowest mantissa bits
cudaError_t launch_cell_words(const double *scp2i, const uint8_t *msk, double dt2, long long n, double *out,
                              cudaStream_t s);
cudaError_t launch_wait_probe(int arrive, int *err, cudaStream_t s);

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
