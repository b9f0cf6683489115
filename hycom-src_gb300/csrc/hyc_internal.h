// hyc_internal.h -- launchers shared between the CUDA translation units and
// the host layer (hyc_host.cpp).  Not part of the public C ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace hyc {

struct FieldDesc;
struct TileArgs;

// Geometry of a tile launch (chosen by the host, see hyc_host.cpp).
struct TileShape {
  int tx, ty;
};

// Fused advem/tsadvc tile kernel; scheme in {0,1,2,4}.  out receives every
// interior cell of each (field, layer) slice it processes.
cudaError_t launch_advect_tiles(int scheme, const TileArgs &a, int nlayers, TileShape shape,
                                cudaStream_t s);
size_t advect_tiles_smem(TileShape shape);
// the tile kernel of this scheme and shape stages its region by TMA when
// the launch carries tensor maps (box (tx+8) x (ty+6), see TileArgs::tmaps)
bool advect_tiles_tma(int scheme, TileShape shape);
bool advect_tile_shape_ok(TileShape shape);

// Copy the interior of out[(fi*kdm+k)] back into field level n for every
// (field, layer) the launch processed (times a.cfac[fi*kdm+k] when set).
cudaError_t launch_copy_back(const TileArgs &a, int nlayers, cudaStream_t s);

// advem's conservation rescale (lconserve): the factors a.cfac for the
// pairs of a tile launch, from the old level n and the new values in
// a.out; rows holds conserve_rows_elems(nfld, kdm, jj) doubles
size_t conserve_rows_elems(int nfld, int kdm, int jj);
cudaError_t launch_conserve(const TileArgs &a, int nlayers, double *rows, double *fac, cudaStream_t s);

struct Fct2cArgs;
// advem_fct2c: work bytes per (field, layer) pair; the stages of one call
size_t fct2c_work_bytes(long long slice);
cudaError_t launch_fct2c(const Fct2cArgs &a, int nreg, int *launches, cudaStream_t s);

// Lateral diffusion (tsdff_1x/tsdff_2x and the density update); the two
// launches of one call
struct TsdffArgs;
cudaError_t launch_tsdff(const TsdffArgs &a, cudaStream_t s);

// Robert-Asselin filter: asselin_save (filter false) or asselin_filter
struct AsselinArgs;
cudaError_t launch_asselin(const AsselinArgs &a, bool filter, cudaStream_t s);

// Continuity equation: work slices, loop 76 (all layers), then the rest
struct CnuityArgs;
size_t cnuity_work_slices();
cudaError_t launch_cnuity_layers(const CnuityArgs &a, int *launches, cudaStream_t s);
cudaError_t launch_cnuity_rest(const CnuityArgs &a, int *launches, cudaStream_t s);

// Isopycnic smoothing of the layer-1 fluxes (mod_tsadvc.F90:1860-1897) into
// us/vs (whole slices, 0 off the smoothed faces).
cudaError_t launch_iso_smooth(const double *uk, const double *vk, const uint8_t *msk, long long slice, int ii, int jj,
                              int nb, int ld1, int margin, double *us, double *vs, cudaStream_t s);

// xctilr on nlev slices (mod_xc_sm.h:1337-1428).
cudaError_t launch_xctilr(double *a, long long slice, int nlev, int ii, int jj, int nbdy, int ld1, int mh,
                          int nh, int nreg, cudaStream_t s);

// Salinity range diagnostic (mod_tsadvc.F90:2065-2084): per layer min/max of
// saln(:,:,k,n) over interior sea cells with dp(:,:,k,n) > onemm.  keys is
// a device array of 2*kdm int64 (min keys then max keys).
cudaError_t launch_saln_range(const double *saln_n, const double *dp_n, const uint8_t *msk, long long slice,
                              int kdm, int ii, int jj, int nbdy, int ld1, long long *keys, cudaStream_t s);
double key_to_double(long long k);
long long double_to_key(double d);

// sum over interior sea cells of fld*(fc+onemu)*scal, two-sum compensated,
// fixed order.  partial: device scratch of at least mass_sum_partials()
// doubles*2; result written to *dres (device).
int mass_sum_partials();
cudaError_t launch_mass_sum(const double *fld, const double *fc, const double *scal, const uint8_t *msk,
                            int ii, int jj, int nbdy, int ld1, double *partial, double *dres, cudaStream_t s);

// Record a message for hyc_last_error(NULL, ...).
void set_library_error(const char *msg);

}  // namespace hyc
