/*
 * hycom_adv.h -- C ABI of the GB300 tracer-advection library (libhycadv.so).
 *
 * Drop-in for HYCOM's layered tracer advection, module mod_tsadvc:
 *   tsadvc(m,n)                         mod_tsadvc.F90:1708  (public entry)
 *   advem(advtyp,fld,fldc,u,v,fco,fcn,  mod_tsadvc.F90:69-79 (module-private
 *         posdef,scal,scali,dt2,btrmas)                      scheme driver)
 *   xctilr(a,l1,ld,mh,nh,itype)         mod_xc_sm.h:1337      (halo fill)
 *   bigrid / indxi / indxj              bigrid.F90:1,417,475  (masks)
 *
 * Every array uses the reference's memory layout: a 2-D slice is the
 * Fortran array a(1-nbdy:idm+nbdy, 1-nbdy:jdm+nbdy) stored column-major
 * (i fastest), ld1 = idm+2*nbdy, ld2 = jdm+2*nbdy, and the pointer passed
 * points at element (1-nbdy,1-nbdy).  3-D/4-D fields are slices stacked as
 * in mod_cb_arrays.F90 (e.g. temp(:,:,k,t) at slice index (k-1)+(t-1)*kdm).
 * Time levels m, n are the reference's 1-based indices.
 *
 * All functions return HYC_OK (0) or a negative HYC_ERR_* code; the text of
 * the last error of a context is available from hyc_last_error().  Where
 * the reference would stop the model (xcstop for a bad advtyp,
 * mod_tsadvc.F90:160-165, or nbdy < mbdy, :1817-1825) the library returns
 * an error instead.  No CPU fallback exists: without a usable GPU every
 * compute call fails with HYC_ERR_CUDA.
 */
#ifndef HYCOM_ADV_H
#define HYCOM_ADV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HYC_OK 0
#define HYC_ERR_ARG -1         /* bad argument (null pointer, size, level) */
#define HYC_ERR_ADVTYP -2      /* advtyp not in {0,1,2,4}, mod_tsadvc.F90:149-166 */
#define HYC_ERR_NBDY -3        /* nbdy < mbdy_advtyp(advtyp), mod_tsadvc.F90:1817 */
#define HYC_ERR_MASK -4        /* iu/iv inconsistent with ip (bigrid.F90:216-252) */
#define HYC_ERR_CUDA -5        /* CUDA runtime error or no device */
#define HYC_ERR_FIELD -6       /* a field tsadvc needs is not bound */
#define HYC_ERR_GRID -7        /* bigrid: 1-point sea, arctic row, ms overflow */
#define HYC_ERR_UNSUPPORTED -8 /* option outside this library's scope */
#define HYC_ERR_NOMEM -9       /* device allocation failed */
#define HYC_ERR_NEGDP -10      /* cnuity: a layer thinner than dpfatal, cnuity.F90:574-580 */

/* nreg of a context that is one block of a basin split over ranks: its
   halos are filled by the caller's exchange with the neighbouring blocks
   (hycadv.decomp), and xctilr leaves them alone */
#define HYC_NREG_EXTERNAL -1

/* where a pointer lives */
#define HYC_HOST 0
#define HYC_DEVICE 1

/* field identifiers for hyc_bind_field (mod_cb_arrays.F90 names) */
#define HYC_F_TEMP 0   /* temp(ld1,ld2,kdm,2)              */
#define HYC_F_SALN 1   /* saln(ld1,ld2,kdm,2)              */
#define HYC_F_TH3D 2   /* th3d(ld1,ld2,kdm,2)              */
#define HYC_F_TRACER 3 /* tracer(ld1,ld2,kdm,2,ntracr)     */
#define HYC_F_UFLX 4   /* uflx(ld1,ld2,kdm)                */
#define HYC_F_VFLX 5   /* vflx(ld1,ld2,kdm)                */
#define HYC_F_DP 6     /* dp(ld1,ld2,kdm,2)                */
#define HYC_F_ONETA 7  /* oneta(ld1,ld2,2), read if btrmas */
#define HYC_F_Q2 8     /* q2(ld1,ld2,0:kdm+1,2), if mxlmy  */
#define HYC_F_Q2L 9    /* q2l(ld1,ld2,0:kdm+1,2), if mxlmy */
/* Robert-Asselin filter state (mod_cb_arrays.F90), hyc_asselin_* only */
#define HYC_F_DPO 10     /* dpo(ld1,ld2,kdm,2)                */
#define HYC_F_ONETAO 11  /* onetao(ld1,ld2,2)                 */
#define HYC_F_PBAVG 12   /* pbavg(ld1,ld2,3)                  */
#define HYC_F_PBOT 13    /* pbot(ld1,ld2)                     */
#define HYC_F_OTEMP 14   /* otemp(ld1,ld2,kdm)                */
#define HYC_F_OSALN 15   /* osaln(ld1,ld2,kdm)                */
#define HYC_F_OTH3D 16   /* oth3d(ld1,ld2,kdm)                */
#define HYC_F_OTRACER 17 /* otracer(ld1,ld2,kdm,ntracr)       */
#define HYC_F_OQ2 18     /* oq2(ld1,ld2,0:kdm+1), if mxlmy    */
#define HYC_F_OQ2L 19    /* oq2l(ld1,ld2,0:kdm+1), if mxlmy   */
/* continuity equation (mod_cb_arrays.F90), hyc_cnuity only */
#define HYC_F_U 20        /* u(ld1,ld2,kdm,2)                  */
#define HYC_F_V 21        /* v(ld1,ld2,kdm,2)                  */
#define HYC_F_DPU 22      /* dpu(ld1,ld2,kdm,2)                */
#define HYC_F_DPV 23      /* dpv(ld1,ld2,kdm,2)                */
#define HYC_F_UBAVG 24    /* ubavg(ld1,ld2,3)                  */
#define HYC_F_VBAVG 25    /* vbavg(ld1,ld2,3)                  */
#define HYC_F_P 26        /* p(ld1,ld2,kdm+1)                  */
#define HYC_F_UFLXAV 27   /* uflxav(ld1,ld2,kdm), optional     */
#define HYC_F_VFLXAV 28   /* vflxav(ld1,ld2,kdm), optional     */
#define HYC_F_DPAV 29     /* dpav(ld1,ld2,kdm), optional       */
#define HYC_F_ONETACNT 30 /* onetacnt(ld1,ld2), if btrmas      */
#define HYC_NFIELDS 31

typedef struct hyc_ctx hyc_ctx;

/* Run-time switches of tsadvc (blkdat.F90:865-911, :1260-1300, :1485). */
typedef struct hyc_tsadvc_params {
  int32_t advtyp;  /* 0 PCM, 1 MPDATA, 2 FCT2, 4 FCT4                  */
  int32_t advflg;  /* 0 advect temp and saln, 1 advect th3d and saln    */
  int32_t btrmas;  /* barotropic mass flag (FCT2 becomes fct2c)        */
  int32_t ntracr;  /* number of tracers in the bound tracer array       */
  int32_t nhybrd;  /* number of hybrid layers                           */
  int32_t isopyc;  /* isopycnic mode (nhybrd==0): layer-1 flux smoothing,
                      mod_tsadvc.F90:1860-1897 (not with btrmas)        */
  int32_t hybrid;  /* nhybrd > 0                                        */
  int32_t mxlmy;   /* Mellor-Yamada mixed layer: also advect q2, q2l   */
  int32_t nstep;   /* model step; the salinity range diagnostic runs when
                      mod(nstep,3)==0 or diagno (mod_tsadvc.F90:2065)   */
  int32_t diagno;
  double delt1;    /* leapfrog time step (2*baclin), passed as dt2      */
  const int32_t *trcflg; /* host array of ntracr flags; 2 = temperature-like */
} hyc_tsadvc_params;

/*
 * Build the land/sea masks from depth, as bigrid does for a single tile
 * (bigrid.F90:1-415; no arctic fold, no f-plane).  depth (ld1*ld2, metres,
 * >0 is sea) is modified in place exactly like bigrid (halo filled, land
 * borders).  Outputs (each ld1*ld2 int32, any may be NULL except ip/iu/iv):
 * ip, iu, iv, iq and the sea-only neighbour indices ipim1/ipip1/ipjm1/ipjp1
 * (Fortran index values).  *nreg receives 0 (closed) or 1 (periodic in x).
 * Replaces: bigrid.F90:1 (subroutine bigrid) plus geopar.F90:256 call site.
 */
int hyc_bigrid(int32_t idm, int32_t jdm, int32_t nbdy, double *depth, int32_t *ip, int32_t *iu,
               int32_t *iv, int32_t *iq, int32_t *ipim1, int32_t *ipip1, int32_t *ipjm1, int32_t *ipjp1,
               int32_t *nreg);

/*
 * Create a context bound to one GPU: grid sizes, nreg (mod_xc: 0 closed,
 * 1 periodic-x/closed-y, 3 periodic in both; HYC_NREG_EXTERNAL for one
 * block of a decomposed basin, whose halos the caller exchanges before
 * hyc_tsadvc / hyc_tsdff / hyc_cnuity; the routines that refresh halos in
 * mid-step, advem_fct2c (btrmas) and cnuity's interface diffusion, return
 * HYC_ERR_UNSUPPORTED there), masks ip/iu/iv and the grid
 * metrics scp2/scp2i (all host arrays of ld1*ld2).  The masks and metrics
 * are copied to the device and stay resident.  Replaces the module state
 * that tsadvc reads through `use mod_dimensions, mod_cb_arrays`
 * (mod_tsadvc.F90:15, :1709).
 */
int hyc_adv_init(hyc_ctx **ctx, int32_t idm, int32_t jdm, int32_t kdm, int32_t nbdy, int32_t nreg,
                 const int32_t *ip, const int32_t *iu, const int32_t *iv, const double *scp2,
                 const double *scp2i, int32_t device);

/* Release everything the context owns. */
int hyc_adv_finalize(hyc_ctx *ctx);

/* Copy the last error message of ctx (or of the library when ctx is NULL). */
int hyc_last_error(const hyc_ctx *ctx, char *buf, size_t n);

/*
 * Use this CUDA stream (a cudaStream_t passed as void*; NULL = the legacy
 * default stream) for later calls.  Until then a context queues its work
 * on a non-blocking stream of its own.  Device memory the caller passes in
 * is read and written in order on that stream: a caller that fills or
 * reads such memory on another stream orders the two itself (an event, a
 * synchronize, or by setting its own stream here).
 */
int hyc_set_stream(hyc_ctx *ctx, void *stream);

/*
 * Bind a model field (HYC_F_*) of nelem doubles.  where = HYC_DEVICE: ptr
 * is device memory owned by the caller and is used in place.  where =
 * HYC_HOST: ptr is the caller's host array; the library allocates a
 * resident device mirror, and hyc_sync_field moves data between them.
 */
int hyc_bind_field(hyc_ctx *ctx, int32_t field, void *ptr, int64_t nelem, int32_t where);

/* Copy a host-bound field: to_device=1 host->device mirror, 0 back. */
int hyc_sync_field(hyc_ctx *ctx, int32_t field, int32_t to_device);

/* Wait for all work queued on the context's stream. */
int hyc_synchronize(hyc_ctx *ctx);

/*
 * tsadvc(m,n), advection part (mod_tsadvc.F90:1708-2132 with temdf2=0):
 * halo fill of the advected fields (as :1829-1840), thickness prep
 * (:1905-1942), advem on every active field of every layer, and the
 * salinity range diagnostic.  Works on the bound (device-resident) fields;
 * xmin/xmax (host, kdm each, may be NULL) receive the per-layer salinity
 * minimum/maximum when the diagnostic runs (mod_tsadvc.F90:2065-2084).
 * Asynchronous on the context stream unless xmin/xmax are requested.
 * Replaces: mod_tsadvc.F90:1708 (subroutine tsadvc), call site
 * mod_hycom.F90:2536.
 */
int hyc_tsadvc(hyc_ctx *ctx, int32_t m, int32_t n, const hyc_tsadvc_params *p, double *xmin,
               double *xmax);

/*
 * advem on one 2-D slice (mod_tsadvc.F90:69-79, same argument meaning):
 * fld (in/out, old level in, new level out on sea points of the interior),
 * fldc (center level), u, v (mass fluxes), fco, fcn (old/new thickness),
 * posdef, scal, scali (metrics), dt2, btrmas.  All pointers are host
 * (where = HYC_HOST) or device (where = HYC_DEVICE) arrays of ld1*ld2
 * doubles.  The grid and masks are those of ctx.  advtyp 2 with btrmas
 * runs advem_fct2c (mod_tsadvc.F90:999-1368), as hyc_tsadvc does then for
 * every field.  Synchronous.
 * Replaces: mod_tsadvc.F90:69 (subroutine advem).
 */
int hyc_advem(hyc_ctx *ctx, int32_t advtyp, double *fld, const double *fldc, const double *u,
              const double *v, const double *fco, const double *fcn, double posdef, const double *scal,
              const double *scali, double dt2, int32_t btrmas, int32_t where);

/*
 * xctilr on nlev consecutive slices of a (mod_xc_sm.h:1337-1428): fill the
 * halo mh wide in i and nh wide in j with vland=0 (closed) or a periodic
 * copy, according to the context's nreg.  where = HYC_HOST or HYC_DEVICE.
 * Replaces: mod_xc_sm.h:1337 (subroutine xctilr), single-tile form.
 */
int hyc_xctilr(hyc_ctx *ctx, double *a, int32_t nlev, int32_t mh, int32_t nh, int32_t where);

/*
 * Grid arrays of the lateral diffusion: aspux, aspvy (aspect ratios at u
 * and v points) and scuy, scvx (grid spacings), mod_cb_arrays.F90 names,
 * host arrays of ld1*ld2 with valid halos.  Copied to the device and kept.
 * Replaces the module state tsdff reads (mod_tsadvc.F90:2275-2285).
 */
int hyc_set_diffusion_grid(hyc_ctx *ctx, const double *aspux, const double *aspvy, const double *scuy,
                           const double *scvx);

/*
 * The diffusion block at the end of tsadvc(m,n) (mod_tsadvc.F90:2138-2230),
 * to be called right after hyc_tsadvc(m,n) with the same p when temdf2 > 0
 * (temdf2 <= 0 returns at once, as the reference skips the block):
 * halo fill of level n (width 2), Laplacian diffusion of temp and saln (and
 * of every tracer, and of q2/q2l when p->mxlmy) in every layer with the
 * face factors temdf2*aspux*scuy*harmonc(dp*oneta) (tsdff_1x/tsdff_2x),
 * then th3d = sig(temp,saln) - thbase at the sea points (17-term equation
 * of state, sigma-2).  Needs oneta bound (onetamas(:,:,n) = oneta(:,:,n)
 * for diffusion, :1805) and hyc_set_diffusion_grid.  Supported: temdfc = 1
 * (what blkdat.F90:1135 requires with the 17-term equation of state) and
 * nhybrd >= kdm (no exactly isopycnal layers, which need theta); else
 * HYC_ERR_UNSUPPORTED.  FP64, bit-identical to the oracle.  Asynchronous.
 * Replaces: mod_tsadvc.F90:2138-2230 with its tsdff_1x/tsdff_2x.
 */
int hyc_tsdff(hyc_ctx *ctx, int32_t m, int32_t n, const hyc_tsadvc_params *p, double temdf2, double temdfc,
              double thbase);

/*
 * asselin_save(m,n) (mod_asselin.F90:28-82), called at the start of a
 * step (mod_hycom.F90:2517): oneta and onetao of both levels from
 * pbavg/pbot at sea points (max with oneta0), level n of temp, saln, th3d,
 * every tracer (and q2/q2l when p->mxlmy) into otemp, osaln, oth3d,
 * otracer (oq2, oq2l) at every interior point, then the halo of oneta and
 * onetao (width 6).  Uses p->ntracr and p->mxlmy.  Asynchronous.
 * Replaces: mod_asselin.F90:28 (subroutine asselin_save).
 */
int hyc_asselin_save(hyc_ctx *ctx, int32_t m, int32_t n, const hyc_tsadvc_params *p, double oneta0);

/*
 * asselin_filter(m,n) (mod_asselin.F90:84-268), called at the end of a
 * step (mod_hycom.F90:2645): oneta of both levels from pbavg/pbot, then at
 * every sea point and layer the Robert-Asselin filter (weight ra2fac) of
 * the thickness dp(m) and of oneta*dp*scalar for saln, temp, every tracer
 * (the form that keeps a constant field constant) and q2/q2l, and
 * th3d(m) = sig(temp(m),saln(m)) - thbase (17-term equation of state).
 * Supported: advflg = 0 and nhybrd >= kdm (the 17-term equation of state
 * has no tofsig for th3d-advecting or exactly isopycnal layers); else
 * HYC_ERR_UNSUPPORTED.  FP64, bit-identical to the oracle.  Asynchronous.
 * Replaces: mod_asselin.F90:84 (subroutine asselin_filter).
 */
int hyc_asselin_filter(hyc_ctx *ctx, int32_t m, int32_t n, const hyc_tsadvc_params *p, double ra2fac,
                       double oneta0, double thbase);

/* Run-time switches of cnuity (blkdat.F90 names). */
typedef struct hyc_cnuity_params {
  int32_t nstep;   /* model step: the fatal negative-thickness check runs when
                      mod(nstep,3)==0 (cnuity.F90:520); the biharmonic
                      diffusion alternates its direction with mod(nstep,2) */
  int32_t btrmas;  /* barotropic mass flag                                  */
  int32_t thkdf;   /* interface-depth diffusion: 0 none, 4 biharmonic
                      (thkdf4 != 0), 2 Laplacian (thkdf2 != 0)              */
  int32_t isopyc;  /* isopycnic mode: unsupported, must be 0               */
  double delt1;    /* leapfrog time step                                    */
  double ra2fac;   /* Robert-Asselin weight                                 */
} hyc_cnuity_params;

/*
 * Grid arrays of cnuity (mod_cb_arrays.F90 names, host arrays of ld1*ld2
 * with valid halos): scuy, scvx, depthu, depthv (u/v-point depths in
 * pressure units) and thkdfu, thkdfv (the reference's thkdf4u/thkdf4v:
 * the interface-diffusion coefficients, biharmonic or Laplacian; NULL when
 * no interface diffusion runs).  Copied to the device and kept.
 */
int hyc_set_cnuity_grid(hyc_ctx *ctx, const double *scuy, const double *scvx, const double *depthu,
                        const double *depthv, const double *thkdfu, const double *thkdfv);

/*
 * cnuity(m,n) (cnuity.F90:14-1419), the continuity equation on the bound
 * fields: halo fill of dp, dpu, dpv, u, v, ubavg, vbavg (width 6); per
 * layer the flux-corrected transport of dp(:,:,k,n) with low-order
 * fluxes, the Zalesak limiter and the clipped antidiffusive fluxes
 * (loop 76), the mass fluxes into uflx/vflx and the interface pressures p;
 * without btrmas the barotropic restoration (loop 77) and the
 * bottom-pressure restoring; the interface-depth diffusion p->thkdf; the
 * cumulative uflxav/vflxav/dpav when all three are bound; with btrmas the
 * restoring to dp' (onetacnt); then the Robert-Asselin filter of dp(m) and
 * dpo.  Needs nbdy >= 6, hyc_set_cnuity_grid, and fields dp, dpo, u, v,
 * dpu, dpv, ubavg, vbavg, pbot, p, uflx, vflx (oneta and onetacnt with
 * btrmas).  dpkmin (host, 2*kdm, may be NULL) receives the minimum
 * thickness of each layer after the low-order and after the antidiffusive
 * update.  A layer thinner than dpfatal = -10 m (checked when
 * mod(nstep,3)==0) stops the reference; here it returns HYC_ERR_NEGDP
 * before the rest of the step.  Not supported: open boundaries (the
 * masks have none), STOKES drift, isopyc, the Kraus-Turner mixed-layer
 * base (mxlkta), floats.  FP64, bit-identical to the oracle.
 * Replaces: cnuity.F90:14 (subroutine cnuity), call site mod_hycom.F90:2520.
 */
int hyc_cnuity(hyc_ctx *ctx, int32_t m, int32_t n, const hyc_cnuity_params *p, double *dpkmin);

/*
 * Tracer content sum over sea points of the interior,
 *   sum_{i,j} fld(i,j) * (fc(i,j) + onemu) * scp2(i,j),
 * accumulated on the device in FP64 with compensated (two-sum) partials
 * and a fixed reduction order, so the result is reproducible run to run.
 * This is the quantity FCT/PCM conserve (mod_tsadvc.F90:788, :976).
 * fld, fc: device arrays of one slice.  Result in *sum.  Synchronous.
 */
int hyc_mass_sum(hyc_ctx *ctx, const double *fld, const double *fc, double *sum);

/*
 * Timers and launch counts, the counterpart of the reference's wall-clock
 * timers xctmr0/xctmr1/xctmrp (mod_xc_sm.h:1431-1627; timer 41 = tsadvc,
 * mod_hycom.F90:1146, timer 12 = xctilr).  When enabled, every timed
 * region is bracketed by CUDA events on the context stream, so the times
 * are device times.  Timer slots: HYC_T_*.
 */
#define HYC_T_TSADVC 0 /* whole hyc_tsadvc call (device span)   */
#define HYC_T_XCTILR 1 /* halo fills                            */
#define HYC_T_ADVECT 2 /* fused advection kernels               */
#define HYC_T_COPY 3   /* copy of updated slices into level n   */
#define HYC_T_DIAG 4   /* salinity range diagnostic             */
#define HYC_T_TSDFF 5  /* lateral diffusion (hyc_tsdff)         */
#define HYC_T_ASSELIN 6 /* Robert-Asselin save and filter      */
#define HYC_T_CNUITY 7  /* continuity equation (hyc_cnuity)    */
#define HYC_NTIMERS 8

typedef struct hyc_stats {
  int64_t launches;            /* kernels launched by this context      */
  int64_t calls[HYC_NTIMERS];  /* timed regions completed per slot      */
  double ms[HYC_NTIMERS];      /* accumulated device milliseconds       */
} hyc_stats;

/*
 * advem's explicit conservation switch (mod_tsadvc.F90:32, lconserve,
 * .false. as shipped; the rescale at :168-203).  on = 1: after every
 * advem of hyc_tsadvc and hyc_advem, the tracer contents before and after,
 * sum(fld_old*fco*scp2) and sum(fld_new*fcn*scp2) over the interior sea
 * points, are summed in xcsum's order (mod_xc_sm.h:900-963) and the new
 * values at sea points are multiplied by 1 + (old-new)/new, bit for bit as
 * the reference does.  Not available with advem_fct2c (btrmas with FCT2),
 * whose scheme forms no such contents (HYC_ERR_UNSUPPORTED).
 */
int hyc_set_conserve(hyc_ctx *ctx, int32_t on);
int hyc_enable_timers(hyc_ctx *ctx, int32_t on);
/* Wait for the stream, fold finished timings in, copy out; reset=1 zeroes. */
int hyc_get_stats(hyc_ctx *ctx, hyc_stats *out, int32_t reset);

/*
 * advem on one 2-D slice that allocates no device memory.  No counterpart
 * in the reference: it exists for callers that cannot allocate device
 * memory when they call the advection -- a model whose device memory is
 * handed in full to its own pool allocator at start-up, or a time loop that
 * must not call into the CUDA allocator because cudaMalloc/cudaFree can
 * synchronise the whole device.  Same arguments and result as hyc_advem
 * with where = HYC_DEVICE, but without a context: the grid sizes and the
 * masks ip/iu/iv (int32, device, one slice each, the bigrid masks) are
 * passed in, and the work runs on `stream` (a cudaStream_t, NULL for the
 * default stream).  The masks are checked on the GPU as hyc_adv_init
 * checks them (iu = ip(i)*ip(i-1), iv = ip(j)*ip(j-1)); the call reads that
 * check back, so it returns after its GPU work, with HYC_ERR_MASK if the
 * masks are inconsistent.  Scratch is a fixed array of 2^21 cells
 * (18 MiB) inside the library that every GPU loading the library holds
 * until exit; slices with more than 2^21 cells ((idm+2*nbdy)*(jdm+2*nbdy))
 * or nbdy > 64 are rejected with HYC_ERR_ARG.
 * All calls on a device share that array: calls whose GPU work overlaps
 * race and must be ordered by the caller.  The first call on a device
 * looks up the array's address; make it before any stream capture.
 * FCT2 with btrmas (fct2c) is not available here.  Errors: HYC_ERR_* and
 * the message from hyc_last_error(NULL, ...).
 */
int hyc_advem_noalloc(int32_t idm, int32_t jdm, int32_t nbdy, int32_t advtyp, double *fld,
                      const double *fldc, const double *u, const double *v, const double *fco,
                      const double *fcn, double posdef, const double *scal, const double *scali,
                      double dt2, const int32_t *ip, const int32_t *iu, const int32_t *iv,
                      void *stream);

/* ------------------------------------------------------------------------
 * Ensemble (batched) form: many independent basins of uneven size, layer
 * and tracer count advected together, one persistent launch per step over
 * a queue of (basin, tile) work items.  No counterpart in the reference
 * (HYCOM runs one basin per executable); each basin's step is tsadvc's
 * advection of its tracers (mod_tsadvc.F90:1708-2048, passive tracers).
 *
 * Precision: HYC_PREC_FP64 (the plain form: FP64 state, bit-identical to
 * hyc_tsadvc) or HYC_PREC_MIXED (FP32 tracer state, fluxes, limiter and
 * update; FP64 dp, continuity and thickness division; see hyc_mixed_col2.cu).
 * The library keeps three leapfrog levels per basin and rotates them, so a
 * step never updates a level in place.
 * ---------------------------------------------------------------------- */
#define HYC_PREC_FP64 0
#define HYC_PREC_MIXED 1

/* what hyc_ens_put / hyc_ens_get move (reference layout, FP64, host or device) */
#define HYC_E_OLD 0  /* tracers at t-1: ntr*kdm slices (tracer-major)  */
#define HYC_E_CUR 1  /* tracers at t:   ntr*kdm slices                 */
#define HYC_E_UFLX 2 /* uflx(:,:,k), kdm slices                        */
#define HYC_E_VFLX 3 /* vflx(:,:,k), kdm slices                        */
#define HYC_E_DP 4   /* dp(:,:,k,n), kdm slices (new thickness)         */

typedef struct hyc_ens hyc_ens;

typedef struct hyc_basin_spec {
  int32_t idm, jdm, kdm, nbdy, nreg, ntr;
  const int32_t *ip, *iu, *iv;  /* host, ld1*ld2 each (bigrid masks)          */
  const double *scp2, *scp2i;   /* host, ld1*ld2 each                         */
} hyc_basin_spec;

int hyc_ens_create(hyc_ens **ens, int32_t nbasin, const hyc_basin_spec *specs, int32_t precision,
                   int32_t device);
int hyc_ens_destroy(hyc_ens *ens);
/* As hyc_set_stream, for an ensemble (graphs are replayed on this stream). */
int hyc_ens_set_stream(hyc_ens *ens, void *stream);
/* src/dst: ld1*ld2*(slices) doubles in the reference layout (pitch idm+2*nbdy) */
int hyc_ens_put(hyc_ens *ens, int32_t basin, int32_t what, const double *src, int32_t where);
int hyc_ens_get(hyc_ens *ens, int32_t basin, int32_t what, double *dst, int32_t where);
/*
 * As hyc_ens_get, but returns once the values are staged on the device:
 * the copy into dst runs on a copy stream of the ensemble and overlaps the
 * puts and steps queued after it (host<->device links are full duplex).
 * dst must stay valid and is not to be read (nor passed to hyc_ens_put)
 * until hyc_ens_wait returns.
 * A later get_async waits for the previous one's copy-out on the device.
 */
int hyc_ens_get_async(hyc_ens *ens, int32_t basin, int32_t what, double *dst, int32_t where);
/* Wait for every hyc_ens_get_async copy-out issued so far. */
int hyc_ens_wait(hyc_ens *ens);
/* The same for the slices [s0, s0+ns) only (tracer-major for HYC_E_OLD/CUR:
 * slice q*kdm+k), so a caller can move one tracer at a time. */
int hyc_ens_put_slices(hyc_ens *ens, int32_t basin, int32_t what, int32_t s0, int32_t ns, const double *src,
                       int32_t where);
int hyc_ens_get_slices(hyc_ens *ens, int32_t basin, int32_t what, int32_t s0, int32_t ns, double *dst,
                       int32_t where);
/* Tile shape of the step kernel; hyc_ens_tune picks one.  Mixed form:
 * tx = 56, the strip kernel (64-column strips streamed by TMA, 56 columns
 * updated), ty = rows per segment, 32 to 2048 (powers of 2).  FP64 form: 32 x 16
 * or 16 x 16 cell tiles. */
int hyc_ens_set_tile(hyc_ens *ens, int32_t tx, int32_t ty);
/*
 * Autotuner: time every supported tile shape on this ensemble (the kernel
 * writes only the spare leapfrog level, so the state does not change),
 * keep the fastest and return it (tx, ty, ms of the best step; may be NULL).
 */
int hyc_ens_tune(hyc_ens *ens, int32_t advtyp, double delt1, int32_t *tx, int32_t *ty, double *ms);
/*
 * Advance every basin nsteps leapfrog steps.  advtyp: FP64 form 0 (PCM),
 * 1 (MPDATA), 2 (FCT2), 4 (FCT4); FP32-mixed form 1 (MPDATA), 2 (FCT2)
 * and 4 (FCT4).  PCM and MPDATA read only level t-1 (mod_tsadvc.F90:152, :495).
 * use_graph = 1: the nsteps launches are captured once into a CUDA graph
 * (per nsteps/advtyp/delt1/tile) and replayed.  Asynchronous.
 */
int hyc_ens_step(hyc_ens *ens, int32_t advtyp, double delt1, int32_t nsteps, int32_t use_graph);
/*
 * FP64 tracer content of basin b, tracer q, level what (HYC_E_OLD with the
 * old thickness fco, or HYC_E_CUR with fcn), summed over layers and interior
 * sea cells: sum fld*(fc+onemu)*scp2, compensated.  Synchronous.
 */
int hyc_ens_content(hyc_ens *ens, int32_t basin, int32_t tracer, int32_t what, double delt1, double *sum);
int hyc_ens_stats(hyc_ens *ens, hyc_stats *out, int32_t reset);
/*
 * Options.  HYC_OPT_PREP64 (mixed form only; default 1): 1 = the per cell
 * and layer thickness prep runs in FP64 -- the continuity update
 * fco+onemu = (dp+onemu) + div*dt2*scp2i, fcn+onemu, the reciprocal
 * 1/(fcn+onemu) (hardware seed and one Newton step, relative error below
 * 2^-40) and W = (fco+onemu)/(fcn+onemu); the face-flux divergence is a
 * compensated (two-sum) FP32 sum of the FP32 fluxes.  0 = the same factors
 * in compensated FP32 (W = 1 + div/(fcn+onemu)), which leaves the FP64 pipe
 * idle (GB300 issues FP64 at ~1/70 of the FP32 rate).  dp is read in FP64
 * either way.
 */
#define HYC_OPT_PREP64 1
/* HYC_OPT_STRIP_TRACERS (mixed form; default 2): tracers advanced per pass
 * over a layer.  2: one warp advances two tracers and shares the per-cell
 * thickness factors between them; 1: one tracer per pass, fewer registers,
 * more warps per SM.  hyc_ens_tune tries both. */
#define HYC_OPT_STRIP_TRACERS 3
int hyc_ens_set_option(hyc_ens *ens, int32_t option, int32_t value);
/*
 * MPDATA offset of one tracer of one basin (default 0).  The reference uses
 * 256 for temp, 32 for th3d, 1 for q2 and 0 for saln and passive tracers
 * (mod_tsadvc.F90:1755-1763); FCT ignores it.  Synchronous.
 */
int hyc_ens_set_posdef(hyc_ens *ens, int32_t basin, int32_t tracer, double posdef);
/*
 * Lateral diffusion of basin b's tracers at the end of each step, fused
 * into the step kernel's epilogue (FP32-mixed form with the FP64 thickness
 * prep): the diffusion block of tsadvc (mod_tsadvc.F90:2138-2230) for
 * hybrid layers with temdfc = 1 -- tsdff_2x / tsdff_1x (:2262-2492) on
 * every tracer of the new level, face factors temdf2*aspux*scuy and
 * temdf2*aspvy*scvx (where iu / iv) times the harmonic mean of max(dp,0)
 * (dp = HYC_E_DP, the new thickness; onetamas = 1), the update
 * -delt1/(scp2*max(dp,eps_har)) times the flux divergence at sea cells.
 * The new values are written once, diffused.  th3d is not formed (the
 * ensemble's tracers are generic).  aspux, aspvy, scuy, scvx: ld1*ld2
 * doubles in the reference layout, halo included, host or device (where);
 * temdf2 = 0 turns it off for the basin.  The FP64 form returns
 * HYC_ERR_UNSUPPORTED (its diffusion is hyc_tsdff).  Synchronous.
 */
int hyc_ens_set_diffusion(hyc_ens *ens, int32_t basin, double temdf2, const double *aspux, const double *aspvy,
                          const double *scuy, const double *scvx, int32_t where);
int hyc_ens_get_option(hyc_ens *ens, int32_t option, int32_t *value);
int hyc_ens_enable_timers(hyc_ens *ens, int32_t on);
const char *hyc_ens_last_error(const hyc_ens *ens);

/* ------------------------------------------------------------------------
 * HYCOM .a/.b field input, so that fields of a HYCOM run (restart or
 * archive files) can feed the advection.
 * ---------------------------------------------------------------------- */
/*
 * Record `record` (1-based) of a .a file -- big-endian IEEE real*4 records of
 * idm*jdm words padded to a multiple of 4096 -- into the interior of h
 * (reference layout (1-nbdy:idm+nbdy, 1-nbdy:jdm+nbdy), doubles, halo
 * untouched; where = HYC_HOST or HYC_DEVICE).  With mask (reference layout,
 * may be NULL) only points with mask != 0 are stored and enter the range,
 * and 2^100 (data void) there is an error; without a mask every point is
 * stored and the range leaves 2^100 out.  hmin/hmax (may be NULL) receive
 * the range.  Synchronous.
 * Replaces: mod_za_sm.h:700 (subroutine zaiord), :944 (zaiordd).
 */
int hyc_za_read(const char *path, int32_t idm, int32_t jdm, int32_t nbdy, int32_t record, const int32_t *mask,
                double *h, int32_t where, double *hmin, double *hmax);
/*
 * One .b line "cfield  : ... = layer level hmin hmax": cfield (9 bytes, may
 * be NULL) receives the first 8 characters, the rest the four numbers after
 * '='.  Replaces the parsing in mod_restart.F90:594-603 (restart_in3d).
 */
int hyc_za_parse_b(const char *line, char *cfield, int32_t *layer, int32_t *level, double *hmin, double *hmax);
/*
 * restart_in3d's consistency test of a field against its .b line
 * (mod_restart.F90:604-605): both ends within 1e-4 relative, else
 * HYC_ERR_ARG.
 */
int hyc_za_check(double hmin_a, double hmax_a, double hmin_b, double hmax_b);

/*
 * Self-test of the streaming kernels' failure path, which faults nothing:
 * one thread on the GPU waits on an mbarrier through the bounded wait the
 * TMA-fed kernels use (limit 2 s).  arrive = 0: nothing completes the
 * barrier, the wait gives up, records the failure in a device error flag
 * and the kernel returns (*gave_up = 1; the device stays usable -- a step
 * kernel in that state makes hyc_ens_stats return HYC_ERR_CUDA); arrive = 1:
 * the barrier completes first (*gave_up = 0).  No counterpart in the
 * reference, which has no recovery path (xcstop).  Synchronous.
 */
int hyc_selftest_wait(int32_t device, int32_t arrive, int32_t *gave_up);

/* Library build identification, e.g. "hycadv 0.1 sm_103a". */
const char *hyc_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HYCOM_ADV_H */
