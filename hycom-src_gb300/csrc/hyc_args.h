// hyc_args.h -- plain-C++ layout of the kernel arguments, shared by the CUDA
// translation units and the host layer.
#pragma once
#include <cstddef>
#include <cstdint>

namespace hyc {

constexpr uint8_t kIP = 1, kIU = 2, kIV = 4;  // mask bits: ip, iu, iv

constexpr int kMaxFields = 16;
enum Scheme { kPCM = 0, kMPDATA = 1, kFCT2 = 2, kFCT4 = 4 };

struct FieldDesc {
  double *nbase;        // first slice of time level n (old in, new out)
  const double *mbase;  // first slice of time level m (center)
  int k_off;            // slice index of layer k=1 (1 for q2/q2l, whose k starts at 0)
  int kmin, kmax;       // the field is advected for kmin <= k <= kmax (1-based)
  int pad;
  double posdef;        // MPDATA offset, mod_tsadvc.F90:1761-1763
};

struct TileArgs {
  int ii, jj, nbdy, ld1, ld2;
  long long slice;  // ld1*ld2
  int ntx, nty;     // tiles in x and y
  int mode;         // 0: tsadvc (fco/fcn from dp, uflx, vflx); 1: advem (fco/fcn given)
  const uint8_t *msk;
  const double *scal, *scali;
  // tsadvc mode, per layer k (0-based): uflx + k*slice, vflx + k*slice, dpn + k*slice
  const double *uflx, *vflx, *dpn;
  const double *oneta_n;  // onetamas(:,:,m) when btrmas (mod_tsadvc.F90:1806), else null
  // tsadvc mode, isopycnic layer 1 only: the fluxes whose divergence gives
  // fco (the smoothed mixed-layer fluxes, mod_tsadvc.F90:1860-1897) when the
  // fields advected by uflx/vflx are not the ones smoothed; null otherwise
  const double *ufco, *vfco;
  // advem's conservation rescale (lconserve): per (field, layer) factor
  // 1 + offset applied by the copy back, index fi*kdm + k; null: none
  const double *cfac;
  // TMA staging of the tile region (null: plain loads): CUtensorMap array
  // in device memory, FP64, box (TX+8) x (TY+6):
  //   [0] uflx, [1] vflx (slice k of the layer; advem: the one slice),
  //   [2] dp(:,:,:,n) (advem: fcn), [3] onetamas(m) (advem: fco; tm_has3 = 0
  //   when absent), [4] scal, [5] scali, then [6 + 2*fi] level n and
  //   [7 + 2*fi] level m of field fi (slice k + k_off)
  const void *tmaps;
  int tm_has3;
  int *err;  // set when a bounded TMA wait gave up (may be null)
  // advem mode (single slice)
  const double *fco, *fcn;
  double dt2;
  int nfld;
  FieldDesc f[kMaxFields];
  // output: out + (fi*kdm + k)*slice; sea cells of the interior are written
  double *out;
  int kdm;
  // >0: also write the periodic-x halo images of output cells with
  // i <= images or i > ii-images (an ensemble level is its own halo source)
  int images;
};

// advem_fct2c (mod_tsadvc.F90:999-1368) over up to kMaxFields (field, layer)
// pairs, see hyc_fct2c.cu
struct Fct2cArgs {
  int ii, jj, nb, ld1, ld2;
  long long slice;
  int mode;  // 0: fco/fcn from dp(n), uflx, vflx, onetamas (tsadvc); 1: given (advem)
  const uint8_t *msk;
  const double *scal, *scali;
  const double *uflx, *vflx, *dpn, *oneta;  // mode 0: per layer k (+k*slice); oneta may be null
  const double *fco, *fcn;                  // mode 1
  double dt2;
  int npair;
  double *work;     // A_N * npair slices
  uint8_t *lcalc;   // npair slices
  double *fld[kMaxFields];         // level n of each pair's layer (in: t-1, out: t+1)
  const double *fldc[kMaxFields];  // level m (t)
  int k[kMaxFields];               // layer (0-based) of each pair
};

// Lateral diffusion of tsadvc (mod_tsadvc.F90:2138-2230) over up to
// kMaxFields fields of every layer, see hyc_tsdff.cu
struct TsdffArgs {
  int ii, jj, nb, ld1, ld2;
  long long slice;
  const uint8_t *msk;
  const double *scp2, *aspux, *aspvy, *scuy, *scvx;
  const double *oneta;  // onetamas(:,:,n) = oneta(:,:,n) (mod_tsadvc.F90:1805, :1808)
  const double *dpn;    // dp(:,:,1,n); layer k at +k*slice
  double temdf2, delt1, thbase;
  int kdm, nfld;
  double *fld[kMaxFields];  // layer 1 of level n of each field; layer k at +k*slice
  double *out;              // new values: out + (fi*kdm + k)*slice
  int eos_t, eos_s;         // fields whose new values give th3d (-1: none)
  double *th3d;             // th3d(:,:,1,n) when eos_t >= 0
};

// Robert-Asselin filter (mod_asselin.F90), see hyc_asselin.cu; arrays in
// the reference layout (mod_cb_arrays.F90)
struct AsselinArgs {
  int ii, jj, nb, ld1, ld2;
  long long slice;
  int kdm, m, n, ntracr, mxlmy;
  const uint8_t *msk;
  double oneta0, ra2fac, thbase;
  double *temp, *saln, *th3d;  // (ld1,ld2,kdm,2)
  double *tracer;              // (ld1,ld2,kdm,2,ntracr)
  double *q2, *q2l;            // (ld1,ld2,0:kdm+1,2)
  double *dp;                  // (ld1,ld2,kdm,2); level m filtered
  const double *dpo;           // (ld1,ld2,kdm,2)
  const double *pbavg, *pbot;  // (ld1,ld2,3), (ld1,ld2)
  double *oneta, *onetao;      // (ld1,ld2,2)
  double *otemp, *osaln, *oth3d, *otracer, *oq2, *oq2l;  // t-1 copies
};

// Continuity equation (cnuity.F90), see hyc_cnuity.cu; arrays in the
// reference layout (mod_cb_arrays.F90)
struct CnuityArgs {
  int ii, jj, nb, ld1, ld2, nreg;
  long long slice;
  int kdm, m, n, nstep, btrmas, thk;  // thk: 0 none, 4 biharmonic, 2 Laplacian interface diffusion
  const uint8_t *msk;
  const double *scp2, *scp2i, *scuy, *scvx, *depthu, *depthv, *thkdfu, *thkdfv, *pbot, *oneta;
  const double *u, *v, *dpu, *dpv;  // (ld1,ld2,kdm,2)
  const double *ubavg, *vbavg;      // (ld1,ld2,3)
  double *dp, *dpo;                 // (ld1,ld2,kdm,2)
  double *p;                        // (ld1,ld2,kdm+1)
  double *uflx, *vflx;              // (ld1,ld2,kdm)
  double *uflxav, *vflxav, *dpav;   // (ld1,ld2,kdm) or null
  double *onetacnt;                 // (ld1,ld2), btrmas
  double delt1, ra2fac;
  double dtinv;                     // 1/delt1, divided once on the host
  double *w;                        // work slices
  long long *keys;                  // 2*kdm dpkmin keys, or null
};

// Region of the generic tile kernel: RW x RY cells (TX x TY output cells and
// a 3-cell ring), rows stored RX apart.  RX = TX + 8 (an even count of
// doubles: TMA boxes of 16-byte rows starting on an even column, the region
// at offset 0 or 1 in each array's slot) when the arrays then fit in shared
// memory, else TX + 6 and plain loads only.
template <int TX, int TY>
struct TileGeom {
  // per-layer arrays: U V FCO FCN HN RH SCAL SCALI ; per-field: FLD FLDC FX FY FLO FXL FNL RP RM QX QN
  static constexpr int NLAYER = 8, NFIELD = 11, NARR = NLAYER + NFIELD;
  static constexpr int RW = TX + 6, RY = TY + 6;
  static constexpr int slot(int rx) { return (rx * RY + 1 + 15) / 16 * 16; }
  static constexpr size_t bytes(int rx) {
    return 128 + (size_t)NARR * slot(rx) * sizeof(double) + (size_t)((rx * RY + 15) / 16) * 16;
  }
  static constexpr bool TMA = bytes(TX + 8) <= 227 * 1024;
  static constexpr int RX = TMA ? TX + 8 : TX + 6;
  static constexpr int NR = RX * RY, N = slot(RX);
  static constexpr unsigned BOX = NR * 8;  // bytes of one TMA box
  static constexpr size_t smem_bytes = bytes(RX);
};

}  // namespace hyc
