// hyc_host.cpp -- host side of libhycadv: contexts, resident fields, the
// tsadvc/advem/xctilr drivers and the C ABI declared in include/hycom_adv.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hycom_adv.h"

#include <cstddef>

#include "hyc_tmap.h"

// The parameter blocks are passed by reference from Fortran as bind(c)
// derived types (ten int32 flags then delt1 and the trcflg pointer; four
// int32 then delt1 and ra2fac; an int64, eight int64 counts, eight doubles):
// their C layout must be exactly the one those types get.
static_assert(sizeof(int32_t) == 4 && sizeof(double) == 8 && sizeof(void *) == 8, "LP64 ABI");
static_assert(offsetof(hyc_tsadvc_params, advtyp) == 0 && offsetof(hyc_tsadvc_params, diagno) == 36 &&
                  offsetof(hyc_tsadvc_params, delt1) == 40 && offsetof(hyc_tsadvc_params, trcflg) == 48 &&
                  sizeof(hyc_tsadvc_params) == 56,
              "hyc_tsadvc_params must match its bind(c) type");
static_assert(offsetof(hyc_cnuity_params, nstep) == 0 && offsetof(hyc_cnuity_params, isopyc) == 12 &&
                  offsetof(hyc_cnuity_params, delt1) == 16 && offsetof(hyc_cnuity_params, ra2fac) == 24 &&
                  sizeof(hyc_cnuity_params) == 32,
              "hyc_cnuity_params must match its bind(c) type");
static_assert(offsetof(hyc_stats, calls) == 8 && offsetof(hyc_stats, ms) == 8 + 8 * HYC_NTIMERS &&
                  sizeof(hyc_stats) == 8 + 16 * HYC_NTIMERS,
              "hyc_stats must match its bind(c) type");
#include "hyc_internal.h"
#include "hyc_args.h"

using hyc::FieldDesc;
using hyc::TileArgs;

namespace {

thread_local std::string g_lib_error;

struct Field {
  double *dev = nullptr;   // device data used by the kernels
  double *host = nullptr;  // caller's host array (HYC_HOST binding)
  int64_t nelem = 0;
  bool owned = false;      // dev allocated by the library
};

}  // namespace

struct hyc_ctx {
  int idm = 0, jdm = 0, kdm = 0, nbdy = 0, nreg = 0, ld1 = 0, ld2 = 0;
  long long slice = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  uint8_t *d_msk = nullptr;
  double *d_scp2 = nullptr, *d_scp2i = nullptr;
  double *d_diff = nullptr;     // aspux, aspvy, scuy, scvx (4 slices), hyc_set_diffusion_grid
  double *d_cngrid = nullptr;   // scuy, scvx, depthu, depthv, thkdfu, thkdfv (6 slices), hyc_set_cnuity_grid
  bool cn_thkdf = false;        // thkdfu/thkdfv were given
  double *d_cnw = nullptr;      // cnuity work slices
  long long *d_cnkeys = nullptr;  // cnuity dpkmin keys (2*kdm)
  Field fields[HYC_NFIELDS];
  double *d_scratch = nullptr;  // advem output slices (fields x layers)
  double *d_iso = nullptr;      // smoothed layer-1 fluxes of isopycnic mode (2 slices)
  bool lconserve = false;       // advem's explicit conservation rescale (hyc_set_conserve)
  CUtensorMap *d_tmaps = nullptr;  // TMA maps of the FCT tile launches of one call
  size_t tmaps_cap = 0;
  int *d_err = nullptr;            // a TMA wait of a tile kernel gave up
  double *d_cons = nullptr;     // its row sums and factors
  size_t cons_elems = 0;
  size_t scratch_elems = 0;
  unsigned char *d_fct2c = nullptr;  // advem_fct2c work arrays (per (field, layer) pair)
  size_t fct2c_bytes = 0;
  double *d_tmp = nullptr;      // staging for host-pointer advem/xctilr (8 slices)
  long long *d_keys = nullptr;  // salinity range keys (2*kdm)
  long long *h_keys = nullptr;  // pinned
  double *d_sum = nullptr;      // mass-sum partials + result
  double *h_sum = nullptr;      // pinned
  hyc::TileShape shape{32, 16};
  std::string err;
  // timers (HYC_T_*) and launch accounting
  bool timing = false;
  struct Pending {
    int slot;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> event_pool;
  hyc_stats stats{};
};

namespace {

int fail(hyc_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  g_lib_error = buf;
  return code;
}

int cuda_fail(hyc_ctx *c, cudaError_t e, const char *what) {
  return fail(c, HYC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                          \
  do {                                          \
    cudaError_t e_ = (call);                    \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

inline long long off(const hyc_ctx *c, int i, int j) {
  return (long long)(i + c->nbdy - 1) + (long long)(j + c->nbdy - 1) * c->ld1;
}

const int kMbdy[5] = {2, 5, 5, 0, 5};  // mbdy_advtyp, mod_tsadvc.F90:24-29

bool valid_advtyp(int a) { return a == 0 || a == 1 || a == 2 || a == 4; }

hyc::TileShape env_shape(hyc::TileShape def) {
  const char *s = getenv("HYC_TILE");
  if (!s) return def;
  hyc::TileShape t{0, 0};
  if (sscanf(s, "%dx%d", &t.tx, &t.ty) == 2 && hyc::advect_tile_shape_ok(t)) return t;
  return def;
}

int ensure_fct2c(hyc_ctx *c, size_t bytes) {
  if (c->fct2c_bytes >= bytes) return HYC_OK;
  if (c->d_fct2c) cudaFree(c->d_fct2c);
  c->d_fct2c = nullptr;
  c->fct2c_bytes = 0;
  cudaError_t e = cudaMalloc(&c->d_fct2c, bytes);
  if (e != cudaSuccess) return fail(c, HYC_ERR_NOMEM, "cannot allocate %zu bytes of fct2c work arrays", bytes);
  c->fct2c_bytes = bytes;
  return HYC_OK;
}

// Pairs per advem_fct2c launch: up to kMaxFields, work arrays within ~4 GB.
int fct2c_batch(const hyc_ctx *c) {
  const size_t per = hyc::fct2c_work_bytes(c->slice);
  size_t n = ((size_t)4 << 30) / (per ? per : 1);
  if (n < 1) n = 1;
  if (n > (size_t)hyc::kMaxFields) n = hyc::kMaxFields;
  return (int)n;
}

void fct2c_bind(hyc::Fct2cArgs &f, const hyc_ctx *c, int npair) {
  const size_t sl = (size_t)c->slice;
  f.npair = npair;
  f.work = (double *)c->d_fct2c;
  f.lcalc = c->d_fct2c + (size_t)npair * sl * 13 * sizeof(double);
}

// TMA maps of the FCT tile kernel for the launches of one call (box TX+8 x
// TY+6, FP64; see TileArgs::tmaps): host list, then one copy to the device.
// use = false when the arrays break a TMA rule (pitch or base alignment):
// those launches stage with plain loads.
struct TileMaps {
  std::vector<CUtensorMap> h;
  bool use = true;
};

// append the maps of launch a; returns its first index, or -1 (plain loads)
long tile_maps_add(const hyc_ctx *c, const hyc::TileArgs &a, int kk, bool flux1, TileMaps &tmv) {
  if (!tmv.use || !hyc::tmap_available()) return -1;
  const int bx = c->shape.tx + 8, by = c->shape.ty + 6;
  const long long w = c->idm + 2LL * c->nbdy, h = c->jdm + 2LL * c->nbdy, ld = c->ld1, sl = c->slice;
  std::vector<CUtensorMap> m(6 + 2 * (size_t)a.nfld);
  bool ok = true;
  auto enc = [&](CUtensorMap *p, const double *base, long long nz) {
    ok = ok && hyc::tmap_encode3(p, base, 8, w, h, ld, sl, nz, bx, by);
  };
  const long long nzf = a.mode == 0 ? (flux1 ? 1 : kk) : 1;
  enc(&m[0], a.uflx, nzf);
  enc(&m[1], a.vflx, nzf);
  enc(&m[2], a.mode == 0 ? a.dpn : a.fcn, a.mode == 0 ? kk : 1);
  const double *m3 = a.mode == 0 ? a.oneta_n : a.fco;
  if (m3) enc(&m[3], m3, 1);
  enc(&m[4], a.scal, 1);
  enc(&m[5], a.scali, 1);
  for (int fi = 0; fi < a.nfld; fi++) {
    const long long nz = kk + 2LL * a.f[fi].k_off;  // q2/q2l: 0..kk+1
    enc(&m[6 + 2 * fi], a.f[fi].nbase, nz);
    enc(&m[7 + 2 * fi], a.f[fi].mbase, nz);
  }
  if (!ok) return -1;
  const long at = (long)tmv.h.size();
  tmv.h.insert(tmv.h.end(), m.begin(), m.end());
  return at;
}

// copy the call's maps to the device; the launches then point into it
int tile_maps_upload(hyc_ctx *c, const TileMaps &tmv) {
  if (tmv.h.empty()) return HYC_OK;
  if (c->tmaps_cap < tmv.h.size()) {
    CK(cudaStreamSynchronize(c->stream), "maps sync");  // earlier launches may read the old buffer
    cudaFree(c->d_tmaps);
    c->d_tmaps = nullptr;
    c->tmaps_cap = 0;
    CK(cudaMalloc(&c->d_tmaps, tmv.h.size() * sizeof(CUtensorMap)), "malloc tensor maps");
    c->tmaps_cap = tmv.h.size();
  }
  CK(cudaMemcpyAsync(c->d_tmaps, tmv.h.data(), tmv.h.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, c->stream),
     "tensor maps");
  return HYC_OK;
}

// the lconserve rescale of one tile launch: a.cfac is set for its copy back
int conserve(hyc_ctx *c, hyc::TileArgs &a, int nlayers) {
  const size_t rows = hyc::conserve_rows_elems(a.nfld, a.kdm, a.jj), need = rows + (size_t)a.nfld * a.kdm;
  if (c->cons_elems < need) {
    cudaFree(c->d_cons);
    c->d_cons = nullptr;
    c->cons_elems = 0;
    cudaError_t e = cudaMalloc(&c->d_cons, need * sizeof(double));
    if (e != cudaSuccess) return fail(c, HYC_ERR_NOMEM, "lconserve work: %s", cudaGetErrorString(e));
    c->cons_elems = need;
  }
  cudaError_t e = hyc::launch_conserve(a, nlayers, c->d_cons, c->d_cons + rows, c->stream);
  if (e != cudaSuccess) return fail(c, HYC_ERR_CUDA, "lconserve: %s", cudaGetErrorString(e));
  c->stats.launches += 2;
  a.cfac = c->d_cons + rows;
  return HYC_OK;
}

int ensure_scratch(hyc_ctx *c, size_t elems) {
  if (c->scratch_elems >= elems) return HYC_OK;
  if (c->d_scratch) cudaFree(c->d_scratch);
  c->d_scratch = nullptr;
  c->scratch_elems = 0;
  cudaError_t e = cudaMalloc(&c->d_scratch, elems * sizeof(double));
  if (e != cudaSuccess) return fail(c, HYC_ERR_NOMEM, "cannot allocate %zu bytes of scratch", elems * 8);
  c->scratch_elems = elems;
  return HYC_OK;
}

// ---------------------------------------------------------------------------
// host xctilr used by bigrid (same halo rule as the device kernel)
// ---------------------------------------------------------------------------
template <class T>
void host_halo(T *a, int ii, int jj, int nb, int ld1, int nreg) {
  auto at = [&](int i, int j) -> T & { return a[(i + nb - 1) + (long long)(j + nb - 1) * ld1]; };
  const bool closed_y = nreg <= 2, closed_x = (nreg == 0 || nreg == 4);
  for (int j = 1; j <= nb; j++)
    for (int i = 1; i <= ii; i++) {
      at(i, 1 - j) = closed_y ? T(0) : at(i, jj + 1 - j);
      at(i, jj + j) = closed_y ? T(0) : at(i, j);
    }
  for (int j = 1 - nb; j <= jj + nb; j++)
    for (int i = 1; i <= nb; i++) {
      at(1 - i, j) = closed_x ? T(0) : at(ii + 1 - i, j);
      at(ii + i, j) = closed_x ? T(0) : at(i, j);
    }
}

cudaEvent_t get_event(hyc_ctx *c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Bracket a region of stream work with events when timers are on.
struct Timed {
  hyc_ctx *c;
  int slot;
  cudaEvent_t a = nullptr;
  Timed(hyc_ctx *c_, int s) : c(c_), slot(s) {
    if (c->timing) {
      a = get_event(c);
      cudaEventRecord(a, c->stream);
    }
  }
  ~Timed() {
    if (c->timing && a) {
      cudaEvent_t b = get_event(c);
      cudaEventRecord(b, c->stream);
      c->pending.push_back({slot, a, b});
    }
  }
};

void fold_timings(hyc_ctx *c) {
  for (auto &p : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      c->stats.ms[p.slot] += ms;
      c->stats.calls[p.slot] += 1;
    }
    c->event_pool.push_back(p.a);
    c->event_pool.push_back(p.b);
  }
  c->pending.clear();
}

}  // namespace

void hyc::set_library_error(const char *msg) { g_lib_error = msg ? msg : ""; }

extern "C" {

int hyc_set_conserve(hyc_ctx *c, int32_t on) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  c->lconserve = on != 0;
  return HYC_OK;
}

int hyc_enable_timers(hyc_ctx *c, int32_t on) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  c->timing = on != 0;
  return HYC_OK;
}

// after a stream synchronisation: a tile kernel's bounded TMA wait gave up
int tma_flag(hyc_ctx *c) {
  int flag = 0;
  CK(cudaMemcpy(&flag, c->d_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (flag) {
    cudaMemset(c->d_err, 0, sizeof(int));
    return fail(c, HYC_ERR_CUDA, "a tile kernel gave up waiting for its TMA loads");
  }
  return HYC_OK;
}

int hyc_get_stats(hyc_ctx *c, hyc_stats *out, int32_t reset) {
  if (!c || !out) return fail(c, HYC_ERR_ARG, "hyc_get_stats: null argument");
  DeviceGuard g(c->device);
  CK(cudaStreamSynchronize(c->stream), "stats sync");
  if (int rc = tma_flag(c)) return rc;
  fold_timings(c);
  *out = c->stats;
  if (reset) c->stats = hyc_stats{};
  return HYC_OK;
}

const char *hyc_version(void) { return "hycadv 0.1 sm_103a"; }

int hyc_last_error(const hyc_ctx *ctx, char *buf, size_t n) {
  if (!buf || n == 0) return HYC_ERR_ARG;
  const std::string &s = ctx ? ctx->err : g_lib_error;
  snprintf(buf, n, "%s", s.c_str());
  return HYC_OK;
}

// ---------------------------------------------------------------------------
// bigrid.F90:1-415 for one tile (i0=j0=0), mapflg != 4.  The land/sea
// masks: ip where depth>0 (over the halo after the halo fill and land
// borders), iu/iv where both neighbouring p-points are sea (interior, then
// halo-filled), iq for interior and promontory vorticity points, and the
// sea-only neighbour indices (W,E,S,N if sea, else the point itself).
// ---------------------------------------------------------------------------
int hyc_bigrid(int32_t idm, int32_t jdm, int32_t nbdy, double *depth, int32_t *ip, int32_t *iu, int32_t *iv,
               int32_t *iq, int32_t *ipim1, int32_t *ipip1, int32_t *ipjm1, int32_t *ipjp1, int32_t *nreg) {
  if (idm < 1 || jdm < 1 || nbdy < 1 || !depth || !ip || !iu || !iv || !nreg)
    return fail(nullptr, HYC_ERR_ARG, "hyc_bigrid: bad arguments");
  const int ii = idm, jj = jdm, nb = nbdy, ld1 = idm + 2 * nbdy, ld2 = jdm + 2 * nbdy;
  auto D = [&](int i, int j) -> double & { return depth[(i + nb - 1) + (long long)(j + nb - 1) * ld1]; };
  // periodicity from sea in the last column / last row (bigrid.F90:25-45)
  bool lperiod = false, larctic = false;
  for (int j = 1; j <= jj; j++) lperiod |= D(ii, j) > 0.0;
  for (int i = 1; i <= ii; i++) larctic |= D(i, jj) > 0.0;
  if (larctic) return fail(nullptr, HYC_ERR_GRID, "hyc_bigrid: sea in row jdm (arctic/f-plane grids unsupported)");
  const int nr = lperiod ? 1 : 0;
  host_halo(depth, ii, jj, nb, ld1, nr);
  for (int j = 1 - nb; j <= jj + nb; j++)
    for (int i = 1 - nb; i <= ii + nb; i++) {
      bool border = j <= 0 || j > jj || (!lperiod && (i <= 0 || i > ii));
      if (border) D(i, j) = 0.0;
    }
  for (int j = 1; j <= jj; j++)  // 1-point seas (bigrid.F90:156-191)
    for (int i = 1; i <= ii; i++)
      if (D(i, j) > 0.0 && D(i - 1, j) <= 0.0 && D(i + 1, j) <= 0.0 && D(i, j - 1) <= 0.0 && D(i, j + 1) <= 0.0)
        return fail(nullptr, HYC_ERR_GRID, "hyc_bigrid: 1-point sea at i=%d j=%d", i, j);
  const size_t n2 = (size_t)ld1 * ld2;
  std::vector<int32_t> p(n2, 0), u(n2, 0), v(n2, 0), q(n2, 0);
  auto at = [&](std::vector<int32_t> &a, int i, int j) -> int32_t & {
    return a[(i + nb - 1) + (size_t)(j + nb - 1) * ld1];
  };
  for (int j = 1 - nb; j <= jj + nb; j++)
    for (int i = 1 - nb; i <= ii + nb; i++) at(p, i, j) = D(i, j) > 0.0 ? 1 : 0;
  for (int j = 1; j <= jj; j++)
    for (int i = 1; i <= ii; i++) {
      int c = at(p, i, j), w = at(p, i - 1, j), s = at(p, i, j - 1), sw = at(p, i - 1, j - 1);
      at(u, i, j) = (w > 0 && c > 0) ? 1 : 0;
      at(v, i, j) = (s > 0 && c > 0) ? 1 : 0;
      at(q, i, j) = ((c > 0 && w > 0 && s > 0 && sw > 0) || (c > 0 && sw > 0) || (w > 0 && s > 0)) ? 1 : 0;
    }
  host_halo(u.data(), ii, jj, nb, ld1, nr);
  host_halo(v.data(), ii, jj, nb, ld1, nr);
  host_halo(q.data(), ii, jj, nb, ld1, nr);
  for (int j = 1 - nb; j <= jj + nb; j++)  // land borders, part II
    for (int i = 1 - nb; i <= ii + nb; i++) {
      bool border = j <= 0 || j > jj || (!lperiod && (i <= 0 || i > ii));
      if (border) at(u, i, j) = at(v, i, j) = at(q, i, j) = 0;
    }
  memcpy(ip, p.data(), n2 * 4);
  memcpy(iu, u.data(), n2 * 4);
  memcpy(iv, v.data(), n2 * 4);
  if (iq) memcpy(iq, q.data(), n2 * 4);
  for (int j = 1 - nb; j <= jj + nb; j++)
    for (int i = 1 - nb; i <= ii + nb; i++) {
      size_t o = (i + nb - 1) + (size_t)(j + nb - 1) * ld1;
      bool edge = i == 1 - nb || i == ii + nb || j == 1 - nb || j == jj + nb;
      if (ipim1) ipim1[o] = (!edge && at(p, i - 1, j) != 0) ? i - 1 : i;
      if (ipip1) ipip1[o] = (!edge && at(p, i + 1, j) != 0) ? i + 1 : i;
      if (ipjm1) ipjm1[o] = (!edge && at(p, i, j - 1) != 0) ? j - 1 : j;
      if (ipjp1) ipjp1[o] = (!edge && at(p, i, j + 1) != 0) ? j + 1 : j;
    }
  *nreg = nr;
  return HYC_OK;
}

int hyc_adv_init(hyc_ctx **out, int32_t idm, int32_t jdm, int32_t kdm, int32_t nbdy, int32_t nreg, const int32_t *ip,
                 const int32_t *iu, const int32_t *iv, const double *scp2, const double *scp2i, int32_t device) {
  if (!out) return fail(nullptr, HYC_ERR_ARG, "hyc_adv_init: ctx is null");
  *out = nullptr;
  if (idm < 1 || jdm < 1 || kdm < 1 || nbdy < 3 || !ip || !iu || !iv || !scp2 || !scp2i)
    return fail(nullptr, HYC_ERR_ARG, "hyc_adv_init: bad sizes or null arrays (need nbdy >= 3)");
  if (!(nreg == 0 || nreg == 1 || nreg == 3 || nreg == 4 || nreg == HYC_NREG_EXTERNAL))
    return fail(nullptr, HYC_ERR_ARG, "hyc_adv_init: nreg %d unsupported (0, 1, 3, 4 or HYC_NREG_EXTERNAL)", nreg);
  hyc_ctx *c = new hyc_ctx;
  c->idm = idm;
  c->jdm = jdm;
  c->kdm = kdm;
  c->nbdy = nbdy;
  c->nreg = nreg;
  c->ld1 = idm + 2 * nbdy;
  c->ld2 = jdm + 2 * nbdy;
  c->slice = (long long)c->ld1 * c->ld2;
  c->device = device;
  c->shape = env_shape(c->shape);
  // masks: iu/iv must be the bigrid ones (iu = ip(i-1)*ip(i), iv = ip(j-1)*ip(j))
  const int nb = nbdy, ii = idm, jj = jdm;
  std::vector<uint8_t> m((size_t)c->slice, 0);
  for (int j = 1 - nb; j <= jj + nb; j++)
    for (int i = 1 - nb; i <= ii + nb; i++) {
      long long o = off(c, i, j);
      bool p = ip[o] != 0, u = iu[o] != 0, v = iv[o] != 0;
      // the outermost halo column/row cannot be checked (no i-1 / j-1) and
      // is never read by the kernels
      if (i > 1 - nb) {
        bool want = p && ip[o - 1] != 0;
        if (u != want) {
          int rc = fail(nullptr, HYC_ERR_MASK, "iu(%d,%d)=%d but ip(i-1)*ip(i)=%d", i, j, (int)u, (int)want);
          delete c;
          return rc;
        }
      }
      if (j > 1 - nb) {
        bool want = p && ip[o - c->ld1] != 0;
        if (v != want) {
          int rc = fail(nullptr, HYC_ERR_MASK, "iv(%d,%d)=%d but ip(j-1)*ip(j)=%d", i, j, (int)v, (int)want);
          delete c;
          return rc;
        }
      }
      m[o] = (p ? hyc::kIP : 0) | (u ? hyc::kIU : 0) | (v ? hyc::kIV : 0);
    }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) {
    int rc = fail(nullptr, HYC_ERR_CUDA, "hyc_adv_init: CUDA device %d not available", device);
    delete c;
    return rc;
  }
  DeviceGuard g(device);
  auto bail = [&](cudaError_t e, const char *w) {
    int rc = cuda_fail(nullptr, e, w);
    hyc_adv_finalize(c);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e, "stream");
  c->own_stream = true;
  if ((e = cudaMalloc(&c->d_msk, c->slice)) != cudaSuccess) return bail(e, "malloc msk");
  if ((e = cudaMalloc(&c->d_scp2, c->slice * 8)) != cudaSuccess) return bail(e, "malloc scp2");
  if ((e = cudaMalloc(&c->d_scp2i, c->slice * 8)) != cudaSuccess) return bail(e, "malloc scp2i");
  if ((e = cudaMalloc(&c->d_keys, 2 * kdm * sizeof(long long))) != cudaSuccess) return bail(e, "malloc keys");
  if ((e = cudaMalloc(&c->d_err, sizeof(int))) != cudaSuccess || (e = cudaMemset(c->d_err, 0, sizeof(int))) != cudaSuccess)
    return bail(e, "error flag");
  if ((e = cudaMallocHost(&c->h_keys, 2 * kdm * sizeof(long long))) != cudaSuccess) return bail(e, "host keys");
  if ((e = cudaMalloc(&c->d_sum, (2 * hyc::mass_sum_partials() + 2) * sizeof(double))) != cudaSuccess)
    return bail(e, "malloc sum");
  if ((e = cudaMallocHost(&c->h_sum, 2 * sizeof(double))) != cudaSuccess) return bail(e, "host sum");
  if ((e = cudaMemcpy(c->d_msk, m.data(), c->slice, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e, "msk");
  if ((e = cudaMemcpy(c->d_scp2, scp2, c->slice * 8, cudaMemcpyHostToDevice)) != cudaSuccess) return bail(e, "scp2");
  if ((e = cudaMemcpy(c->d_scp2i, scp2i, c->slice * 8, cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(e, "scp2i");
  *out = c;
  return HYC_OK;
}

int hyc_adv_finalize(hyc_ctx *c) {
  if (!c) return HYC_OK;
  {
    DeviceGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &f : c->fields)
      if (f.owned && f.dev) cudaFree(f.dev);
    cudaFree(c->d_msk);
    cudaFree(c->d_scp2);
    cudaFree(c->d_scp2i);
    cudaFree(c->d_diff);
    cudaFree(c->d_cngrid);
    cudaFree(c->d_cnw);
    cudaFree(c->d_cnkeys);
    cudaFree(c->d_scratch);
    cudaFree(c->d_iso);
    cudaFree(c->d_tmaps);
    cudaFree(c->d_err);
    cudaFree(c->d_cons);
    cudaFree(c->d_fct2c);
    cudaFree(c->d_tmp);
    cudaFree(c->d_keys);
    cudaFree(c->d_sum);
    for (auto &p : c->pending) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    for (auto e : c->event_pool) cudaEventDestroy(e);
    if (c->h_keys) cudaFreeHost(c->h_keys);
    if (c->h_sum) cudaFreeHost(c->h_sum);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  }
  delete c;
  return HYC_OK;
}

int hyc_set_stream(hyc_ctx *c, void *stream) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  DeviceGuard g(c->device);
  if (c->own_stream && c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return HYC_OK;
}

int hyc_synchronize(hyc_ctx *c) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  DeviceGuard g(c->device);
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return tma_flag(c);
}

int hyc_bind_field(hyc_ctx *c, int32_t field, void *ptr, int64_t nelem, int32_t where) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (field < 0 || field >= HYC_NFIELDS || !ptr || nelem <= 0 || (where != HYC_HOST && where != HYC_DEVICE))
    return fail(c, HYC_ERR_ARG, "hyc_bind_field: bad arguments (field %d)", field);
  DeviceGuard g(c->device);
  Field &f = c->fields[field];
  if (f.owned && f.dev) cudaFree(f.dev);
  f = Field{};
  f.nelem = nelem;
  if (where == HYC_DEVICE) {
    f.dev = (double *)ptr;
  } else {
    f.host = (double *)ptr;
    CK(cudaMalloc(&f.dev, (size_t)nelem * sizeof(double)), "malloc field mirror");
    f.owned = true;
  }
  return HYC_OK;
}

int hyc_sync_field(hyc_ctx *c, int32_t field, int32_t to_device) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (field < 0 || field >= HYC_NFIELDS) return fail(c, HYC_ERR_ARG, "bad field %d", field);
  Field &f = c->fields[field];
  if (!f.dev) return fail(c, HYC_ERR_FIELD, "field %d not bound", field);
  if (!f.host) return HYC_OK;  // device-bound: nothing to move
  DeviceGuard g(c->device);
  size_t bytes = (size_t)f.nelem * sizeof(double);
  if (to_device)
    CK(cudaMemcpyAsync(f.dev, f.host, bytes, cudaMemcpyHostToDevice, c->stream), "sync h2d");
  else
    CK(cudaMemcpyAsync(f.host, f.dev, bytes, cudaMemcpyDeviceToHost, c->stream), "sync d2h");
  return HYC_OK;
}

int hyc_xctilr(hyc_ctx *c, double *a, int32_t nlev, int32_t mh, int32_t nh, int32_t where) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!a || nlev < 1) return fail(c, HYC_ERR_ARG, "hyc_xctilr: bad arguments");
  DeviceGuard g(c->device);
  if (where == HYC_DEVICE) {
    Timed t(c, HYC_T_XCTILR);
    CK(hyc::launch_xctilr(a, c->slice, nlev, c->idm, c->jdm, c->nbdy, c->ld1, mh, nh, c->nreg, c->stream), "xctilr");
    c->stats.launches += (nlev + 65534) / 65535;
    return HYC_OK;
  }
  // host array: stage one slice at a time through the staging buffer
  if (!c->d_tmp) CK(cudaMalloc(&c->d_tmp, 8 * c->slice * sizeof(double)), "malloc staging");
  for (int l = 0; l < nlev; l++) {
    double *h = a + (long long)l * c->slice;
    CK(cudaMemcpyAsync(c->d_tmp, h, c->slice * 8, cudaMemcpyHostToDevice, c->stream), "h2d");
    CK(hyc::launch_xctilr(c->d_tmp, c->slice, 1, c->idm, c->jdm, c->nbdy, c->ld1, mh, nh, c->nreg, c->stream),
       "xctilr");
    c->stats.launches += 1;
    CK(cudaMemcpyAsync(h, c->d_tmp, c->slice * 8, cudaMemcpyDeviceToHost, c->stream), "d2h");
  }
  CK(cudaStreamSynchronize(c->stream), "xctilr sync");
  return HYC_OK;
}

int hyc_advem(hyc_ctx *c, int32_t advtyp, double *fld, const double *fldc, const double *u, const double *v,
              const double *fco, const double *fcn, double posdef, const double *scal, const double *scali, double dt2,
              int32_t btrmas, int32_t where) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!valid_advtyp(advtyp)) return fail(c, HYC_ERR_ADVTYP, "advem called with advtyp = %d", advtyp);
  if (c->nbdy < kMbdy[advtyp]) return fail(c, HYC_ERR_NBDY, "nbdy must be at least %d", kMbdy[advtyp]);
  if (!fld || !u || !v || !fco || !fcn || !scal || !scali || (advtyp >= 2 && !fldc))
    return fail(c, HYC_ERR_ARG, "hyc_advem: null array");
  if (where != HYC_HOST && where != HYC_DEVICE) return fail(c, HYC_ERR_ARG, "bad where");
  DeviceGuard g(c->device);
  const long long sl = c->slice;
  double *dfld = fld;
  const double *dfldc = fldc, *du = u, *dv = v, *dfco = fco, *dfcn = fcn, *dscal = scal, *dscali = scali;
  if (where == HYC_HOST) {
    if (!c->d_tmp) CK(cudaMalloc(&c->d_tmp, 8 * sl * sizeof(double)), "malloc staging");
    const double *src[8] = {fld, fldc ? fldc : fld, u, v, fco, fcn, scal, scali};
    for (int q = 0; q < 8; q++)
      CK(cudaMemcpyAsync(c->d_tmp + q * sl, src[q], sl * 8, cudaMemcpyHostToDevice, c->stream), "advem h2d");
    dfld = c->d_tmp;
    dfldc = c->d_tmp + sl;
    du = c->d_tmp + 2 * sl;
    dv = c->d_tmp + 3 * sl;
    dfco = c->d_tmp + 4 * sl;
    dfcn = c->d_tmp + 5 * sl;
    dscal = c->d_tmp + 6 * sl;
    dscali = c->d_tmp + 7 * sl;
  }
  if (advtyp == 2 && btrmas) {  // advem_fct2c, mod_tsadvc.F90:154-155
    if (c->lconserve)  // advem_fct2c forms no fldao/fldan (mod_tsadvc.F90:999-1368)
      return fail(c, HYC_ERR_UNSUPPORTED, "lconserve with advem_fct2c (btrmas) is not supported");
    if (c->nreg < 0)
      return fail(c, HYC_ERR_UNSUPPORTED, "advem_fct2c refreshes halos in mid-scheme: not with external halos");
    int rc = ensure_fct2c(c, hyc::fct2c_work_bytes(sl));
    if (rc) return rc;
    hyc::Fct2cArgs f;
    memset(&f, 0, sizeof f);
    f.ii = c->idm;
    f.jj = c->jdm;
    f.nb = c->nbdy;
    f.ld1 = c->ld1;
    f.ld2 = c->ld2;
    f.slice = sl;
    f.mode = 1;
    f.msk = c->d_msk;
    f.scal = dscal;
    f.scali = dscali;
    f.uflx = du;
    f.vflx = dv;
    f.fco = dfco;
    f.fcn = dfcn;
    f.dt2 = dt2;
    fct2c_bind(f, c, 1);
    f.fld[0] = dfld;
    f.fldc[0] = dfldc;
    f.k[0] = 0;
    int nl = 0;
    {
      Timed t(c, HYC_T_ADVECT);
      CK(hyc::launch_fct2c(f, c->nreg, &nl, c->stream), "advem_fct2c");
    }
    c->stats.launches += nl;
    if (where == HYC_HOST)
      CK(cudaMemcpyAsync(fld, c->d_tmp, sl * 8, cudaMemcpyDeviceToHost, c->stream), "advem d2h");
    CK(cudaStreamSynchronize(c->stream), "advem");
    return HYC_OK;
  }
  int rc = ensure_scratch(c, (size_t)sl);
  if (rc) return rc;
  TileArgs a;
  memset(&a, 0, sizeof a);
  a.ii = c->idm;
  a.jj = c->jdm;
  a.nbdy = c->nbdy;
  a.ld1 = c->ld1;
  a.ld2 = c->ld2;
  a.slice = sl;
  a.ntx = (c->idm + c->shape.tx - 1) / c->shape.tx;
  a.nty = (c->jdm + c->shape.ty - 1) / c->shape.ty;
  a.mode = 1;
  a.msk = c->d_msk;
  a.scal = dscal;
  a.scali = dscali;
  a.uflx = du;
  a.vflx = dv;
  a.fco = dfco;
  a.fcn = dfcn;
  a.dt2 = dt2;
  a.nfld = 1;
  a.f[0].nbase = dfld;
  a.f[0].mbase = dfldc ? dfldc : dfld;
  a.f[0].k_off = 0;
  a.f[0].kmin = 1;
  a.f[0].kmax = 1;
  a.f[0].posdef = posdef;
  a.out = c->d_scratch;
  a.kdm = 1;
  a.err = c->d_err;
  if (hyc::advect_tiles_tma(advtyp, c->shape)) {  // the tile kernel stages by TMA
    TileMaps tmv;
    const long m0 = tile_maps_add(c, a, 1, true, tmv);
    if (m0 >= 0) {
      if ((rc = tile_maps_upload(c, tmv))) return rc;
      a.tmaps = c->d_tmaps + m0;
      a.tm_has3 = 1;  // fco
    }
  }
  {
    Timed t(c, HYC_T_ADVECT);
    CK(hyc::launch_advect_tiles(advtyp, a, 1, c->shape, c->stream), "advem kernel");
  }
  if (c->lconserve && (rc = conserve(c, a, 1))) return rc;
  CK(hyc::launch_copy_back(a, 1, c->stream), "advem copy");
  c->stats.launches += 2;
  if (where == HYC_HOST)
    CK(cudaMemcpyAsync(fld, c->d_tmp, sl * 8, cudaMemcpyDeviceToHost, c->stream), "advem d2h");
  CK(cudaStreamSynchronize(c->stream), "advem");
  return HYC_OK;
}

int hyc_tsadvc(hyc_ctx *c, int32_t m, int32_t n, const hyc_tsadvc_params *p, double *xmin, double *xmax) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!p || m < 1 || m > 2 || n < 1 || n > 2) return fail(c, HYC_ERR_ARG, "hyc_tsadvc: bad m/n/params");
  const int at = p->advtyp < 0 ? -p->advtyp : p->advtyp;
  if (!valid_advtyp(at)) return fail(c, HYC_ERR_ADVTYP, "advem called with advtyp = %d", p->advtyp);
  if (c->nbdy < kMbdy[at])
    return fail(c, HYC_ERR_NBDY, "nbdy (dimensions.h) must be at least %d for advtyp %d", kMbdy[at], at);
  if (p->isopyc && (p->nhybrd != 0 || p->hybrid))
    return fail(c, HYC_ERR_ARG, "isopycnic mode is nhybrd = 0 (no hybrid layers)");
  if (p->isopyc && at == 2 && p->btrmas)
    return fail(c, HYC_ERR_UNSUPPORTED, "isopycnic flux smoothing with advem_fct2c (btrmas) is not supported");
  if (c->lconserve && at == 2 && p->btrmas)  // advem_fct2c forms no fldao/fldan (mod_tsadvc.F90:999-1368)
    return fail(c, HYC_ERR_UNSUPPORTED, "lconserve with advem_fct2c (btrmas) is not supported");
  if (p->ntracr < 0 || (p->ntracr > 0 && !p->trcflg)) return fail(c, HYC_ERR_ARG, "ntracr/trcflg");
  const int kk = c->kdm;
  const long long sl = c->slice;
  Field *F = c->fields;
  auto need = [&](int id, int64_t nel, const char *name) -> int {
    if (!F[id].dev) return fail(c, HYC_ERR_FIELD, "field %s is not bound", name);
    if (F[id].nelem < nel) return fail(c, HYC_ERR_FIELD, "field %s has %lld elements, needs %lld", name,
                                       (long long)F[id].nelem, (long long)nel);
    return HYC_OK;
  };
  const bool use_temp = p->advflg == 0 && p->nhybrd >= 1;
  const bool use_th3d = p->advflg == 1 && p->hybrid && p->nhybrd >= 1;
  int rc;
  if ((rc = need(HYC_F_SALN, 2LL * kk * sl, "saln"))) return rc;
  if ((rc = need(HYC_F_UFLX, (long long)kk * sl, "uflx"))) return rc;
  if ((rc = need(HYC_F_VFLX, (long long)kk * sl, "vflx"))) return rc;
  if ((rc = need(HYC_F_DP, 2LL * kk * sl, "dp"))) return rc;
  if (use_temp && (rc = need(HYC_F_TEMP, 2LL * kk * sl, "temp"))) return rc;
  if ((use_th3d || p->isopyc) && (rc = need(HYC_F_TH3D, 2LL * kk * sl, "th3d"))) return rc;
  if (p->ntracr > 0 && (rc = need(HYC_F_TRACER, 2LL * kk * sl * p->ntracr, "tracer"))) return rc;
  if (p->mxlmy && ((rc = need(HYC_F_Q2, 2LL * (kk + 2) * sl, "q2")) || (rc = need(HYC_F_Q2L, 2LL * (kk + 2) * sl, "q2l"))))
    return rc;
  if (p->btrmas && (rc = need(HYC_F_ONETA, 2LL * sl, "oneta"))) return rc;
  if (p->btrmas && at == 2 && c->nreg < 0)
    return fail(c, HYC_ERR_UNSUPPORTED, "advem_fct2c refreshes halos in mid-scheme: not with external halos");
  DeviceGuard g(c->device);
  cudaStream_t s = c->stream;
  const int mm = m - 1, nn = n - 1;
  Timed t_all(c, HYC_T_TSADVC);

  // halo refresh, mod_tsadvc.F90:1827-1840 (dp halo is up to date on entry)
  const int l = kMbdy[at];
  auto halo = [&](int id, int nlev) -> cudaError_t {
    if (!F[id].dev) return cudaSuccess;
    c->stats.launches += (nlev + 65534) / 65535;
    return hyc::launch_xctilr(F[id].dev, sl, nlev, c->idm, c->jdm, c->nbdy, c->ld1, l, l, c->nreg, s);
  };
  {
  Timed t_halo(c, HYC_T_XCTILR);
  CK(halo(HYC_F_SALN, 2 * kk), "xctilr saln");
  CK(halo(HYC_F_TEMP, 2 * kk), "xctilr temp");
  CK(halo(HYC_F_TH3D, 2 * kk), "xctilr th3d");
  CK(halo(HYC_F_UFLX, kk), "xctilr uflx");
  CK(halo(HYC_F_VFLX, kk), "xctilr vflx");
  if (p->ntracr > 0) {
    c->stats.launches += (2 * kk * p->ntracr + 65534) / 65535;
    CK(hyc::launch_xctilr(F[HYC_F_TRACER].dev, sl, 2 * kk * p->ntracr, c->idm, c->jdm, c->nbdy, c->ld1, l, l,
                          c->nreg, s), "xctilr tracer");
  }
  if (p->mxlmy) {
    CK(halo(HYC_F_Q2, 2 * kk + 4), "xctilr q2");
    CK(halo(HYC_F_Q2L, 2 * kk + 4), "xctilr q2l");
  }
  }

  // field list in the reference's call order (mod_tsadvc.F90:1969-2048)
  std::vector<FieldDesc> fl;
  auto add = [&](double *base, long long lev, int koff, int kmin, int kmax, double posdef) {
    FieldDesc d;
    memset(&d, 0, sizeof d);
    d.nbase = base + (long long)nn * lev;
    d.mbase = base + (long long)mm * lev;
    d.k_off = koff;
    d.kmin = kmin;
    d.kmax = kmax;
    d.posdef = posdef;
    fl.push_back(d);
  };
  const double pdzero = 0.0, pdtemp = 256.0, pdth3d = 32.0, pdq2 = 1.0;  // :1761-1763
  const int nh = p->nhybrd < kk ? p->nhybrd : kk;
  // isopycnic mode (:1855-1859, :1983-1991): layer 1 advects th3d and saln
  // with the smoothed fluxes; the tracers (and q2, q2l) of layer 1 keep
  // the layer's own fluxes but share its thickness factors, which come
  // from the smoothed ones; deeper layers advect saln (and the tracers)
  // only.  iso1 = fields of layer 1 advected by the smoothed fluxes,
  // isot = the rest of layer 1; fl = every field of layers >= 2.
  std::vector<FieldDesc> iso1, isot;
  const int k1 = p->isopyc ? 2 : 1;  // first layer of the general launch
  if (use_temp) add(F[HYC_F_TEMP].dev, (long long)kk * sl, 0, 1, nh, pdtemp);
  if (use_th3d) add(F[HYC_F_TH3D].dev, (long long)kk * sl, 0, 1, nh, pdth3d);
  if (p->isopyc) {
    add(F[HYC_F_TH3D].dev, (long long)kk * sl, 0, 1, 1, pdth3d);
    add(F[HYC_F_SALN].dev, (long long)kk * sl, 0, 1, 1, pdzero);
    iso1.swap(fl);
  }
  add(F[HYC_F_SALN].dev, (long long)kk * sl, 0, k1, kk, pdzero);
  for (int t = 0; t < p->ntracr; t++)
    add(F[HYC_F_TRACER].dev + (long long)t * 2 * kk * sl, (long long)kk * sl, 0, 1, kk,
        p->trcflg[t] == 2 ? pdtemp : pdzero);
  if (p->mxlmy) {
    add(F[HYC_F_Q2].dev, (long long)(kk + 2) * sl, 1, 1, kk, pdq2);
    add(F[HYC_F_Q2L].dev, (long long)(kk + 2) * sl, 1, 1, kk, pdq2);
  }
  if (p->isopyc)  // split the tracers (and q2, q2l) at layer 1
    for (auto &d : fl)
      if (d.kmin == 1) {
        FieldDesc e = d;
        e.kmax = 1;
        isot.push_back(e);
        d.kmin = 2;
      }

  TileArgs a;
  memset(&a, 0, sizeof a);
  a.ii = c->idm;
  a.jj = c->jdm;
  a.nbdy = c->nbdy;
  a.ld1 = c->ld1;
  a.ld2 = c->ld2;
  a.slice = sl;
  a.ntx = (c->idm + c->shape.tx - 1) / c->shape.tx;
  a.nty = (c->jdm + c->shape.ty - 1) / c->shape.ty;
  a.mode = 0;
  a.msk = c->d_msk;
  a.scal = c->d_scp2;
  a.scali = c->d_scp2i;
  a.uflx = F[HYC_F_UFLX].dev;
  a.vflx = F[HYC_F_VFLX].dev;
  a.dpn = F[HYC_F_DP].dev + (long long)nn * kk * sl;
  a.oneta_n = p->btrmas ? F[HYC_F_ONETA].dev + (long long)nn * sl : nullptr;
  a.dt2 = p->delt1;
  a.kdm = kk;
  if (at == 2 && p->btrmas) {  // advem_fct2c per (field, layer), mod_tsadvc.F90:154-155
    std::vector<std::pair<int, int>> pairs;  // (layer, field) in the reference's call order
    for (int k = 0; k < kk; k++)
      for (int q = 0; q < (int)fl.size(); q++)
        if (k + 1 >= fl[q].kmin && k + 1 <= fl[q].kmax) pairs.push_back({k, q});
    const int nb = fct2c_batch(c);
    if ((rc = ensure_fct2c(c, (size_t)nb * hyc::fct2c_work_bytes(sl)))) return rc;
    hyc::Fct2cArgs f;
    memset(&f, 0, sizeof f);
    f.ii = c->idm;
    f.jj = c->jdm;
    f.nb = c->nbdy;
    f.ld1 = c->ld1;
    f.ld2 = c->ld2;
    f.slice = sl;
    f.mode = 0;
    f.msk = c->d_msk;
    f.scal = c->d_scp2;
    f.scali = c->d_scp2i;
    f.uflx = F[HYC_F_UFLX].dev;
    f.vflx = F[HYC_F_VFLX].dev;
    f.dpn = a.dpn;
    f.oneta = a.oneta_n;
    f.dt2 = p->delt1;
    for (size_t p0 = 0; p0 < pairs.size(); p0 += nb) {
      const int np = (int)std::min(pairs.size() - p0, (size_t)nb);
      fct2c_bind(f, c, np);
      for (int i = 0; i < np; i++) {
        const int k = pairs[p0 + i].first;
        const FieldDesc &d = fl[pairs[p0 + i].second];
        f.k[i] = k;
        f.fld[i] = d.nbase + (long long)(k + d.k_off) * sl;
        f.fldc[i] = d.mbase + (long long)(k + d.k_off) * sl;
      }
      int nl = 0;
      {
        Timed t(c, HYC_T_ADVECT);
        CK(hyc::launch_fct2c(f, c->nreg, &nl, s), "advem_fct2c");
      }
      c->stats.launches += nl;
    }
    fl.clear();  // done: no tile launches below
  }
  const int chunk = hyc::kMaxFields;
  const size_t most = std::max(fl.size(), std::max(iso1.size(), isot.size()));
  const int nchunk0 = (int)most < chunk ? (int)most : chunk;
  if (most > 0 && (rc = ensure_scratch(c, (size_t)nchunk0 * kk * sl))) return rc;
  a.out = c->d_scratch;
  a.err = c->d_err;
  // the tile launches of this call: each group of fields over layers
  // 1..nlay in chunks of kMaxFields, with the TMA maps of the FCT kernel
  struct Launch {
    TileArgs a;
    int nlay;
    long map0;  // first TMA map, -1: plain loads
  };
  std::vector<Launch> launches;
  TileMaps tmv;
  const bool fct = hyc::advect_tiles_tma(at, c->shape);  // the tile kernel stages by TMA
  auto plan = [&](const std::vector<FieldDesc> &grp, int nlay, bool flux1) {
    for (size_t f0 = 0; f0 < grp.size(); f0 += chunk) {
      Launch L{a, nlay, -1};
      L.a.nfld = (int)(grp.size() - f0) < chunk ? (int)(grp.size() - f0) : chunk;
      for (int q = 0; q < L.a.nfld; q++) L.a.f[q] = grp[f0 + q];
      if (fct) L.map0 = tile_maps_add(c, L.a, kk, flux1, tmv);
      launches.push_back(L);
    }
  };
  double *us = nullptr, *vs = nullptr;
  if (p->isopyc && (!iso1.empty() || !isot.empty())) {  // layer 1, :1860-1897
    if (!c->d_iso) CK(cudaMalloc(&c->d_iso, 2 * sl * sizeof(double)), "malloc isopycnic fluxes");
    us = c->d_iso;
    vs = c->d_iso + sl;
    a.uflx = us;  // layer 1 of the launch reads uflx + 0*slice
    a.vflx = vs;
    plan(iso1, 1, true);
    a.uflx = F[HYC_F_UFLX].dev;
    a.vflx = F[HYC_F_VFLX].dev;
    a.ufco = us;
    a.vfco = vs;
    plan(isot, 1, false);
    a.ufco = nullptr;
    a.vfco = nullptr;
  }
  plan(fl, kk, false);
  if ((rc = tile_maps_upload(c, tmv))) return rc;
  if (us) {
    CK(hyc::launch_iso_smooth(F[HYC_F_UFLX].dev, F[HYC_F_VFLX].dev, c->d_msk, sl, c->idm, c->jdm, c->nbdy, c->ld1,
                              kMbdy[at] - 1, us, vs, s),
       "isopycnic smoothing");
    c->stats.launches += 1;
  }
  for (Launch &L : launches) {
    if (L.map0 >= 0) {
      L.a.tmaps = c->d_tmaps + L.map0;
      L.a.tm_has3 = L.a.oneta_n != nullptr;
    }
    {
      Timed t(c, HYC_T_ADVECT);
      CK(hyc::launch_advect_tiles(at, L.a, L.nlay, c->shape, s), "advect kernel");
      int rc2;
      if (c->lconserve && (rc2 = conserve(c, L.a, L.nlay))) return rc2;
    }
    {
      Timed t(c, HYC_T_COPY);
      CK(hyc::launch_copy_back(L.a, L.nlay, s), "copy back");
    }
    c->stats.launches += 2;
  }

  // salinity range diagnostic, mod_tsadvc.F90:2065-2084
  if (xmin && xmax && (p->nstep % 3 == 0 || p->diagno)) {
    for (int k = 0; k < kk; k++) {
      c->h_keys[k] = hyc::double_to_key(999.);
      c->h_keys[kk + k] = hyc::double_to_key(-999.);
    }
    CK(cudaMemcpyAsync(c->d_keys, c->h_keys, 2 * kk * sizeof(long long), cudaMemcpyHostToDevice, s), "keys h2d");
    {
      Timed t(c, HYC_T_DIAG);
      CK(hyc::launch_saln_range(F[HYC_F_SALN].dev + (long long)nn * kk * sl, a.dpn, c->d_msk, sl, kk, c->idm,
                                c->jdm, c->nbdy, c->ld1, c->d_keys, s), "saln range");
    }
    c->stats.launches += 1;
    CK(cudaMemcpyAsync(c->h_keys, c->d_keys, 2 * kk * sizeof(long long), cudaMemcpyDeviceToHost, s), "keys d2h");
    CK(cudaStreamSynchronize(s), "saln range sync");
    for (int k = 0; k < kk; k++) {
      xmin[k] = hyc::key_to_double(c->h_keys[k]);
      xmax[k] = hyc::key_to_double(c->h_keys[kk + k]);
    }
  }
  return HYC_OK;
}

int hyc_set_diffusion_grid(hyc_ctx *c, const double *aspux, const double *aspvy, const double *scuy,
                           const double *scvx) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!aspux || !aspvy || !scuy || !scvx) return fail(c, HYC_ERR_ARG, "hyc_set_diffusion_grid: null array");
  DeviceGuard g(c->device);
  const size_t sl = (size_t)c->slice;
  if (!c->d_diff) CK(cudaMalloc(&c->d_diff, 4 * sl * sizeof(double)), "malloc diffusion grid");
  const double *src[4] = {aspux, aspvy, scuy, scvx};
  for (int q = 0; q < 4; q++)
    CK(cudaMemcpyAsync(c->d_diff + q * sl, src[q], sl * 8, cudaMemcpyHostToDevice, c->stream), "diffusion grid");
  CK(cudaStreamSynchronize(c->stream), "diffusion grid sync");
  return HYC_OK;
}

int hyc_tsdff(hyc_ctx *c, int32_t m, int32_t n, const hyc_tsadvc_params *p, double temdf2, double temdfc,
              double thbase) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!p || m < 1 || m > 2 || n < 1 || n > 2) return fail(c, HYC_ERR_ARG, "hyc_tsdff: bad m/n/params");
  if (!(temdf2 > 0.0)) return HYC_OK;  // mod_tsadvc.F90:2138
  if (p->isopyc) return fail(c, HYC_ERR_UNSUPPORTED, "isopycnic (nhybrd=0) mode is not supported");
  if (temdfc != 1.0)
    return fail(c, HYC_ERR_UNSUPPORTED, "temdfc = %g: only temdfc = 1 (temperature diffusion) is supported", temdfc);
  const int kk = c->kdm;
  if (p->nhybrd < kk)
    return fail(c, HYC_ERR_UNSUPPORTED, "nhybrd = %d < kdm: exactly isopycnal layers are not supported", p->nhybrd);
  if (p->ntracr < 0) return fail(c, HYC_ERR_ARG, "ntracr");
  if (!c->d_diff) return fail(c, HYC_ERR_FIELD, "hyc_tsdff: call hyc_set_diffusion_grid first");
  const long long sl = c->slice;
  Field *F = c->fields;
  auto need = [&](int id, int64_t nel, const char *name) -> int {
    if (!F[id].dev) return fail(c, HYC_ERR_FIELD, "field %s is not bound", name);
    if (F[id].nelem < nel) return fail(c, HYC_ERR_FIELD, "field %s has %lld elements, needs %lld", name,
                                       (long long)F[id].nelem, (long long)nel);
    return HYC_OK;
  };
  int rc;
  if ((rc = need(HYC_F_TEMP, 2LL * kk * sl, "temp")) || (rc = need(HYC_F_SALN, 2LL * kk * sl, "saln")) ||
      (rc = need(HYC_F_TH3D, 2LL * kk * sl, "th3d")) || (rc = need(HYC_F_DP, 2LL * kk * sl, "dp")) ||
      (rc = need(HYC_F_ONETA, 2LL * sl, "oneta")))
    return rc;
  if (p->ntracr > 0 && (rc = need(HYC_F_TRACER, 2LL * kk * sl * p->ntracr, "tracer"))) return rc;
  if (p->mxlmy && ((rc = need(HYC_F_Q2, 2LL * (kk + 2) * sl, "q2")) || (rc = need(HYC_F_Q2L, 2LL * (kk + 2) * sl, "q2l"))))
    return rc;
  DeviceGuard g(c->device);
  cudaStream_t s = c->stream;
  const int nn = n - 1;
  Timed t_all(c, HYC_T_TSDFF);
  // level n of every diffused field, halo 2 (:2139-2152)
  const int mdf = 2;
  std::vector<std::pair<double *, int>> halos = {{F[HYC_F_SALN].dev + (long long)nn * kk * sl, kk},
                                                 {F[HYC_F_TEMP].dev + (long long)nn * kk * sl, kk},
                                                 {F[HYC_F_TH3D].dev + (long long)nn * kk * sl, kk}};
  if (p->mxlmy) {
    halos.push_back({F[HYC_F_Q2].dev + (long long)nn * (kk + 2) * sl, kk + 2});
    halos.push_back({F[HYC_F_Q2L].dev + (long long)nn * (kk + 2) * sl, kk + 2});
  }
  for (int t = 0; t < p->ntracr; t++)
    halos.push_back({F[HYC_F_TRACER].dev + ((long long)t * 2 * kk + (long long)nn * kk) * sl, kk});
  {
    Timed t(c, HYC_T_XCTILR);
    for (auto &h : halos) {
      CK(hyc::launch_xctilr(h.first, sl, h.second, c->idm, c->jdm, c->nbdy, c->ld1, mdf, mdf, c->nreg, s), "xctilr");
      c->stats.launches += (h.second + 65534) / 65535;
    }
  }
  // the diffused fields, layer 1 of level n; temp and saln first (they give th3d)
  std::vector<double *> fl = {F[HYC_F_TEMP].dev + (long long)nn * kk * sl, F[HYC_F_SALN].dev + (long long)nn * kk * sl};
  if (p->mxlmy) {
    fl.push_back(F[HYC_F_Q2].dev + ((long long)nn * (kk + 2) + 1) * sl);
    fl.push_back(F[HYC_F_Q2L].dev + ((long long)nn * (kk + 2) + 1) * sl);
  }
  for (int t = 0; t < p->ntracr; t++) fl.push_back(F[HYC_F_TRACER].dev + ((long long)t * 2 * kk + (long long)nn * kk) * sl);
  const int chunk = hyc::kMaxFields;
  const int nchunk0 = (int)fl.size() < chunk ? (int)fl.size() : chunk;
  if ((rc = ensure_scratch(c, (size_t)nchunk0 * kk * sl))) return rc;
  hyc::TsdffArgs a;
  memset(&a, 0, sizeof a);
  a.ii = c->idm;
  a.jj = c->jdm;
  a.nb = c->nbdy;
  a.ld1 = c->ld1;
  a.ld2 = c->ld2;
  a.slice = sl;
  a.msk = c->d_msk;
  a.scp2 = c->d_scp2;
  a.aspux = c->d_diff;
  a.aspvy = c->d_diff + sl;
  a.scuy = c->d_diff + 2 * sl;
  a.scvx = c->d_diff + 3 * sl;
  a.oneta = F[HYC_F_ONETA].dev + (long long)nn * sl;
  a.dpn = F[HYC_F_DP].dev + (long long)nn * kk * sl;
  a.temdf2 = temdf2;
  a.delt1 = p->delt1;
  a.thbase = thbase;
  a.kdm = kk;
  a.out = c->d_scratch;
  a.th3d = F[HYC_F_TH3D].dev + (long long)nn * kk * sl;
  for (size_t f0 = 0; f0 < fl.size(); f0 += chunk) {
    a.nfld = (int)std::min(fl.size() - f0, (size_t)chunk);
    for (int q = 0; q < a.nfld; q++) a.fld[q] = fl[f0 + q];
    a.eos_t = f0 == 0 ? 0 : -1;
    a.eos_s = f0 == 0 ? 1 : -1;
    CK(hyc::launch_tsdff(a, s), "tsdff");
    c->stats.launches += 2;
  }
  return HYC_OK;
}

namespace {

// Bind the arrays of the Robert-Asselin filter; checks what the switches need.
int asselin_args(hyc_ctx *c, int m, int n, const hyc_tsadvc_params *p, bool filter, hyc::AsselinArgs &a) {
  if (!p || m < 1 || m > 2 || n < 1 || n > 2) return fail(c, HYC_ERR_ARG, "asselin: bad m/n/params");
  if (p->ntracr < 0) return fail(c, HYC_ERR_ARG, "ntracr");
  const int kk = c->kdm;
  const long long sl = c->slice;
  Field *F = c->fields;
  auto need = [&](int id, int64_t nel, const char *name) -> int {
    if (!F[id].dev) return fail(c, HYC_ERR_FIELD, "field %s is not bound", name);
    if (F[id].nelem < nel) return fail(c, HYC_ERR_FIELD, "field %s has %lld elements, needs %lld", name,
                                       (long long)F[id].nelem, (long long)nel);
    return HYC_OK;
  };
  int rc;
  if ((rc = need(HYC_F_TEMP, 2LL * kk * sl, "temp")) || (rc = need(HYC_F_SALN, 2LL * kk * sl, "saln")) ||
      (rc = need(HYC_F_TH3D, 2LL * kk * sl, "th3d")) || (rc = need(HYC_F_ONETA, 2LL * sl, "oneta")) ||
      (rc = need(HYC_F_ONETAO, 2LL * sl, "onetao")) || (rc = need(HYC_F_PBAVG, 3LL * sl, "pbavg")) ||
      (rc = need(HYC_F_PBOT, sl, "pbot")) || (rc = need(HYC_F_OTEMP, (long long)kk * sl, "otemp")) ||
      (rc = need(HYC_F_OSALN, (long long)kk * sl, "osaln")))
    return rc;
  if (!filter && (rc = need(HYC_F_OTH3D, (long long)kk * sl, "oth3d"))) return rc;
  if (filter && ((rc = need(HYC_F_DP, 2LL * kk * sl, "dp")) || (rc = need(HYC_F_DPO, 2LL * kk * sl, "dpo"))))
    return rc;
  if (p->ntracr > 0 && ((rc = need(HYC_F_TRACER, 2LL * kk * sl * p->ntracr, "tracer")) ||
                        (rc = need(HYC_F_OTRACER, (long long)kk * sl * p->ntracr, "otracer"))))
    return rc;
  if (p->mxlmy && ((rc = need(HYC_F_Q2, 2LL * (kk + 2) * sl, "q2")) || (rc = need(HYC_F_Q2L, 2LL * (kk + 2) * sl, "q2l")) ||
                   (rc = need(HYC_F_OQ2, (long long)(kk + 2) * sl, "oq2")) ||
                   (rc = need(HYC_F_OQ2L, (long long)(kk + 2) * sl, "oq2l"))))
    return rc;
  memset(&a, 0, sizeof a);
  a.ii = c->idm;
  a.jj = c->jdm;
  a.nb = c->nbdy;
  a.ld1 = c->ld1;
  a.ld2 = c->ld2;
  a.slice = sl;
  a.kdm = kk;
  a.m = m;
  a.n = n;
  a.ntracr = p->ntracr;
  a.mxlmy = p->mxlmy ? 1 : 0;
  a.msk = c->d_msk;
  a.temp = F[HYC_F_TEMP].dev;
  a.saln = F[HYC_F_SALN].dev;
  a.th3d = F[HYC_F_TH3D].dev;
  a.tracer = F[HYC_F_TRACER].dev;
  a.q2 = F[HYC_F_Q2].dev;
  a.q2l = F[HYC_F_Q2L].dev;
  a.dp = F[HYC_F_DP].dev;
  a.dpo = F[HYC_F_DPO].dev;
  a.pbavg = F[HYC_F_PBAVG].dev;
  a.pbot = F[HYC_F_PBOT].dev;
  a.oneta = F[HYC_F_ONETA].dev;
  a.onetao = F[HYC_F_ONETAO].dev;
  a.otemp = F[HYC_F_OTEMP].dev;
  a.osaln = F[HYC_F_OSALN].dev;
  a.oth3d = F[HYC_F_OTH3D].dev;
  a.otracer = F[HYC_F_OTRACER].dev;
  a.oq2 = F[HYC_F_OQ2].dev;
  a.oq2l = F[HYC_F_OQ2L].dev;
  return HYC_OK;
}

}  // namespace

int hyc_asselin_save(hyc_ctx *c, int32_t m, int32_t n, const hyc_tsadvc_params *p, double oneta0) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  hyc::AsselinArgs a;
  int rc = asselin_args(c, m, n, p, false, a);
  if (rc) return rc;
  a.oneta0 = oneta0;
  DeviceGuard g(c->device);
  Timed t(c, HYC_T_ASSELIN);
  CK(hyc::launch_asselin(a, false, c->stream), "asselin_save");
  CK(hyc::launch_xctilr(a.oneta, c->slice, 2, c->idm, c->jdm, c->nbdy, c->ld1, 6, 6, c->nreg, c->stream),
     "xctilr oneta");
  CK(hyc::launch_xctilr(a.onetao, c->slice, 2, c->idm, c->jdm, c->nbdy, c->ld1, 6, 6, c->nreg, c->stream),
     "xctilr onetao");
  c->stats.launches += 3;
  return HYC_OK;
}

int hyc_asselin_filter(hyc_ctx *c, int32_t m, int32_t n, const hyc_tsadvc_params *p, double ra2fac, double oneta0,
                       double thbase) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (p && (p->advflg != 0 || p->isopyc))
    return fail(c, HYC_ERR_UNSUPPORTED, "asselin_filter: only advflg = 0 hybrid layers (no tofsig in the 17-term "
                                        "equation of state)");
  if (p && p->nhybrd < c->kdm)
    return fail(c, HYC_ERR_UNSUPPORTED, "asselin_filter: nhybrd = %d < kdm: exactly isopycnal layers need theta",
                p->nhybrd);
  hyc::AsselinArgs a;
  int rc = asselin_args(c, m, n, p, true, a);
  if (rc) return rc;
  a.oneta0 = oneta0;
  a.ra2fac = ra2fac;
  a.thbase = thbase;
  DeviceGuard g(c->device);
  Timed t(c, HYC_T_ASSELIN);
  CK(hyc::launch_asselin(a, true, c->stream), "asselin_filter");
  c->stats.launches += 1;
  return HYC_OK;
}

int hyc_set_cnuity_grid(hyc_ctx *c, const double *scuy, const double *scvx, const double *depthu, const double *depthv,
                        const double *thkdfu, const double *thkdfv) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!scuy || !scvx || !depthu || !depthv || (!thkdfu != !thkdfv))
    return fail(c, HYC_ERR_ARG, "hyc_set_cnuity_grid: null array");
  DeviceGuard g(c->device);
  const size_t sl = (size_t)c->slice;
  if (!c->d_cngrid) CK(cudaMalloc(&c->d_cngrid, 6 * sl * sizeof(double)), "malloc cnuity grid");
  const double *src[6] = {scuy, scvx, depthu, depthv, thkdfu, thkdfv};
  for (int q = 0; q < 6; q++)
    if (src[q])
      CK(cudaMemcpyAsync(c->d_cngrid + q * sl, src[q], sl * 8, cudaMemcpyHostToDevice, c->stream), "cnuity grid");
  CK(cudaStreamSynchronize(c->stream), "cnuity grid sync");
  c->cn_thkdf = thkdfu != nullptr;
  return HYC_OK;
}

int hyc_cnuity(hyc_ctx *c, int32_t m, int32_t n, const hyc_cnuity_params *p, double *dpkmin) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!p || m < 1 || m > 2 || n < 1 || n > 2) return fail(c, HYC_ERR_ARG, "hyc_cnuity: bad m/n/params");
  if (p->isopyc) return fail(c, HYC_ERR_UNSUPPORTED, "isopycnic (nhybrd=0) mode is not supported");
  if (p->thkdf != 0 && p->thkdf != 2 && p->thkdf != 4) return fail(c, HYC_ERR_ARG, "thkdf must be 0, 2 or 4");
  if (c->nbdy < 6) return fail(c, HYC_ERR_NBDY, "cnuity needs nbdy >= 6 (its halo is 6 wide)");
  if (!c->d_cngrid) return fail(c, HYC_ERR_FIELD, "hyc_cnuity: call hyc_set_cnuity_grid first");
  if (p->thkdf && !c->cn_thkdf) return fail(c, HYC_ERR_FIELD, "hyc_cnuity: interface diffusion without thkdfu/thkdfv");
  if (p->thkdf && c->nreg < 0)
    return fail(c, HYC_ERR_UNSUPPORTED, "the interface diffusion refreshes halos in mid-step: not with external halos");
  const int kk = c->kdm;
  const long long sl = c->slice;
  Field *F = c->fields;
  auto need = [&](int id, int64_t nel, const char *name) -> int {
    if (!F[id].dev) return fail(c, HYC_ERR_FIELD, "field %s is not bound", name);
    if (F[id].nelem < nel) return fail(c, HYC_ERR_FIELD, "field %s has %lld elements, needs %lld", name,
                                       (long long)F[id].nelem, (long long)nel);
    return HYC_OK;
  };
  int rc;
  if ((rc = need(HYC_F_DP, 2LL * kk * sl, "dp")) || (rc = need(HYC_F_DPO, 2LL * kk * sl, "dpo")) ||
      (rc = need(HYC_F_U, 2LL * kk * sl, "u")) || (rc = need(HYC_F_V, 2LL * kk * sl, "v")) ||
      (rc = need(HYC_F_DPU, 2LL * kk * sl, "dpu")) || (rc = need(HYC_F_DPV, 2LL * kk * sl, "dpv")) ||
      (rc = need(HYC_F_UBAVG, 3LL * sl, "ubavg")) || (rc = need(HYC_F_VBAVG, 3LL * sl, "vbavg")) ||
      (rc = need(HYC_F_PBOT, sl, "pbot")) || (rc = need(HYC_F_P, (long long)(kk + 1) * sl, "p")) ||
      (rc = need(HYC_F_UFLX, (long long)kk * sl, "uflx")) || (rc = need(HYC_F_VFLX, (long long)kk * sl, "vflx")))
    return rc;
  if (p->btrmas && ((rc = need(HYC_F_ONETA, 2LL * sl, "oneta")) || (rc = need(HYC_F_ONETACNT, sl, "onetacnt"))))
    return rc;
  const bool cumul = F[HYC_F_UFLXAV].dev && F[HYC_F_VFLXAV].dev && F[HYC_F_DPAV].dev;
  if (cumul && ((rc = need(HYC_F_UFLXAV, (long long)kk * sl, "uflxav")) ||
                (rc = need(HYC_F_VFLXAV, (long long)kk * sl, "vflxav")) ||
                (rc = need(HYC_F_DPAV, (long long)kk * sl, "dpav"))))
    return rc;
  DeviceGuard g(c->device);
  cudaStream_t s = c->stream;
  const size_t nw = hyc::cnuity_work_slices();
  if (!c->d_cnw) {
    CK(cudaMalloc(&c->d_cnw, nw * sl * sizeof(double)), "malloc cnuity work");
    CK(cudaMemsetAsync(c->d_cnw, 0, nw * sl * sizeof(double), s), "cnuity work");
  }
  const bool want_keys = dpkmin || p->nstep % 3 == 0;
  if (want_keys) {
    if (!c->d_cnkeys) CK(cudaMalloc(&c->d_cnkeys, 2 * kk * sizeof(long long)), "malloc keys");
    std::vector<long long> k0(2 * kk, hyc::double_to_key(999.));  // dpmin = 999. (:296, :482)
    CK(cudaMemcpyAsync(c->d_cnkeys, k0.data(), k0.size() * sizeof(long long), cudaMemcpyHostToDevice, s), "keys");
  }
  Timed t_all(c, HYC_T_CNUITY);
  const int mm = m - 1;
  // halos, cnuity.F90:100-107 (dpmixl is not carried)
  struct H {
    double *a;
    int nlev;
  } halos[] = {{F[HYC_F_DP].dev, 2 * kk},
               {F[HYC_F_DPU].dev + (long long)mm * kk * sl, kk},
               {F[HYC_F_DPV].dev + (long long)mm * kk * sl, kk},
               {F[HYC_F_U].dev + (long long)mm * kk * sl, kk},
               {F[HYC_F_V].dev + (long long)mm * kk * sl, kk},
               {F[HYC_F_UBAVG].dev + (long long)mm * sl, 1},
               {F[HYC_F_VBAVG].dev + (long long)mm * sl, 1}};
  for (auto &h : halos) {
    CK(hyc::launch_xctilr(h.a, sl, h.nlev, c->idm, c->jdm, c->nbdy, c->ld1, 6, 6, c->nreg, s), "xctilr");
    c->stats.launches += 1;
  }
  hyc::CnuityArgs a;
  memset(&a, 0, sizeof a);
  a.ii = c->idm;
  a.jj = c->jdm;
  a.nb = c->nbdy;
  a.ld1 = c->ld1;
  a.ld2 = c->ld2;
  a.nreg = c->nreg;
  a.slice = sl;
  a.kdm = kk;
  a.m = m;
  a.n = n;
  a.nstep = p->nstep;
  a.btrmas = p->btrmas ? 1 : 0;
  a.thk = p->thkdf;
  a.msk = c->d_msk;
  a.scp2 = c->d_scp2;
  a.scp2i = c->d_scp2i;
  a.scuy = c->d_cngrid;
  a.scvx = c->d_cngrid + sl;
  a.depthu = c->d_cngrid + 2 * sl;
  a.depthv = c->d_cngrid + 3 * sl;
  a.thkdfu = c->d_cngrid + 4 * sl;
  a.thkdfv = c->d_cngrid + 5 * sl;
  a.pbot = F[HYC_F_PBOT].dev;
  a.oneta = F[HYC_F_ONETA].dev;
  a.u = F[HYC_F_U].dev;
  a.v = F[HYC_F_V].dev;
  a.dpu = F[HYC_F_DPU].dev;
  a.dpv = F[HYC_F_DPV].dev;
  a.ubavg = F[HYC_F_UBAVG].dev;
  a.vbavg = F[HYC_F_VBAVG].dev;
  a.dp = F[HYC_F_DP].dev;
  a.dpo = F[HYC_F_DPO].dev;
  a.p = F[HYC_F_P].dev;
  a.uflx = F[HYC_F_UFLX].dev;
  a.vflx = F[HYC_F_VFLX].dev;
  if (cumul) {
    a.uflxav = F[HYC_F_UFLXAV].dev;
    a.vflxav = F[HYC_F_VFLXAV].dev;
    a.dpav = F[HYC_F_DPAV].dev;
  }
  a.onetacnt = F[HYC_F_ONETACNT].dev;
  a.delt1 = p->delt1;
  a.dtinv = 1. / p->delt1;  // cnuity.F90:758, :987 (the same IEEE quotient as on the device)
  a.ra2fac = p->ra2fac;
  a.w = c->d_cnw;
  a.keys = want_keys ? c->d_cnkeys : nullptr;
  int nl = 0;
  CK(hyc::launch_cnuity_layers(a, &nl, s), "cnuity loop 76");
  std::vector<long long> keys(want_keys ? 2 * kk : 0);
  if (want_keys) {
    CK(cudaMemcpyAsync(keys.data(), c->d_cnkeys, keys.size() * sizeof(long long), cudaMemcpyDeviceToHost, s), "keys");
    CK(cudaStreamSynchronize(s), "keys sync");
    if (dpkmin)
      for (int k = 0; k < 2 * kk; k++) dpkmin[k] = hyc::key_to_double(keys[k]);
  }
  if (p->nstep % 3 == 0) {  // cnuity.F90:574-580
    const double onem = 9.806 / (1.0 / 1000.0), dpfatal = -10.0;
    double mn = hyc::key_to_double(keys[kk]);
    for (int k = kk + 1; k < 2 * kk; k++) mn = std::min(mn, hyc::key_to_double(keys[k]));
    if (mn < dpfatal * onem) {
      c->stats.launches += nl;
      return fail(c, HYC_ERR_NEGDP, "cnuity: neg. dp (m) < %g (minimum %g m)", dpfatal, mn / onem);
    }
  }
  CK(hyc::launch_cnuity_rest(a, &nl, s), "cnuity");
  c->stats.launches += nl;
  return HYC_OK;
}

int hyc_mass_sum(hyc_ctx *c, const double *fld, const double *fc, double *sum) {
  if (!c) return fail(nullptr, HYC_ERR_ARG, "null ctx");
  if (!fld || !fc || !sum) return fail(c, HYC_ERR_ARG, "hyc_mass_sum: null pointer");
  DeviceGuard g(c->device);
  double *partial = c->d_sum, *res = c->d_sum + 2 * hyc::mass_sum_partials();
  CK(hyc::launch_mass_sum(fld, fc, c->d_scp2, c->d_msk, c->idm, c->jdm, c->nbdy, c->ld1, partial, res, c->stream),
     "mass sum");
  c->stats.launches += 2;
  CK(cudaMemcpyAsync(c->h_sum, res, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "mass sum d2h");
  CK(cudaStreamSynchronize(c->stream), "mass sum sync");
  *sum = c->h_sum[0];
  return HYC_OK;
}

}  // extern "C"
