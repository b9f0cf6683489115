// hyc_ens_host.cpp -- host side of the ensemble (batched) form: storage,
// leapfrog level rotation, work queue, CUDA-graph capture and the tile-shape
// autotuner.  C ABI in include/hycom_adv.h (hyc_ens_*).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hycom_adv.h"
#include "hyc_args.h"
#include "hyc_ens.h"
#include "hyc_internal.h"
#include "hyc_tmap.h"

using hyc::MixBasin;
using hyc::TileArgs;

namespace {

struct EBasin {
  int idm, jdm, kdm, nbdy, nreg, ntr, ld1r, ld1, ld2;  // ld1r: reference pitch, ld1: ensemble pitch
  long long slice;
  uint8_t *msk = nullptr;
  double *scp2 = nullptr, *scp2i = nullptr;
  void *uflx = nullptr, *vflx = nullptr;  // FP32 (mixed) or FP64
  double *dp = nullptr;
  void *lev[3] = {nullptr, nullptr, nullptr};  // tracer state, physical levels
  double *cell = nullptr;                       // strip kernel per-cell words (mixed form)
  float2 *gd = nullptr;                         // diffusion grid table of the strip kernel (mixed form)
  double temdf2 = 0.0;                          // lateral diffusion after each step (0: none)
  long long work = 0;                           // cells*layers*tracers, for queue ordering
  std::vector<double> posdef;                   // MPDATA offset per tracer (0 unless set)
};

}  // namespace

struct hyc_ens {
  int device = 0, prec = HYC_PREC_FP64, nsm = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaStream_t cap_stream = nullptr;  // graphs are recorded here, then launched on `stream`
  std::vector<EBasin> b;
  int rot = 0;           // logical OLD = lev[rot], CUR = lev[(rot+1)%3], NEW = lev[(rot+2)%3]
  bool primed = false;   // NEW level initialised (land and halo cells) from CUR
  hyc::TileShape shape{32, 16};
  bool prep64 = true;  // FP32-mixed: thickness prep in FP64 (else compensated FP32)
  int maxntr = 1;        // largest tracer count
  int strip_nq = 2;      // strip kernel: tracers per pass (1 or 2)
  bool diff = false;     // some basin diffuses its tracers after each step (mixed form)
  CUtensorMap *d_cmaps = nullptr;  // [nbasin][kMaps]: strip kernel maps (levels 0-2, u, v, dp, cell words)
  CUtensorMap *d_fmaps = nullptr;  // FP64 form: the FCT tile kernel's maps, 3 rotations x basins
  size_t fmaps_cap = 0;
  int *d_err = nullptr;            // device error flag (bounded waits that gave up)
  // device tables, one per rotation
  MixBasin *d_mix[3] = {nullptr, nullptr, nullptr};
  // the one-tracer launch of the strip kernel that advances an odd tracer
  // count's last tracer when the main launch takes the tracers in pairs
  MixBasin *d_mixt[3] = {nullptr, nullptr, nullptr};
  TileArgs *d_targs[3] = {nullptr, nullptr, nullptr};
  std::vector<TileArgs> h_targs[3];  // host copies (FP64 PCM/MPDATA run the plain tile kernel per basin)
  double tbl_dt2 = -1.0;
  int4 *d_items = nullptr;  // the main launch's items, then the one-tracer launch's
  int nitems = 0, nitems_t = 0;
  int items_nq = 0;         // tracers per pass the strip items were built for
  int items_tx = 0, items_ty = 0, items_layers = -1;
  int *d_head = nullptr;  // two queue counters per step slot (main and one-tracer launch)
  int nhead = 0;
  double *d_partial = nullptr;
  int npartial = 0;
  // put staging (reference layout, FP64), two buffers used in turn: a put's
  // host-to-device copy runs on in_stream while the previous put's halo and
  // repitch kernels (and the step) run on the ensemble's stream
  double *d_stage[2] = {nullptr, nullptr};
  size_t stage_bytes[2] = {0, 0};
  int stage_next = 0;
  bool stage_used[2] = {false, false};
  cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_used[2] = {nullptr, nullptr}, ev_entry = nullptr;
  cudaStream_t in_stream = nullptr;
  // get staging; hyc_ens_get_async copies it out on copy_stream so the
  // device-to-host transfer overlaps later puts (the link is full duplex)
  double *d_gstage = nullptr;
  size_t gstage_bytes = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_staged = nullptr, ev_gdone = nullptr;
  bool get_pending = false;
  // graph cache
  cudaGraphExec_t gexec = nullptr;
  int g_nsteps = 0, g_advtyp = -1, g_rot = -1, g_tx = 0, g_ty = 0;
  double g_dt = 0.0;
  // timers
  bool timing = false;
  struct Span {
    int slot;
    cudaEvent_t a, z;
  };
  std::vector<Span> pending;  // timed spans, folded into stats by hyc_ens_stats
  hyc_stats stats{};
  std::string err;
};

namespace {

int efail(hyc_ens *e, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (e) e->err = buf;
  hyc::set_library_error(buf);
  return code;
}

#define ECK(call, what)                                                                    \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return efail(e, HYC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
  } while (0)

struct Dev {
  int prev = -1;
  explicit Dev(int d) {
    cudaGetDevice(&prev);
    if (prev != d) cudaSetDevice(d);
  }
  ~Dev() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

size_t esz(const hyc_ens *e) { return e->prec == HYC_PREC_MIXED ? 4 : 8; }

// tx == 56 selects the two-column strip kernel (ty = rows per segment)
bool is_col2(hyc::TileShape t) { return t.tx == hyc::kCol2Strip; }
constexpr int kMaps = 8;  // strip kernel maps per basin

void free_all(hyc_ens *e) {
  for (auto &b : e->b) {
    cudaFree(b.msk);
    cudaFree(b.scp2);
    cudaFree(b.scp2i);
    cudaFree(b.uflx);
    cudaFree(b.vflx);
    cudaFree(b.dp);
    cudaFree(b.cell);
    cudaFree(b.gd);
    for (auto &l : b.lev) cudaFree(l);
  }
  for (int r = 0; r < 3; r++) {
    cudaFree(e->d_mix[r]);
    cudaFree(e->d_mixt[r]);
    cudaFree(e->d_targs[r]);
  }
  cudaFree(e->d_items);
  cudaFree(e->d_head);
  cudaFree(e->d_partial);
  if (e->in_stream) cudaStreamSynchronize(e->in_stream);
  if (e->copy_stream) cudaStreamSynchronize(e->copy_stream);
  for (int q = 0; q < 2; q++) {
    cudaFree(e->d_stage[q]);
    if (e->ev_copied[q]) cudaEventDestroy(e->ev_copied[q]);
    if (e->ev_used[q]) cudaEventDestroy(e->ev_used[q]);
  }
  if (e->ev_entry) cudaEventDestroy(e->ev_entry);
  cudaFree(e->d_gstage);
  if (e->ev_staged) cudaEventDestroy(e->ev_staged);
  if (e->ev_gdone) cudaEventDestroy(e->ev_gdone);
  if (e->copy_stream) cudaStreamDestroy(e->copy_stream);
  if (e->in_stream) cudaStreamDestroy(e->in_stream);
  cudaFree(e->d_cmaps);
  cudaFree(e->d_fmaps);
  cudaFree(e->d_err);
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  for (auto &p : e->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.z);
  }
}

// maps of the two-column strip kernel; they depend only on the allocations
int encode_strip_maps(hyc_ens *e) {
  const int bx = hyc::kCol2Box, by = hyc::kCol2Rows;
  std::vector<CUtensorMap> h(e->b.size() * kMaps);
  for (size_t i = 0; i < e->b.size(); i++) {
    EBasin &b = e->b[i];
    CUtensorMap *m = &h[i * kMaps];
    bool ok = true;
    // widths are the pitch: the padding columns are zeros, as out of range
    for (int l = 0; l < 3; l++)
      ok &= hyc::tmap_encode3(m + l, b.lev[l], 4, b.ld1, b.ld2, b.ld1, b.slice, (long long)b.ntr * b.kdm, bx, by);
    ok &= hyc::tmap_encode3(m + 3, b.uflx, 4, b.ld1, b.ld2, b.ld1, b.slice, b.kdm, bx, by);
    ok &= hyc::tmap_encode3(m + 4, b.vflx, 4, b.ld1, b.ld2, b.ld1, b.slice, b.kdm, bx, by);
    ok &= hyc::tmap_encode3(m + 5, b.dp, 8, b.ld1, b.ld2, b.ld1, b.slice, b.kdm, bx, by);
    ok &= hyc::tmap_encode3(m + 6, b.cell, 8, b.ld1, b.ld2, b.ld1, b.slice, 1, bx, by);
    if (b.gd) ok &= hyc::tmap_encode3(m + 7, b.gd, 8, b.ld1, b.ld2, b.ld1, b.slice, 1, bx, by);
    if (!ok) return efail(e, HYC_ERR_CUDA, "cuTensorMapEncodeTiled failed for the strip maps (basin %zu)", i);
  }
  ECK(cudaMemcpy(e->d_cmaps, h.data(), h.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice), "strip maps copy");
  return HYC_OK;
}

// Layers per work item of the two-column strip kernel: enough items for
// about 16 per resident warp over the whole ensemble (so the last wave of
// the queue is short), and no more than 8 layers per item unless the
// ensemble is small.
int col2_kchunk(const hyc_ens *e, const EBasin &) {
  long long cols = 0;  // (strip, segment, layer) units over the ensemble
  for (const auto &b : e->b) {
    const long long nstrip = (b.nbdy + b.idm - 4 + hyc::kCol2Strip - 1) / hyc::kCol2Strip;
    const long long nseg = (b.jdm + e->shape.ty - 1) / e->shape.ty;
    cols += nstrip * nseg * b.kdm;
  }
  const long long want = 16LL * e->nsm * 8;  // ~16 items per warp at 8 warps per SM
  long long kc = cols / std::max(want, 1LL);
  return (int)std::max(1LL, std::min(8LL, kc));
}

// device tables for the three rotations (rebuilt when delt1 changes)
int build_tables(hyc_ens *e, double dt2) {
  if (e->tbl_dt2 == dt2) return HYC_OK;
  ECK(cudaStreamSynchronize(e->stream), "tables sync");  // earlier steps may still read the tables
  const int nb = (int)e->b.size();
  if (e->prec == HYC_PREC_MIXED)
    for (auto &b : e->b) ECK(hyc::launch_cell_words(b.scp2i, b.msk, dt2, b.slice, b.cell, e->stream), "cell words");
  for (int r = 0; r < 3; r++) {
    const int lo = r, lc = (r + 1) % 3, ln = (r + 2) % 3;
    if (e->prec == HYC_PREC_MIXED) {
      std::vector<MixBasin> t(nb);
      for (int i = 0; i < nb; i++) {
        const EBasin &b = e->b[i];
        MixBasin &m = t[i];
        memset(&m, 0, sizeof m);
        m.ii = b.idm;
        m.jj = b.jdm;
        m.nbdy = b.nbdy;
        m.ld1 = b.ld1;
        m.ld2 = b.ld2;
        m.slice = b.slice;
        m.kdm = b.kdm;
        m.ntr = b.ntr;
        m.images = b.nreg == 1 ? std::min(5, b.nbdy) : 0;
        m.fnew = (float *)b.lev[ln];
        m.seg = e->shape.ty;
        m.kchunk = col2_kchunk(e, b);
        m.q0 = 0;
        if (e->items_nq == 2 && b.ntr > 1) m.ntr = b.ntr & ~1;  // pairs; an odd last tracer is the other launch's
        for (int q = 0; q < b.ntr && q < hyc::kMaxFields; q++) m.posdef[q] = (float)b.posdef[q];
        const CUtensorMap *c = e->d_cmaps + i * kMaps;
        m.c2_old = c + lo;
        m.c2_cur = c + lc;
        m.c2_u = c + 3;
        m.c2_v = c + 4;
        m.c2_dp = c + 5;
        m.c2_cg = c + 6;
        m.c2_gd = c + 7;
      }
      std::vector<MixBasin> tt(t);  // the one-tracer launch: each basin's last tracer
      for (int i = 0; i < nb; i++) {
        tt[i].q0 = e->b[i].ntr - 1;
        tt[i].ntr = 1;
      }
      ECK(cudaMemcpy(e->d_mix[r], t.data(), nb * sizeof(MixBasin), cudaMemcpyHostToDevice), "mix table");
      ECK(cudaMemcpy(e->d_mixt[r], tt.data(), nb * sizeof(MixBasin), cudaMemcpyHostToDevice), "mix table");
    } else {
      std::vector<TileArgs> t(nb);
      for (int i = 0; i < nb; i++) {
        const EBasin &b = e->b[i];
        TileArgs &a = t[i];
        memset(&a, 0, sizeof a);
        a.ii = b.idm;
        a.jj = b.jdm;
        a.nbdy = b.nbdy;
        a.ld1 = b.ld1;
        a.ld2 = b.ld2;
        a.slice = b.slice;
        a.ntx = (b.idm + e->shape.tx - 1) / e->shape.tx;
        a.nty = (b.jdm + e->shape.ty - 1) / e->shape.ty;
        a.mode = 0;
        a.msk = b.msk;
        a.scal = b.scp2;
        a.scali = b.scp2i;
        a.uflx = (const double *)b.uflx;
        a.vflx = (const double *)b.vflx;
        a.dpn = b.dp;
        a.dt2 = dt2;
        a.nfld = b.ntr;
        for (int q = 0; q < b.ntr; q++) {
          a.f[q].nbase = (double *)b.lev[lo] + (long long)q * b.kdm * b.slice;
          a.f[q].mbase = (const double *)b.lev[lc] + (long long)q * b.kdm * b.slice;
          a.f[q].k_off = 0;
          a.f[q].kmin = 1;
          a.f[q].kmax = b.kdm;
          a.f[q].posdef = b.posdef[q];
        }
        a.out = (double *)b.lev[ln];
        a.kdm = b.kdm;
        a.images = b.nreg == 1 ? std::min(5, b.nbdy) : 0;
      }
      // TMA maps of the FCT tile kernel (box tx+8 x ty+6): uflx, vflx, dp,
      // (no onetamas), scp2, scp2i, then levels t-1 and t of each tracer
      if (r == 0) {
        size_t need = 0;
        for (const auto &b : e->b) need += 3 * (6 + 2 * (size_t)b.ntr);
        if (e->fmaps_cap < need) {
          cudaFree(e->d_fmaps);
          e->d_fmaps = nullptr;
          e->fmaps_cap = 0;
          ECK(cudaMalloc(&e->d_fmaps, need * sizeof(CUtensorMap)), "fp64 tensor maps");
          e->fmaps_cap = need;
        }
      }
      {
        std::vector<CUtensorMap> h;
        size_t base = 0;  // the rotations' maps one after another
        for (int rr = 0; rr < r; rr++)
          for (const auto &b : e->b) base += 6 + 2 * (size_t)b.ntr;
        const int bx = e->shape.tx + 8, by = e->shape.ty + 6;
        size_t at = base;
        for (int i = 0; i < nb; i++) {
          const EBasin &b = e->b[i];
          const long long w = b.idm + 2LL * b.nbdy, hh = b.jdm + 2LL * b.nbdy;
          std::vector<CUtensorMap> m(6 + 2 * (size_t)b.ntr);
          bool ok = hyc::tmap_available();
          auto enc = [&](CUtensorMap *p, const void *ptr, long long nz) {
            ok = ok && hyc::tmap_encode3(p, ptr, 8, w, hh, b.ld1, b.slice, nz, bx, by);
          };
          enc(&m[0], b.uflx, b.kdm);
          enc(&m[1], b.vflx, b.kdm);
          enc(&m[2], b.dp, b.kdm);
          enc(&m[4], b.scp2, 1);
          enc(&m[5], b.scp2i, 1);
          for (int q = 0; q < b.ntr; q++) {
            enc(&m[6 + 2 * q], t[i].f[q].nbase, b.kdm);
            enc(&m[7 + 2 * q], t[i].f[q].mbase, b.kdm);
          }
          if (ok) {
            t[i].tmaps = e->d_fmaps + at;
            t[i].tm_has3 = 0;
          }
          t[i].err = e->d_err;
          h.insert(h.end(), m.begin(), m.end());
          at += m.size();
        }
        ECK(cudaMemcpy(e->d_fmaps + base, h.data(), h.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice),
            "fp64 tensor maps copy");
      }
      ECK(cudaMemcpy(e->d_targs[r], t.data(), nb * sizeof(TileArgs), cudaMemcpyHostToDevice), "fp64 table");
      e->h_targs[r] = t;
    }
  }
  e->tbl_dt2 = dt2;
  return HYC_OK;
}

// queue of work items, largest first (longest-processing-time order)
// tracers per pass of the strip kernel's main launch
int strip_pass(const hyc_ens *e) { return std::min(e->strip_nq, e->maxntr); }

int build_items(hyc_ens *e) {
  const bool per_layer = e->prec != HYC_PREC_MIXED;
  const int nqm = strip_pass(e);
  if (e->d_items && e->items_tx == e->shape.tx && e->items_ty == e->shape.ty && e->items_nq == nqm) return HYC_OK;
  struct W {
    long long work;
    int4 it;
  };
  std::vector<W> w, wt;  // main launch, one-tracer launch
  for (int i = 0; i < (int)e->b.size(); i++) {
    const EBasin &b = e->b[i];
    const int ntx = (b.idm + e->shape.tx - 1) / e->shape.tx, nty = (b.jdm + e->shape.ty - 1) / e->shape.ty;
    if (is_col2(e->shape)) {  // (basin, 56-column strip, segment, chunk of layers), all tracers
      // the layer chunks of a segment are queued together: the per-cell
      // words of the segment's rows are then read from DRAM about once
      // and from L2 by the other chunks
      // with pairs of tracers per pass, an odd count's last tracer goes to the
      // one-tracer launch instead of a pass that advances it twice
      const int nstrip = (b.nbdy + b.idm - 4 + hyc::kCol2Strip - 1) / hyc::kCol2Strip;
      const int kc = col2_kchunk(e, b), nkc = (b.kdm + kc - 1) / kc;
      const int trm = nqm == 2 ? (b.ntr & ~1) : b.ntr;
      const bool tail = nqm == 2 && (b.ntr & 1);
      for (int sg = 0; sg < nty; sg++)
        for (int kq = 0; kq < nkc; kq++)
          for (int st = 0; st < nstrip; st++) {
            const long long lay = std::min(b.kdm, (kq + 1) * kc) - kq * kc;
            if (trm > 0) w.push_back({lay * trm, make_int4(i, st, sg, kq)});
            if (tail) wt.push_back({lay, make_int4(i, st, sg, kq)});
          }
      continue;
    }
    for (int t = 0; t < ntx * nty; t++) {
      if (per_layer) {
        for (int k = 0; k < b.kdm; k++) w.push_back({(long long)b.ntr, make_int4(i, t, k, 0)});
      } else {
        w.push_back({(long long)b.kdm * b.ntr, make_int4(i, t, 0, 0)});
      }
    }
  }
  std::stable_sort(w.begin(), w.end(), [](const W &a, const W &c) { return a.work > c.work; });
  std::stable_sort(wt.begin(), wt.end(), [](const W &a, const W &c) { return a.work > c.work; });
  ECK(cudaStreamSynchronize(e->stream), "items sync");
  std::vector<int4> it;
  it.reserve(w.size() + wt.size());
  for (const auto &x : w) it.push_back(x.it);
  for (const auto &x : wt) it.push_back(x.it);
  cudaFree(e->d_items);
  e->d_items = nullptr;
  ECK(cudaMalloc(&e->d_items, std::max<size_t>(1, it.size()) * sizeof(int4)), "items");
  ECK(cudaMemcpy(e->d_items, it.data(), it.size() * sizeof(int4), cudaMemcpyHostToDevice), "items copy");
  e->nitems = (int)w.size();
  e->nitems_t = (int)wt.size();
  e->items_tx = e->shape.tx;
  e->items_ty = e->shape.ty;
  e->items_nq = nqm;
  e->tbl_dt2 = -1.0;  // ntx/nty in the tables depend on the shape
  return HYC_OK;
}

int ensure_heads(hyc_ens *e, int n) {
  if (e->nhead >= n) return HYC_OK;
  cudaFree(e->d_head);
  e->d_head = nullptr;
  ECK(cudaMalloc(&e->d_head, 2 * n * sizeof(int)), "queue heads");
  e->nhead = n;
  return HYC_OK;
}

// NEW level <- CUR level for every basin (land cells and halo of the spare level)
int prime(hyc_ens *e) {
  if (e->primed) return HYC_OK;
  const int lc = (e->rot + 1) % 3, ln = (e->rot + 2) % 3;
  for (auto &b : e->b)
    ECK(cudaMemcpyAsync(b.lev[ln], b.lev[lc], (size_t)b.ntr * b.kdm * b.slice * esz(e), cudaMemcpyDeviceToDevice,
                        e->stream),
        "prime");
  e->primed = true;
  return HYC_OK;
}

// one step's launches (queue reset + step kernel) for rotation r, head slot h
int enqueue_step(hyc_ens *e, int advtyp, int r, int h, cudaStream_t st) {
  ECK(cudaMemsetAsync(e->d_head + 2 * h, 0, 2 * sizeof(int), st), "queue reset");
  cudaError_t c = cudaSuccess;
  int launches = 1;
  if (e->prec == HYC_PREC_MIXED) {
    if (e->nitems > 0)
      c = hyc::launch_mix_col2(advtyp, e->d_mix[r], e->d_items, e->nitems, e->d_head + 2 * h, e->nsm, strip_pass(e),
                               e->prep64, e->diff, e->d_err, st);
    if (c == cudaSuccess && e->nitems_t > 0) {  // the odd counts' last tracers
      c = hyc::launch_mix_col2(advtyp, e->d_mixt[r], e->d_items + e->nitems, e->nitems_t, e->d_head + 2 * h + 1,
                               e->nsm, 1, e->prep64, e->diff, e->d_err, st);
      launches = (e->nitems > 0) + 1;
    }
  } else if (e->prec != HYC_PREC_MIXED && (advtyp == 0 || advtyp == 1)) {
    // FP64 PCM/MPDATA: the plain form's tile kernel per basin, then the periodic halo
    c = cudaSuccess;
    for (size_t i = 0; i < e->b.size() && c == cudaSuccess; i++) {
      const EBasin &b = e->b[i];
      c = hyc::launch_advect_tiles(advtyp, e->h_targs[r][i], b.kdm, e->shape, st);
      if (c == cudaSuccess && b.nreg == 1)
        c = hyc::launch_xctilr((double *)b.lev[(r + 2) % 3], b.slice, b.ntr * b.kdm, b.idm, b.jdm, b.nbdy, b.ld1,
                               std::min(5, b.nbdy), std::min(5, b.nbdy), b.nreg, st);
    }
  }
  else
    c = hyc::launch_fct_queue(advtyp, e->shape, e->d_targs[r], e->d_items, e->nitems, e->d_head + 2 * h, e->nsm,
                              st);
  if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "step kernel: %s", cudaGetErrorString(c));
  e->stats.launches += launches;
  return HYC_OK;
}

// Schemes per form and kernel: FP64 FCT2/FCT4 (queue kernel) and PCM/MPDATA
// (plain tile kernel); FP32-mixed FCT2, FCT4 and MPDATA (strip kernel).
bool scheme_ok(const hyc_ens *e, int advtyp) {
  if (e->prec == HYC_PREC_MIXED) return advtyp == 1 || advtyp == 2 || advtyp == 4;
  return advtyp == 0 || advtyp == 1 || advtyp == 2 || advtyp == 4;
}

bool shape_ok(const hyc_ens *e, hyc::TileShape t) {
  if (e->prec == HYC_PREC_MIXED)
    return is_col2(t) && (t.ty == 32 || t.ty == 64 || t.ty == 128 || t.ty == 256 || t.ty == 512 || t.ty == 1024 ||
                           t.ty == 2048);
  return (t.tx == 32 && t.ty == 16) || (t.tx == 16 && t.ty == 16);
}

}  // namespace

extern "C" {

const char *hyc_ens_last_error(const hyc_ens *e) { return e ? e->err.c_str() : ""; }

int hyc_ens_create(hyc_ens **out, int32_t nbasin, const hyc_basin_spec *specs, int32_t precision, int32_t device) {
  if (!out || nbasin < 1 || !specs || (precision != HYC_PREC_FP64 && precision != HYC_PREC_MIXED))
    return efail(nullptr, HYC_ERR_ARG, "hyc_ens_create: bad arguments");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return efail(nullptr, HYC_ERR_CUDA, "hyc_ens_create: CUDA device %d not available", device);
  hyc_ens *e = new hyc_ens;
  e->device = device;
  e->prec = precision;
  Dev g(device);
  cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, device);
  auto bail = [&](int rc) {
    free_all(e);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    delete e;
    return rc;
  };
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(efail(nullptr, HYC_ERR_CUDA, "stream"));
  e->own_stream = true;
  const int align = precision == HYC_PREC_MIXED ? 4 : 2;  // 16-byte rows
  int maxk = 0;
  for (int i = 0; i < nbasin; i++) {
    const hyc_basin_spec &s = specs[i];
    if (s.idm < 1 || s.jdm < 1 || s.kdm < 1 || s.nbdy < 5 || s.ntr < 1 || s.ntr > hyc::kMaxFields ||
        !(s.nreg == 0 || s.nreg == 1) || !s.ip || !s.iu || !s.iv || !s.scp2 || !s.scp2i)
      return bail(efail(nullptr, HYC_ERR_ARG, "basin %d: bad spec (nbdy>=5, 1<=ntr<=16, nreg 0/1)", i));
    EBasin b;
    b.idm = s.idm;
    b.jdm = s.jdm;
    b.kdm = s.kdm;
    b.nbdy = s.nbdy;
    b.nreg = s.nreg;
    b.ntr = s.ntr;
    b.ld1r = s.idm + 2 * s.nbdy;
    b.ld1 = (b.ld1r + align - 1) / align * align;
    b.ld2 = s.jdm + 2 * s.nbdy;
    b.slice = (long long)b.ld1 * b.ld2;
    b.work = (long long)s.idm * s.jdm * s.kdm * s.ntr;
    b.posdef.assign(s.ntr, 0.0);
    maxk = std::max(maxk, s.kdm);
    e->maxntr = std::max(e->maxntr, s.ntr);
    // masks (validated like hyc_adv_init) and metrics, repitched
    std::vector<uint8_t> m((size_t)b.slice, 0);
    std::vector<double> sc((size_t)b.slice, 1.0), si((size_t)b.slice, 1.0);
    for (int j = 0; j < b.ld2; j++)
      for (int ia = 0; ia < b.ld1r; ia++) {
        const size_t o = (size_t)ia + (size_t)j * b.ld1r, d = (size_t)ia + (size_t)j * b.ld1;
        const bool p = s.ip[o] != 0, u = s.iu[o] != 0, v = s.iv[o] != 0;
        if (ia > 0 && u != (p && s.ip[o - 1] != 0))
          return bail(efail(nullptr, HYC_ERR_MASK, "basin %d: iu inconsistent with ip", i));
        if (j > 0 && v != (p && s.ip[o - b.ld1r] != 0))
          return bail(efail(nullptr, HYC_ERR_MASK, "basin %d: iv inconsistent with ip", i));
        m[d] = (p ? hyc::kIP : 0) | (u ? hyc::kIU : 0) | (v ? hyc::kIV : 0);
        sc[d] = s.scp2[o];
        si[d] = s.scp2i[o];
      }
    const size_t es = precision == HYC_PREC_MIXED ? 4 : 8;
    bool ok = cudaMalloc(&b.msk, b.slice) == cudaSuccess && cudaMalloc(&b.scp2, b.slice * 8) == cudaSuccess &&
              cudaMalloc(&b.scp2i, b.slice * 8) == cudaSuccess &&
              cudaMalloc(&b.uflx, b.slice * b.kdm * es) == cudaSuccess &&
              cudaMalloc(&b.vflx, b.slice * b.kdm * es) == cudaSuccess &&
              cudaMalloc(&b.dp, b.slice * b.kdm * 8) == cudaSuccess;
    for (int l = 0; l < 3 && ok; l++) ok = cudaMalloc(&b.lev[l], b.slice * b.kdm * b.ntr * es) == cudaSuccess;
    if (ok && precision == HYC_PREC_MIXED) ok = cudaMalloc(&b.cell, b.slice * sizeof(double)) == cudaSuccess;
    e->b.push_back(b);
    if (!ok) return bail(efail(nullptr, HYC_ERR_NOMEM, "basin %d: device allocation failed", i));
    EBasin &bb = e->b.back();
    bool cp = cudaMemcpy(bb.msk, m.data(), bb.slice, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(bb.scp2, sc.data(), bb.slice * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(bb.scp2i, si.data(), bb.slice * 8, cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemset(bb.uflx, 0, bb.slice * bb.kdm * es) == cudaSuccess &&
              cudaMemset(bb.vflx, 0, bb.slice * bb.kdm * es) == cudaSuccess &&
              cudaMemset(bb.dp, 0, bb.slice * bb.kdm * 8) == cudaSuccess;
    for (int l = 0; l < 3 && cp; l++) cp = cudaMemset(bb.lev[l], 0, bb.slice * bb.kdm * bb.ntr * es) == cudaSuccess;
    if (!cp) return bail(efail(nullptr, HYC_ERR_CUDA, "basin %d: upload failed", i));
  }
  for (int r = 0; r < 3; r++) {
    bool ok = precision == HYC_PREC_MIXED ? cudaMalloc(&e->d_mix[r], nbasin * sizeof(MixBasin)) == cudaSuccess &&
                                                cudaMalloc(&e->d_mixt[r], nbasin * sizeof(MixBasin)) == cudaSuccess
                                          : cudaMalloc(&e->d_targs[r], nbasin * sizeof(TileArgs)) == cudaSuccess;
    if (!ok) return bail(efail(nullptr, HYC_ERR_NOMEM, "tables"));
  }
  e->npartial = maxk;
  if (cudaMalloc(&e->d_partial, 2 * maxk * sizeof(double)) != cudaSuccess)
    return bail(efail(nullptr, HYC_ERR_NOMEM, "partials"));
  if (cudaMalloc(&e->d_err, sizeof(int)) != cudaSuccess || cudaMemset(e->d_err, 0, sizeof(int)) != cudaSuccess)
    return bail(efail(nullptr, HYC_ERR_NOMEM, "error flag"));
  if (precision == HYC_PREC_MIXED) {  // the strip kernel streams its rows by TMA
    if (!hyc::tmap_available())
      return bail(efail(nullptr, HYC_ERR_UNSUPPORTED, "the mixed form needs cuTensorMapEncodeTiled (driver)"));
    if (cudaMalloc(&e->d_cmaps, nbasin * kMaps * sizeof(CUtensorMap)) != cudaSuccess)
      return bail(efail(nullptr, HYC_ERR_NOMEM, "strip maps"));
    int rc = encode_strip_maps(e);
    if (rc) return bail(rc);
    e->shape = hyc::TileShape{hyc::kCol2Strip, 128};
  }
  *out = e;
  return HYC_OK;
}

int hyc_ens_destroy(hyc_ens *e) {
  if (!e) return HYC_OK;
  {
    Dev g(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    free_all(e);
    if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
    if (e->cap_stream) cudaStreamDestroy(e->cap_stream);
  }
  delete e;
  return HYC_OK;
}

int hyc_ens_set_stream(hyc_ens *e, void *stream) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  Dev g(e->device);
  if (e->own_stream && e->stream) {
    cudaStreamSynchronize(e->stream);
    cudaStreamDestroy(e->stream);
  }
  e->stream = (cudaStream_t)stream;
  e->own_stream = false;
  if (e->gexec) {
    cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
  }
  return HYC_OK;
}

// Open a timed span on stream st (timers on): returns the start event.
static cudaEvent_t span_open(hyc_ens *e, cudaStream_t st) {
  if (!e->timing) return nullptr;
  cudaEvent_t a = nullptr;
  cudaEventCreate(&a);
  cudaEventRecord(a, st);
  return a;
}
static void span_close(hyc_ens *e, cudaEvent_t a, int slot, cudaStream_t st) {
  if (!a) return;
  cudaEvent_t z = nullptr;
  cudaEventCreate(&z);
  cudaEventRecord(z, st);
  e->pending.push_back({slot, a, z});
}

static int grow(hyc_ens *e, double **buf, size_t *have, size_t bytes, const char *what) {
  if (*have >= bytes) return HYC_OK;
  cudaFree(*buf);
  *buf = nullptr;
  *have = 0;
  ECK(cudaMalloc(buf, bytes), what);
  *have = bytes;
  return HYC_OK;
}

static int ensure_io(hyc_ens *e) {
  if (e->in_stream) return HYC_OK;
  ECK(cudaStreamCreateWithFlags(&e->in_stream, cudaStreamNonBlocking), "input stream");
  ECK(cudaStreamCreateWithFlags(&e->copy_stream, cudaStreamNonBlocking), "copy stream");
  for (int q = 0; q < 2; q++) {
    ECK(cudaEventCreateWithFlags(&e->ev_copied[q], cudaEventDisableTiming), "event");
    ECK(cudaEventCreateWithFlags(&e->ev_used[q], cudaEventDisableTiming), "event");
  }
  ECK(cudaEventCreateWithFlags(&e->ev_entry, cudaEventDisableTiming), "event");
  ECK(cudaEventCreateWithFlags(&e->ev_staged, cudaEventDisableTiming), "event");
  ECK(cudaEventCreateWithFlags(&e->ev_gdone, cudaEventDisableTiming), "event");
  return HYC_OK;
}

// Host-link copies with timers on: slot HYC_T_COPY; halo/repitch kernels: HYC_T_XCTILR.
static int move(hyc_ens *e, int32_t basin, int32_t what, int32_t s0, int32_t ns_req, void *host, int32_t where,
                bool put, bool async_get = false) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  if (basin < 0 || basin >= (int)e->b.size() || what < HYC_E_OLD || what > HYC_E_DP || !host ||
      (where != HYC_HOST && where != HYC_DEVICE) || (!put && what > HYC_E_CUR && what != HYC_E_DP))
    return efail(e, HYC_ERR_ARG, "hyc_ens_put/get: bad arguments");
  Dev g(e->device);
  EBasin &b = e->b[basin];
  void *dst;
  int dfp32 = e->prec == HYC_PREC_MIXED;
  int ns;
  switch (what) {
    case HYC_E_OLD: dst = b.lev[e->rot]; ns = b.ntr * b.kdm; break;
    case HYC_E_CUR: dst = b.lev[(e->rot + 1) % 3]; ns = b.ntr * b.kdm; break;
    case HYC_E_UFLX: dst = b.uflx; ns = b.kdm; break;
    case HYC_E_VFLX: dst = b.vflx; ns = b.kdm; break;
    default: dst = b.dp; ns = b.kdm; dfp32 = 0; break;
  }
  // a contiguous run of slices [s0, s0+ns_req); ns_req < 0 means all of them
  if (ns_req < 0) {
    if (s0 != 0) return efail(e, HYC_ERR_ARG, "hyc_ens_put/get: s0 without a slice count");
    ns_req = ns;
  }
  if (s0 < 0 || ns_req < 1 || (long long)s0 + ns_req > ns)
    return efail(e, HYC_ERR_ARG, "hyc_ens_put/get: slices [%d, %d) outside [0, %d)", s0, s0 + ns_req, ns);
  ns = ns_req;
  dst = (char *)dst + (size_t)s0 * b.slice * (dfp32 ? 4 : 8);
  const long long rsl = (long long)b.ld1r * b.ld2;
  const size_t bytes = (size_t)rsl * ns * 8;
  int rc;
  if ((rc = ensure_io(e))) return rc;
  const cudaMemcpyKind kin = where == HYC_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind kout = where == HYC_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  cudaError_t c;
  if (put) {
    const int q = e->stage_next;
    e->stage_next ^= 1;
    if (e->stage_bytes[q] < bytes) {  // nothing may still use the old buffer
      ECK(cudaStreamSynchronize(e->stream), "put sync");
      ECK(cudaStreamSynchronize(e->in_stream), "put sync");
      e->stage_used[q] = false;
      if ((rc = grow(e, &e->d_stage[q], &e->stage_bytes[q], bytes, "staging"))) return rc;
    }
    double *stage = e->d_stage[q];
    // the copy waits for the last kernels that read this buffer; a device
    // source may still be written by work queued on the ensemble's stream
    if (e->stage_used[q]) ECK(cudaStreamWaitEvent(e->in_stream, e->ev_used[q], 0), "wait staging");
    if (where == HYC_DEVICE) {
      ECK(cudaEventRecord(e->ev_entry, e->stream), "event");
      ECK(cudaStreamWaitEvent(e->in_stream, e->ev_entry, 0), "wait source");
    }
    cudaEvent_t t0 = span_open(e, e->in_stream);
    ECK(cudaMemcpyAsync(stage, host, bytes, kin, e->in_stream), "put copy");
    span_close(e, t0, HYC_T_COPY, e->in_stream);
    ECK(cudaEventRecord(e->ev_copied[q], e->in_stream), "event");
    ECK(cudaStreamWaitEvent(e->stream, e->ev_copied[q], 0), "wait copy");
    cudaEvent_t t1 = span_open(e, e->stream);
    // tsadvc refreshes these halos before advecting (mod_tsadvc.F90:1829-1836); dp's is taken as given
    if (what != HYC_E_DP) {
      c = hyc::launch_xctilr(stage, rsl, ns, b.idm, b.jdm, b.nbdy, b.ld1r, 5, 5, b.nreg, e->stream);
      if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "put halo: %s", cudaGetErrorString(c));
    }
    c = hyc::launch_repitch(stage, 0, b.ld1r, rsl, dst, dfp32, b.ld1, b.slice, b.ld1r, b.ld2, ns, e->stream);
    if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "put: %s", cudaGetErrorString(c));
    span_close(e, t1, HYC_T_XCTILR, e->stream);
    ECK(cudaEventRecord(e->ev_used[q], e->stream), "event");
    e->stage_used[q] = true;
    // the caller's buffer is free once its copy is done; the kernels go on
    ECK(cudaEventSynchronize(e->ev_copied[q]), "put copy sync");
    if (what == HYC_E_OLD || what == HYC_E_CUR) e->primed = false;
    return HYC_OK;
  }
  // get: repitch into the get staging on the ensemble's stream (after any
  // copy-out still reading it), then copy out
  if (e->gstage_bytes < bytes) {
    ECK(cudaStreamSynchronize(e->copy_stream), "copy stream sync");
    e->get_pending = false;
    if ((rc = grow(e, &e->d_gstage, &e->gstage_bytes, bytes, "get staging"))) return rc;
  }
  if (e->get_pending) ECK(cudaStreamWaitEvent(e->stream, e->ev_gdone, 0), "wait copy-out");
  cudaEvent_t t1 = span_open(e, e->stream);
  c = hyc::launch_repitch(dst, dfp32, b.ld1, b.slice, e->d_gstage, 0, b.ld1r, rsl, b.ld1r, b.ld2, ns, e->stream);
  if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "get: %s", cudaGetErrorString(c));
  span_close(e, t1, HYC_T_XCTILR, e->stream);
  ECK(cudaEventRecord(e->ev_staged, e->stream), "event");
  ECK(cudaStreamWaitEvent(e->copy_stream, e->ev_staged, 0), "wait staged");
  cudaEvent_t t0 = span_open(e, e->copy_stream);
  ECK(cudaMemcpyAsync(host, e->d_gstage, bytes, kout, e->copy_stream), "get copy");
  span_close(e, t0, HYC_T_COPY, e->copy_stream);
  ECK(cudaEventRecord(e->ev_gdone, e->copy_stream), "event");
  e->get_pending = true;
  if (!async_get) {
    ECK(cudaEventSynchronize(e->ev_gdone), "get sync");
    e->get_pending = false;
  }
  return HYC_OK;
}

int hyc_ens_put(hyc_ens *e, int32_t basin, int32_t what, const double *src, int32_t where) {
  return move(e, basin, what, 0, -1, (void *)src, where, true);
}

int hyc_ens_get(hyc_ens *e, int32_t basin, int32_t what, double *dst, int32_t where) {
  return move(e, basin, what, 0, -1, dst, where, false);
}

int hyc_ens_get_async(hyc_ens *e, int32_t basin, int32_t what, double *dst, int32_t where) {
  return move(e, basin, what, 0, -1, dst, where, false, true);
}

int hyc_selftest_wait(int32_t device, int32_t arrive, int32_t *gave_up) {
  if (!gave_up) return efail(nullptr, HYC_ERR_ARG, "hyc_selftest_wait: null argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return efail(nullptr, HYC_ERR_CUDA, "hyc_selftest_wait: no CUDA device %d", device);
  Dev g(device);
  int *d = nullptr, flag = 0;
  cudaError_t c = cudaMalloc(&d, sizeof(int));
  if (c == cudaSuccess) c = cudaMemset(d, 0, sizeof(int));
  if (c == cudaSuccess) c = hyc::launch_wait_probe(arrive != 0, d, nullptr);
  if (c == cudaSuccess) c = cudaDeviceSynchronize();
  if (c == cudaSuccess) c = cudaMemcpy(&flag, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (c != cudaSuccess) return efail(nullptr, HYC_ERR_CUDA, "hyc_selftest_wait: %s", cudaGetErrorString(c));
  *gave_up = flag;
  return HYC_OK;
}

int hyc_ens_wait(hyc_ens *e) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  Dev g(e->device);
  if (e->copy_stream) ECK(cudaStreamSynchronize(e->copy_stream), "copy-out sync");
  e->get_pending = false;
  return HYC_OK;
}

int hyc_ens_put_slices(hyc_ens *e, int32_t basin, int32_t what, int32_t s0, int32_t ns, const double *src,
                       int32_t where) {
  return move(e, basin, what, s0, ns, (void *)src, where, true);
}

int hyc_ens_get_slices(hyc_ens *e, int32_t basin, int32_t what, int32_t s0, int32_t ns, double *dst,
                       int32_t where) {
  return move(e, basin, what, s0, ns, dst, where, false);
}

int hyc_ens_set_tile(hyc_ens *e, int32_t tx, int32_t ty) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  hyc::TileShape t{tx, ty};
  if (!shape_ok(e, t)) return efail(e, HYC_ERR_ARG, "tile %dx%d not available", tx, ty);
  if (t.tx != e->shape.tx || t.ty != e->shape.ty) {
    e->shape = t;
    e->tbl_dt2 = -1.0;
    if (e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
  }
  return HYC_OK;
}

int hyc_ens_set_option(hyc_ens *e, int32_t option, int32_t value) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  if (option == HYC_OPT_PREP64) {
    if (e->prec != HYC_PREC_MIXED) return efail(e, HYC_ERR_ARG, "HYC_OPT_PREP64 applies to the mixed form");
    if (e->prep64 != (value != 0) && e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
    e->prep64 = value != 0;
    return HYC_OK;
  }
  if (option == HYC_OPT_STRIP_TRACERS) {
    if (e->prec != HYC_PREC_MIXED || value < 1 || value > 2)
      return efail(e, HYC_ERR_ARG, "HYC_OPT_STRIP_TRACERS: 1 or 2, mixed form");
    if (e->strip_nq != value && e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
    e->strip_nq = value;
    return HYC_OK;
  }
  return efail(e, HYC_ERR_ARG, "unknown option %d", option);
}

int hyc_ens_set_posdef(hyc_ens *e, int32_t basin, int32_t tracer, double posdef) {
  if (!e || basin < 0 || basin >= (int)e->b.size() || tracer < 0 || tracer >= e->b[basin].ntr)
    return efail(e, HYC_ERR_ARG, "hyc_ens_set_posdef: bad basin or tracer");
  if (e->b[basin].posdef[tracer] != posdef) {
    Dev g(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);  // steps in flight read the tables
    e->b[basin].posdef[tracer] = posdef;
    e->tbl_dt2 = -1.0;
    if (e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
  }
  return HYC_OK;
}

int hyc_ens_set_diffusion(hyc_ens *e, int32_t basin, double temdf2, const double *aspux, const double *aspvy,
                          const double *scuy, const double *scvx, int32_t where) {
  if (!e || basin < 0 || basin >= (int)e->b.size()) return efail(e, HYC_ERR_ARG, "hyc_ens_set_diffusion: bad basin");
  if (e->prec != HYC_PREC_MIXED)
    return efail(e, HYC_ERR_UNSUPPORTED, "hyc_ens_set_diffusion: the FP32-mixed form only (FP64: hyc_tsdff)");
  if (!(temdf2 >= 0.0)) return efail(e, HYC_ERR_ARG, "hyc_ens_set_diffusion: temdf2 < 0");
  if (temdf2 > 0.0 && (!aspux || !aspvy || !scuy || !scvx))
    return efail(e, HYC_ERR_ARG, "hyc_ens_set_diffusion: null grid array");
  if (where != HYC_HOST && where != HYC_DEVICE) return efail(e, HYC_ERR_ARG, "hyc_ens_set_diffusion: bad where");
  Dev g(e->device);
  ECK(cudaStreamSynchronize(e->stream), "diffusion sync");  // steps in flight read the tables
  // every basin gets a table once one diffuses (zeros: no diffusion)
  if (temdf2 > 0.0 && !e->diff) {
    for (auto &b : e->b)
      if (!b.gd) {
        if (cudaMalloc(&b.gd, b.slice * sizeof(float2)) != cudaSuccess)
          return efail(e, HYC_ERR_NOMEM, "hyc_ens_set_diffusion: table allocation");
        ECK(cudaMemset(b.gd, 0, b.slice * sizeof(float2)), "diffusion table");
      }
  }
  EBasin &b = e->b[basin];
  if (b.gd) {
    if (temdf2 > 0.0) {
      const size_t rsl = (size_t)b.ld1r * b.ld2;
      const double *src[4] = {aspux, aspvy, scuy, scvx};
      double *tmp = nullptr;
      if (where == HYC_HOST) {
        if (cudaMalloc(&tmp, 4 * rsl * sizeof(double)) != cudaSuccess)
          return efail(e, HYC_ERR_NOMEM, "hyc_ens_set_diffusion: staging");
        for (int a = 0; a < 4; a++) {
          cudaError_t c = cudaMemcpy(tmp + a * rsl, src[a], rsl * sizeof(double), cudaMemcpyHostToDevice);
          if (c != cudaSuccess) {
            cudaFree(tmp);
            return efail(e, HYC_ERR_CUDA, "hyc_ens_set_diffusion: copy: %s", cudaGetErrorString(c));
          }
          src[a] = tmp + a * rsl;
        }
      }
      cudaError_t c = hyc::launch_diff_table(src[0], src[1], src[2], src[3], b.msk, temdf2, b.ld1r, b.ld1, b.ld2,
                                             b.gd, e->stream);
      if (c == cudaSuccess) c = cudaStreamSynchronize(e->stream);
      cudaFree(tmp);
      if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "hyc_ens_set_diffusion: %s", cudaGetErrorString(c));
    } else {
      ECK(cudaMemset(b.gd, 0, b.slice * sizeof(float2)), "diffusion table");
    }
  }
  b.temdf2 = temdf2;
  bool any = false;
  for (const auto &x : e->b) any |= x.temdf2 > 0.0;
  if (any != e->diff || temdf2 > 0.0) {
    e->diff = any;
    int rc = encode_strip_maps(e);
    if (rc) return rc;
    e->tbl_dt2 = -1.0;
    if (e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
  }
  return HYC_OK;
}

int hyc_ens_get_option(hyc_ens *e, int32_t option, int32_t *value) {
  if (!e || !value) return efail(e, HYC_ERR_ARG, "null argument");
  switch (option) {
    case HYC_OPT_PREP64: *value = e->prep64; return HYC_OK;
    case HYC_OPT_STRIP_TRACERS: *value = e->strip_nq; return HYC_OK;
    default: return efail(e, HYC_ERR_ARG, "unknown option %d", option);
  }
}

int hyc_ens_enable_timers(hyc_ens *e, int32_t on) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  e->timing = on != 0;
  return HYC_OK;
}

int hyc_ens_stats(hyc_ens *e, hyc_stats *out, int32_t reset) {
  if (!e || !out) return efail(e, HYC_ERR_ARG, "null argument");
  Dev g(e->device);
  ECK(cudaStreamSynchronize(e->stream), "stats sync");
  int flag = 0;
  ECK(cudaMemcpy(&flag, e->d_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
  if (flag) return efail(e, HYC_ERR_CUDA, "a step kernel gave up waiting for its TMA loads");
  if (e->in_stream) ECK(cudaStreamSynchronize(e->in_stream), "stats sync");
  if (e->copy_stream) ECK(cudaStreamSynchronize(e->copy_stream), "stats sync");
  for (auto &p : e->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.z) == cudaSuccess) {
      e->stats.ms[p.slot] += ms;
      e->stats.calls[p.slot] += 1;
    }
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.z);
  }
  e->pending.clear();
  *out = e->stats;
  if (reset) e->stats = hyc_stats{};
  return HYC_OK;
}

int hyc_ens_step(hyc_ens *e, int32_t advtyp, double delt1, int32_t nsteps, int32_t use_graph) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  if (nsteps < 1) return efail(e, HYC_ERR_ARG, "nsteps < 1");
  if (!scheme_ok(e, advtyp))
    return efail(e, HYC_ERR_UNSUPPORTED, "ensemble advtyp %d not available for this precision", advtyp);
  if (e->diff && !e->prep64)
    return efail(e, HYC_ERR_UNSUPPORTED, "the diffusion epilogue needs the FP64 thickness prep (HYC_OPT_PREP64)");
  Dev g(e->device);
  int rc;
  if ((rc = build_items(e)) ||
      (rc = build_tables(e, delt1)) || (rc = ensure_heads(e, nsteps)) || (rc = prime(e)))
    return rc;
  cudaEvent_t a = nullptr, z = nullptr;
  if (e->timing) {
    cudaEventCreate(&a);
    cudaEventCreate(&z);
    cudaEventRecord(a, e->stream);
  }
  if (!use_graph) {
    for (int s = 0; s < nsteps; s++) {
      if ((rc = enqueue_step(e, advtyp, e->rot, s, e->stream))) return rc;
      e->rot = (e->rot + 1) % 3;
    }
  } else {
    const bool reuse = e->gexec && e->g_nsteps == nsteps && e->g_advtyp == advtyp && e->g_dt == delt1 &&
                       e->g_rot == e->rot && e->g_tx == e->shape.tx && e->g_ty == e->shape.ty;
    if (!reuse) {
      if (e->gexec) {
        cudaGraphExecDestroy(e->gexec);
        e->gexec = nullptr;
      }
      // recorded on a private stream (the caller's may be the legacy default
      // stream, which cannot be captured), launched on the caller's stream
      if (!e->cap_stream) ECK(cudaStreamCreateWithFlags(&e->cap_stream, cudaStreamNonBlocking), "capture stream");
      ECK(cudaStreamSynchronize(e->stream), "pre-capture sync");
      cudaGraph_t graph = nullptr;
      ECK(cudaStreamBeginCapture(e->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      int r = e->rot;
      int64_t l0 = e->stats.launches;
      for (int s = 0; s < nsteps; s++) {
        if ((rc = enqueue_step(e, advtyp, r, s, e->cap_stream))) {
          cudaStreamEndCapture(e->cap_stream, &graph);
          if (graph) cudaGraphDestroy(graph);
          return rc;
        }
        r = (r + 1) % 3;
      }
      e->stats.launches = l0;
      ECK(cudaStreamEndCapture(e->cap_stream, &graph), "end capture");
      cudaError_t c = cudaGraphInstantiate(&e->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(c));
      e->g_nsteps = nsteps;
      e->g_advtyp = advtyp;
      e->g_dt = delt1;
      e->g_rot = e->rot;
      e->g_tx = e->shape.tx;
      e->g_ty = e->shape.ty;
    }
    ECK(cudaGraphLaunch(e->gexec, e->stream), "graph launch");
    e->stats.launches += nsteps;
    e->rot = (e->rot + nsteps) % 3;
  }
  if (e->timing) {
    cudaEventRecord(z, e->stream);
    e->pending.push_back({HYC_T_ADVECT, a, z});
  }
  return HYC_OK;
}

int hyc_ens_tune(hyc_ens *e, int32_t advtyp, double delt1, int32_t *tx, int32_t *ty, double *ms_out) {
  if (!e) return efail(nullptr, HYC_ERR_ARG, "null ensemble");
  if (e->diff && !e->prep64)
    return efail(e, HYC_ERR_UNSUPPORTED, "the diffusion epilogue needs the FP64 thickness prep (HYC_OPT_PREP64)");
  Dev g(e->device);
  static const hyc::TileShape cands[] = {{32, 16},  {16, 16},  {56, 32},   {56, 64},  {56, 128},
                                         {56, 256}, {56, 512}, {56, 1024}, {56, 2048}};
  hyc::TileShape best = e->shape;
  float best_ms = 1e30f;
  const hyc::TileShape keep = e->shape;
  cudaEvent_t a, z;
  cudaEventCreate(&a);
  cudaEventCreate(&z);
  int rc = prime(e);
  if (rc) return rc;
  int best_nq = e->strip_nq;
  const int keep_nq = e->strip_nq;
  std::vector<std::pair<hyc::TileShape, int>> trials;
  for (const auto &c : cands) {
    if (!shape_ok(e, c) || !scheme_ok(e, advtyp)) continue;
    if (is_col2(c) && e->maxntr > 1) trials.push_back({c, 1});
    trials.push_back({c, 2});
  }
  for (const auto &tr : trials) {
    const hyc::TileShape c = tr.first;
    e->strip_nq = tr.second;
    e->shape = c;
    e->tbl_dt2 = -1.0;
    if ((rc = build_items(e)) ||
        (rc = build_tables(e, delt1)) || (rc = ensure_heads(e, 1)))
      break;
    // the step kernel writes only the spare level: the state is unchanged
    if ((rc = enqueue_step(e, advtyp, e->rot, 0, e->stream))) break;  // warm-up
    float tot = 0.f;
    const int reps = 3;
    for (int r = 0; r < reps && !rc; r++) {
      cudaEventRecord(a, e->stream);
      rc = enqueue_step(e, advtyp, e->rot, 0, e->stream);
      cudaEventRecord(z, e->stream);
      cudaEventSynchronize(z);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, z);
      tot += ms;
    }
    if (rc) break;
    if (tot / reps < best_ms) {
      best_ms = tot / reps;
      best = c;
      best_nq = tr.second;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(z);
  if (rc) {
    e->shape = keep;
    e->strip_nq = keep_nq;
    e->tbl_dt2 = -1.0;
    return rc;
  }
  e->shape = best;
  e->strip_nq = is_col2(best) ? best_nq : keep_nq;
  e->tbl_dt2 = -1.0;
  e->items_tx = 0;  // force the queue for the chosen shape
  if (e->gexec) {
    cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
  }
  if (tx) *tx = best.tx;
  if (ty) *ty = best.ty;
  if (ms_out) *ms_out = best_ms;
  return HYC_OK;
}

int hyc_ens_content(hyc_ens *e, int32_t basin, int32_t tracer, int32_t what, double delt1, double *sum) {
  if (!e || !sum || basin < 0 || basin >= (int)e->b.size() || (what != HYC_E_OLD && what != HYC_E_CUR))
    return efail(e, HYC_ERR_ARG, "hyc_ens_content: bad arguments");
  EBasin &b = e->b[basin];
  if (tracer < 0 || tracer >= b.ntr) return efail(e, HYC_ERR_ARG, "tracer out of range");
  Dev g(e->device);
  const int lev = what == HYC_E_OLD ? e->rot : (e->rot + 1) % 3;
  const size_t es = esz(e);
  const char *base = (const char *)b.lev[lev] + (size_t)tracer * b.kdm * b.slice * es;
  const int fp32 = e->prec == HYC_PREC_MIXED;
  cudaError_t c = hyc::launch_content(base, fp32, b.uflx, b.vflx, fp32, b.dp, b.scp2, b.scp2i, b.msk, b.idm, b.jdm,
                                      b.nbdy, b.ld1, b.slice, b.kdm, what == HYC_E_OLD, delt1, e->d_partial,
                                      e->stream);
  if (c != cudaSuccess) return efail(e, HYC_ERR_CUDA, "content: %s", cudaGetErrorString(c));
  std::vector<double> p(2 * b.kdm);
  ECK(cudaMemcpyAsync(p.data(), e->d_partial, p.size() * 8, cudaMemcpyDeviceToHost, e->stream), "content d2h");
  ECK(cudaStreamSynchronize(e->stream), "content sync");
  double hi = 0.0, lo = 0.0;
  for (int k = 0; k < b.kdm; k++) {  // compensated, fixed order
    const double s = hi + p[2 * k];
    const double bb = s - hi;
    lo += (hi - (s - bb)) + (p[2 * k] - bb) + p[2 * k + 1];
    hi = s;
  }
  *sum = hi + lo;
  return HYC_OK;
}

}  // extern "C"
