/*
 * hyc_oracle.c -- CPU oracle for HYCOM's layered tracer-advection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA
 * product path is compared against (tests, smoke check, the CPU baseline
 * leg of the benchmark).  Nothing in the product library links it.
 *
 * It restates, loop for loop and in the reference's expression order, the
 * following routines of HYCOM-src (all FP64, REAL*8 build):
 *   mod_tsadvc.F90:69-205     advem        (scheme dispatch)
 *   mod_tsadvc.F90:207-493    advem_mpdata
 *   mod_tsadvc.F90:495-643    advem_pcm
 *   mod_tsadvc.F90:645-997    advem_fct2
 *   mod_tsadvc.F90:999-1368   advem_fct2c
 *   mod_tsadvc.F90:1370-1706  advem_fct4
 *   mod_tsadvc.F90:1708-2132  tsadvc       (advection part, no diffusion)
 *   mod_xc_sm.h:1337-1428     xctilr       (single tile, closed/periodic)
 *   mod_xc_sm.h:900-963       xcsum        (fixed-order FP64 sum)
 *   bigrid.F90:1-541          bigrid, indxi, indxj (masks, sections)
 *
 * Semantics kept on purpose:
 *   - the 16 (+9 for fct2c) work arrays are module state that persists
 *     between calls (mod_tsadvc.F90:38-65) and start as NaN (r_init under
 *     NAN2003, mod_dimensions.F90:264-277), so a read of a value that the
 *     reference never wrote shows up as NaN;
 *   - loop margins, section-edge flux zeroing and the coastal ipip1/ipjp1
 *     use in the Zalesak limiter (mod_tsadvc.F90:880-883) are as written;
 *   - built with -ffp-contract=off: no fused multiply-add contraction,
 *     every product and sum rounded separately, left to right, honouring
 *     Fortran's parentheses.
 *
 * Parity unpinned: the reference ships no golden vectors or known-answer
 * tests for this path and no Fortran compiler exists on either machine, so
 * this restatement is checked against the reference's own run-time
 * invariants (mod_pipe.F90:1516-1546) and analytic known answers instead.
 *
 * Arrays use the reference layout: column-major (i fastest), lower bound
 * 1-nbdy in i and j; a 2-D slice has ld1=idm+2*nbdy by ld2=jdm+2*nbdy
 * elements and the pointer passed points at element (1-nbdy,1-nbdy).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define HYO_OK 0
#define HYO_ERR_ARG -1
#define HYO_ERR_GRID -2
#define HYO_ERR_ADVTYP -3
#define HYO_ERR_NBDY -4
#define HYO_ERR_MEM -5

typedef struct hyo_grid {
  int ii, jj, nbdy, ld1, ld2, nreg, ms;
  int lperiod;
  int32_t *ip, *iu, *iv, *iq;
  int32_t *ipim1, *ipip1, *ipjm1, *ipjp1;
  /* sections: ifp(j,l) with j in 1-nbdy..jj+nbdy, l in 1..ms */
  int32_t *ifp, *ilp, *isp, *jfp, *jlp, *jsp;
  double *scp2, *scp2i;
  /* module work arrays of mod_tsadvc (persist between calls) */
  double *fmx, *fmn, *flx, *fly, *fldlo, *fmxlo, *fmnlo, *fax, *fay, *rp, *rm,
      *flxdiv, *tx1, *ty1, *fldao, *fldan;
  double *uloc, *vloc, *hloc, *dtloc, *ucumdt, *vcumdt, *flxcum, *flycum;
  unsigned char *lcalc;
  /* tsadvc work */
  double *util1, *util2, *uflux, *vflux;
  /* second-field diffusive fluxes (mod_cb_arrays uflux2/vflux2): 0 on every
     face a sea cell touches, as geopar.F90:833 leaves them */
  double *uflux2, *vflux2;
  int nthreads; /* 0 = OpenMP default */
  int lconserve; /* advem's explicit conservation rescale, mod_tsadvc.F90:32 (.false. as shipped) */
} hyo_grid;

#define P(g, i, j) ((size_t)((i) + (g)->nbdy - 1) + (size_t)((j) + (g)->nbdy - 1) * (size_t)(g)->ld1)
/* section arrays: ifp(j,l) -> column-major (1-nbdy:jj+nbdy, ms) */
#define SJ(g, j, l) ((size_t)((j) + (g)->nbdy - 1) + (size_t)((l)-1) * (size_t)(g)->ld2)
#define SI(g, i, l) ((size_t)((i) + (g)->nbdy - 1) + (size_t)((l)-1) * (size_t)(g)->ld1)

static const double ONEMU = 9806.e-12; /* mod_tsadvc.F90:236,519,671,1396 */
/* onem = g/svref with g = 9.806, svref = 1/1000 (mod_cb_arrays.F90:843-846),
   folded in double: 9805.999999999998, not 9806 */
#define ONEM (9.806 / (1.0 / 1000.0))
static const double EPSIL = 1.e-10;    /* mod_tsadvc.F90:1027 */

static inline double mx2(double a, double b) { return a > b ? a : b; }
static inline double mn2(double a, double b) { return a < b ? a : b; }
static inline double mx3(double a, double b, double c) { return mx2(mx2(a, b), c); }
static inline double mn3(double a, double b, double c) { return mn2(mn2(a, b), c); }
static inline double mx5(double a, double b, double c, double d, double e) {
  return mx2(mx2(mx2(mx2(a, b), c), d), e);
}
static inline double mn5(double a, double b, double c, double d, double e) {
  return mn2(mn2(mn2(mn2(a, b), c), d), e);
}

static double *nan_array(size_t n) {
  double *a = (double *)malloc(n * sizeof(double));
  if (!a) return NULL;
  double q = NAN;
  for (size_t k = 0; k < n; k++) a[k] = q;
  return a;
}

void hyo_set_threads(hyo_grid *g, int n) { g->nthreads = n; }
void hyo_set_conserve(hyo_grid *g, int on) { g->lconserve = on != 0; }

static int nthr(const hyo_grid *g) {
#ifdef _OPENMP
  return g->nthreads > 0 ? g->nthreads : omp_get_max_threads();
#else
  (void)g;
  return 1;
#endif
}

int hyo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* xctilr: mod_xc_sm.h:1337-1428 (single tile, non-ARCTIC)             */
/* a points at a(1-nbdy,1-nbdy,1); nlev slices of ld1*ld2 each.        */
/* ------------------------------------------------------------------ */
void hyo_xctilr(const hyo_grid *g, double *a, int nlev, int mh, int nh) {
  if (g->nreg < 0) return; /* a tile of a decomposed basin: its halo is exchanged by the caller */
  const int ii = g->ii, jj = g->jj, nbdy = g->nbdy;
  const size_t sl = (size_t)g->ld1 * g->ld2;
  const double vland = 0.0; /* mod_xc_sm.h:841 */
  int mhl = mh < nbdy ? mh : nbdy;
  if (mhl < 0) mhl = 0;
  int nhl = nh < nbdy ? nh : nbdy;
  if (nhl < 0) nhl = 0;
  for (int k = 0; k < nlev; k++) {
    double *s = a + (size_t)k * sl;
    if (nhl > 0) {
      if (g->nreg <= 2) {
        for (int j = 1; j <= nhl; j++)
          for (int i = 1; i <= ii; i++) {
            s[P(g, i, 1 - j)] = vland;
            s[P(g, i, jj + j)] = vland;
          }
      } else {
        for (int j = 1; j <= nhl; j++)
          for (int i = 1; i <= ii; i++) {
            s[P(g, i, 1 - j)] = s[P(g, i, jj + 1 - j)];
            s[P(g, i, jj + j)] = s[P(g, i, j)];
          }
      }
    }
    if (mhl > 0) {
      if (g->nreg == 0 || g->nreg == 4) {
        for (int j = 1 - nhl; j <= jj + nhl; j++)
          for (int i = 1; i <= mhl; i++) {
            s[P(g, 1 - i, j)] = vland;
            s[P(g, ii + i, j)] = vland;
          }
      } else {
        for (int j = 1 - nhl; j <= jj + nhl; j++)
          for (int i = 1; i <= mhl; i++) {
            s[P(g, 1 - i, j)] = s[P(g, ii + 1 - i, j)];
            s[P(g, ii + i, j)] = s[P(g, i, j)];
          }
      }
    }
  }
}

/* ------------------------------------------------------------------ */
/* indxi / indxj: bigrid.F90:417-530                                    */
/* ------------------------------------------------------------------ */
static int indxi(hyo_grid *g, const int32_t *ipt, int32_t *iff, int32_t *ill, int32_t *is) {
  const int nbdy = g->nbdy, ii = g->ii, jj = g->jj, ms = g->ms;
  for (int j = 1 - nbdy; j <= jj + nbdy; j++) {
    is[j + nbdy - 1] = 0;
    for (int k = 1; k <= ms; k++) {
      iff[SJ(g, j, k)] = 0;
      ill[SJ(g, j, k)] = 0;
    }
    int k = 1;
    int last = ipt[P(g, 1 - nbdy, j)];
    if (last == 1) iff[SJ(g, j, k)] = 1 - nbdy;
    for (int i = 2 - nbdy; i <= ii + nbdy; i++) {
      int v = ipt[P(g, i, j)];
      if (last == 1 && v == 0) {
        ill[SJ(g, j, k)] = i - 1;
        k = k + 1;
      } else if (last == 0 && v == 1) {
        if (k > ms) return HYO_ERR_GRID;
        iff[SJ(g, j, k)] = i;
      }
      last = v;
    }
    if (last == 1) {
      ill[SJ(g, j, k)] = ii + nbdy;
      is[j + nbdy - 1] = k;
    } else {
      is[j + nbdy - 1] = k - 1;
    }
  }
  return HYO_OK;
}

static int indxj(hyo_grid *g, const int32_t *jpt, int32_t *jf, int32_t *jl, int32_t *js) {
  const int nbdy = g->nbdy, ii = g->ii, jj = g->jj, ms = g->ms;
  for (int i = 1 - nbdy; i <= ii + nbdy; i++) {
    js[i + nbdy - 1] = 0;
    for (int k = 1; k <= ms; k++) {
      jf[SI(g, i, k)] = 0;
      jl[SI(g, i, k)] = 0;
    }
    int k = 1;
    int last = jpt[P(g, i, 1 - nbdy)];
    if (last == 1) jf[SI(g, i, k)] = 1 - nbdy;
    for (int j = 2 - nbdy; j <= jj + nbdy; j++) {
      int v = jpt[P(g, i, j)];
      if (last == 1 && v == 0) {
        jl[SI(g, i, k)] = j - 1;
        k = k + 1;
      } else if (last == 0 && v == 1) {
        if (k > ms) return HYO_ERR_GRID;
        jf[SI(g, i, k)] = j;
      }
      last = v;
    }
    if (last == 1) {
      jl[SI(g, i, k)] = jj + nbdy;
      js[i + nbdy - 1] = k;
    } else {
      js[i + nbdy - 1] = k - 1;
    }
  }
  return HYO_OK;
}

void hyo_grid_free(hyo_grid *g) {
  if (!g) return;
  void *ptrs[] = {g->ip,    g->iu,    g->iv,    g->iq,     g->ipim1,  g->ipip1,  g->ipjm1, g->ipjp1,
                  g->ifp,   g->ilp,   g->isp,   g->jfp,    g->jlp,    g->jsp,    g->scp2,  g->scp2i,
                  g->fmx,   g->fmn,   g->flx,   g->fly,    g->fldlo,  g->fmxlo,  g->fmnlo, g->fax,
                  g->fay,   g->rp,    g->rm,    g->flxdiv, g->tx1,    g->ty1,    g->fldao, g->fldan,
                  g->uloc,  g->vloc,  g->hloc,  g->dtloc,  g->ucumdt, g->vcumdt, g->flxcum,
                  g->flycum, g->lcalc, g->util1, g->util2, g->uflux, g->vflux, g->uflux2, g->vflux2};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
  free(g);
}

/* arrays of a grid of g->ld1 x g->ld2 points; the work arrays start as NaN */
static int grid_alloc(hyo_grid *g) {
  const size_t n2 = (size_t)g->ld1 * g->ld2;
  g->ip = (int32_t *)calloc(n2, 4);
  g->iu = (int32_t *)calloc(n2, 4);
  g->iv = (int32_t *)calloc(n2, 4);
  g->iq = (int32_t *)calloc(n2, 4);
  g->ipim1 = (int32_t *)calloc(n2, 4);
  g->ipip1 = (int32_t *)calloc(n2, 4);
  g->ipjm1 = (int32_t *)calloc(n2, 4);
  g->ipjp1 = (int32_t *)calloc(n2, 4);
  g->ifp = (int32_t *)calloc((size_t)g->ld2 * g->ms, 4);
  g->ilp = (int32_t *)calloc((size_t)g->ld2 * g->ms, 4);
  g->isp = (int32_t *)calloc((size_t)g->ld2, 4);
  g->jfp = (int32_t *)calloc((size_t)g->ld1 * g->ms, 4);
  g->jlp = (int32_t *)calloc((size_t)g->ld1 * g->ms, 4);
  g->jsp = (int32_t *)calloc((size_t)g->ld1, 4);
  g->scp2 = (double *)malloc(n2 * 8);
  g->scp2i = (double *)malloc(n2 * 8);
  double **work[] = {&g->fmx,   &g->fmn,   &g->flx,    &g->fly,    &g->fldlo,  &g->fmxlo,  &g->fmnlo,
                     &g->fax,   &g->fay,   &g->rp,     &g->rm,     &g->flxdiv, &g->tx1,    &g->ty1,
                     &g->fldao, &g->fldan, &g->uloc,   &g->vloc,   &g->hloc,   &g->dtloc,  &g->ucumdt,
                     &g->vcumdt, &g->flxcum, &g->flycum, &g->util1, &g->util2, &g->uflux, &g->vflux};
  int bad = !g->ip || !g->iu || !g->iv || !g->iq || !g->ipim1 || !g->ipip1 || !g->ipjm1 || !g->ipjp1 ||
            !g->ifp || !g->ilp || !g->isp || !g->jfp || !g->jlp || !g->jsp || !g->scp2 || !g->scp2i;
  for (size_t k = 0; k < sizeof(work) / sizeof(work[0]); k++) {
    *work[k] = nan_array(n2);
    bad |= (*work[k] == NULL);
  }
  g->lcalc = (unsigned char *)calloc(n2, 1);
  g->uflux2 = (double *)calloc(n2, 8);
  g->vflux2 = (double *)calloc(n2, 8);
  bad |= !g->uflux2 || !g->vflux2 || !g->lcalc;
  if (bad) {
    hyo_grid_free(g);
    return HYO_ERR_MEM;
  }
  return HYO_OK;
}

/* sea-only neighbour indices (bigrid.F90:316-333; outer ring = self) and
   the sea sections (indxi/indxj) from ip */
static int grid_finish(hyo_grid *g) {
  const int ii = g->ii, jj = g->jj, nbdy = g->nbdy;
  for (int j = 1 - nbdy; j <= jj + nbdy; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++) {
      size_t c = P(g, i, j);
      g->ipim1[c] = i;
      g->ipip1[c] = i;
      g->ipjm1[c] = j;
      g->ipjp1[c] = j;
    }
  for (int j = 2 - nbdy; j <= jj + nbdy - 1; j++)
    for (int i = 2 - nbdy; i <= ii + nbdy - 1; i++) {
      size_t c = P(g, i, j);
      g->ipim1[c] = g->ip[P(g, i - 1, j)] != 0 ? i - 1 : i;
      g->ipip1[c] = g->ip[P(g, i + 1, j)] != 0 ? i + 1 : i;
      g->ipjm1[c] = g->ip[P(g, i, j - 1)] != 0 ? j - 1 : j;
      g->ipjp1[c] = g->ip[P(g, i, j + 1)] != 0 ? j + 1 : j;
    }
  if (indxi(g, g->ip, g->ifp, g->ilp, g->isp) != HYO_OK || indxj(g, g->ip, g->jfp, g->jlp, g->jsp) != HYO_OK)
    return HYO_ERR_GRID;
  return HYO_OK;
}

/*
 * bigrid: bigrid.F90:1-415 for a single tile (i0=j0=0, ii=itdm, jj=jtdm),
 * mapflg != 4 (no f-plane).  depth is (ld1*ld2) with halo; it is modified
 * in place exactly as bigrid does (halo fill, land borders).
 * Returns a new grid or NULL with *err set:
 *   HYO_ERR_GRID   arctic (north row has sea), 1-point sea, or ms overflow.
 */
hyo_grid *hyo_grid_create(int idm, int jdm, int nbdy, double *depth, const double *scp2,
                          const double *scp2i, int *err, int *nfill) {
  *err = HYO_OK;
  if (nfill) *nfill = 0;
  if (idm < 1 || jdm < 1 || nbdy < 1) {
    *err = HYO_ERR_ARG;
    return NULL;
  }
  hyo_grid *g = (hyo_grid *)calloc(1, sizeof(hyo_grid));
  if (!g) {
    *err = HYO_ERR_MEM;
    return NULL;
  }
  g->ii = idm;
  g->jj = jdm;
  g->nbdy = nbdy;
  g->ld1 = idm + 2 * nbdy;
  g->ld2 = jdm + 2 * nbdy;
  g->ms = 99; /* mod_dimensions.F90:37 */
  g->nreg = -1;
  const int ii = idm, jj = jdm;
  const size_t n2 = (size_t)g->ld1 * g->ld2;

  /* periodicity detection: bigrid.F90:25-45 */
  double depmax = 0.0;
  for (int j = 1; j <= jj; j++) depmax = mx2(depmax, depth[P(g, ii, j)]);
  int lperiod = depmax > 0.0;
  depmax = 0.0;
  for (int i = 1; i <= ii; i++) depmax = mx2(depmax, depth[P(g, i, jj)]);
  int larctic = depmax > 0.0;
  if (larctic) { /* ARCTIC tripole grids are out of scope */
    *err = HYO_ERR_GRID;
    free(g);
    return NULL;
  }
  g->nreg = lperiod ? 1 : 0; /* bigrid.F90:59-91, TYPE=one */
  g->lperiod = lperiod;

  hyo_xctilr(g, depth, 1, nbdy, nbdy); /* bigrid.F90:115 */
  /* land borders: bigrid.F90:117-154 */
  for (int j = 1 - nbdy; j <= 0; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++) depth[P(g, i, j)] = 0.0;
  for (int j = jj + 1; j <= jj + nbdy; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++) depth[P(g, i, j)] = 0.0;
  if (!lperiod) {
    for (int j = 1 - nbdy; j <= jj + nbdy; j++)
      for (int i = 1 - nbdy; i <= 0; i++) depth[P(g, i, j)] = 0.0;
    for (int j = 1 - nbdy; j <= jj + nbdy; j++)
      for (int i = ii + 1; i <= ii + nbdy; i++) depth[P(g, i, j)] = 0.0;
  }
  /* 1-point seas: bigrid.F90:156-191 */
  int rnfill = 0;
  for (int j = 1; j <= jj; j++)
    for (int i = 1; i <= ii; i++) {
      if (depth[P(g, i, j)] > 0.0) {
        int nzero = 0;
        if (depth[P(g, i - 1, j)] <= 0.0) nzero++;
        if (depth[P(g, i + 1, j)] <= 0.0) nzero++;
        if (depth[P(g, i, j - 1)] <= 0.0) nzero++;
        if (depth[P(g, i, j + 1)] <= 0.0) nzero++;
        if (nzero == 4) rnfill++;
      }
    }
  if (nfill) *nfill = rnfill;
  if (rnfill > 0) {
    *err = HYO_ERR_GRID;
    free(g);
    return NULL;
  }
  if (grid_alloc(g) != HYO_OK) {
    *err = HYO_ERR_MEM;
    return NULL;
  }
  memcpy(g->scp2, scp2, n2 * 8);
  memcpy(g->scp2i, scp2i, n2 * 8);
  /* masks: bigrid.F90:193-290 */
  for (int j = 1 - nbdy; j <= jj + nbdy; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++)
      if (depth[P(g, i, j)] > 0.) g->ip[P(g, i, j)] = 1;
  double *u1 = nan_array(n2), *u2 = nan_array(n2), *u3 = nan_array(n2);
  if (!u1 || !u2 || !u3) {
    free(u1);
    free(u2);
    free(u3);
    hyo_grid_free(g);
    *err = HYO_ERR_MEM;
    return NULL;
  }
  for (int j = 1; j <= jj; j++)
    for (int i = 1; i <= ii; i++) {
      size_t c = P(g, i, j);
      int32_t *ip = g->ip;
      int iuv = 0, ivv = 0, iqv = 0;
      if (ip[P(g, i - 1, j)] > 0 && ip[c] > 0) iuv = 1;
      if (ip[P(g, i, j - 1)] > 0 && ip[c] > 0) ivv = 1;
      int mn = ip[c];
      if (ip[P(g, i - 1, j)] < mn) mn = ip[P(g, i - 1, j)];
      if (ip[P(g, i, j - 1)] < mn) mn = ip[P(g, i, j - 1)];
      if (ip[P(g, i - 1, j - 1)] < mn) mn = ip[P(g, i - 1, j - 1)];
      if (mn > 0)
        iqv = 1;
      else if ((ip[c] > 0 && ip[P(g, i - 1, j - 1)] > 0) || (ip[P(g, i - 1, j)] > 0 && ip[P(g, i, j - 1)] > 0))
        iqv = 1;
      u1[c] = iuv;
      u2[c] = ivv;
      u3[c] = iqv;
    }
  hyo_xctilr(g, u1, 1, nbdy, nbdy);
  hyo_xctilr(g, u2, 1, nbdy, nbdy);
  hyo_xctilr(g, u3, 1, nbdy, nbdy);
  for (int j = 1 - nbdy; j <= jj + nbdy; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++) {
      size_t c = P(g, i, j);
      /* halo corners beyond nbdy-filled range stay NaN -> treat as land */
      g->iu[c] = (u1[c] == u1[c]) ? (int32_t)u1[c] : 0;
      g->iv[c] = (u2[c] == u2[c]) ? (int32_t)u2[c] : 0;
      g->iq[c] = (u3[c] == u3[c]) ? (int32_t)u3[c] : 0;
    }
  free(u1);
  free(u2);
  free(u3);
  /* part II land borders */
  for (int j = 1 - nbdy; j <= 0; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++) g->iq[P(g, i, j)] = g->iu[P(g, i, j)] = g->iv[P(g, i, j)] = 0;
  for (int j = jj + 1; j <= jj + nbdy; j++)
    for (int i = 1 - nbdy; i <= ii + nbdy; i++) g->iq[P(g, i, j)] = g->iu[P(g, i, j)] = g->iv[P(g, i, j)] = 0;
  if (!lperiod) {
    for (int j = 1 - nbdy; j <= jj + nbdy; j++)
      for (int i = 1 - nbdy; i <= 0; i++) g->iq[P(g, i, j)] = g->iu[P(g, i, j)] = g->iv[P(g, i, j)] = 0;
    for (int j = 1 - nbdy; j <= jj + nbdy; j++)
      for (int i = ii + 1; i <= ii + nbdy; i++) g->iq[P(g, i, j)] = g->iu[P(g, i, j)] = g->iv[P(g, i, j)] = 0;
  }
  if (grid_finish(g) != HYO_OK) {
    hyo_grid_free(g);
    *err = HYO_ERR_GRID;
    return NULL;
  }
  return g;
}

/*
 * A grid with given masks: one tile of a decomposed basin (its window of
 * the basin's ip/iu/iv with halo, ld1*ld2 each).  nreg < 0: the tile's
 * halos are exchanged by the caller, xctilr leaves them alone.
 */
hyo_grid *hyo_grid_from_masks(int idm, int jdm, int nbdy, int nreg, const int32_t *ip, const int32_t *iu,
                              const int32_t *iv, const double *scp2, const double *scp2i, int *err) {
  *err = HYO_OK;
  if (idm < 1 || jdm < 1 || nbdy < 1 || !ip || !iu || !iv || !scp2 || !scp2i) {
    *err = HYO_ERR_ARG;
    return NULL;
  }
  hyo_grid *g = (hyo_grid *)calloc(1, sizeof(hyo_grid));
  if (!g) {
    *err = HYO_ERR_MEM;
    return NULL;
  }
  g->ii = idm;
  g->jj = jdm;
  g->nbdy = nbdy;
  g->ld1 = idm + 2 * nbdy;
  g->ld2 = jdm + 2 * nbdy;
  g->ms = 99;
  g->nreg = nreg;
  g->lperiod = nreg == 1 || nreg == 3;
  const size_t n2 = (size_t)g->ld1 * g->ld2;
  if (grid_alloc(g) != HYO_OK) {
    *err = HYO_ERR_MEM;
    return NULL;
  }
  memcpy(g->scp2, scp2, n2 * 8);
  memcpy(g->scp2i, scp2i, n2 * 8);
  memcpy(g->ip, ip, n2 * 4);
  memcpy(g->iu, iu, n2 * 4);
  memcpy(g->iv, iv, n2 * 4);
  if (grid_finish(g) != HYO_OK) {
    hyo_grid_free(g);
    *err = HYO_ERR_GRID;
    return NULL;
  }
  return g;
}

/* accessors used by the Python wrapper */
int hyo_grid_nreg(const hyo_grid *g) { return g->nreg; }
void hyo_grid_masks(const hyo_grid *g, int32_t *ip, int32_t *iu, int32_t *iv, int32_t *ipim1, int32_t *ipip1,
                    int32_t *ipjm1, int32_t *ipjp1) {
  size_t n2 = (size_t)g->ld1 * g->ld2 * 4;
  memcpy(ip, g->ip, n2);
  memcpy(iu, g->iu, n2);
  memcpy(iv, g->iv, n2);
  memcpy(ipim1, g->ipim1, n2);
  memcpy(ipip1, g->ipip1, n2);
  memcpy(ipjm1, g->ipjm1, n2);
  memcpy(ipjp1, g->ipjp1, n2);
}
/* copy one named work array out (for stage-by-stage comparisons) */
int hyo_grid_work(const hyo_grid *g, const char *name, double *out) {
  struct {
    const char *n;
    double *a;
  } t[] = {{"fmx", g->fmx},     {"fmn", g->fmn},       {"flx", g->flx},       {"fly", g->fly},
           {"fldlo", g->fldlo}, {"fmxlo", g->fmxlo},   {"fmnlo", g->fmnlo},   {"fax", g->fax},
           {"fay", g->fay},     {"rp", g->rp},         {"rm", g->rm},         {"flxdiv", g->flxdiv},
           {"fldao", g->fldao}, {"fldan", g->fldan},   {"util1", g->util1},   {"util2", g->util2},
           {"hloc", g->hloc},   {"flxcum", g->flxcum}, {"flycum", g->flycum}, {"tx1", g->tx1}};
  for (size_t k = 0; k < sizeof(t) / sizeof(t[0]); k++)
    if (!strcmp(t[k].n, name)) {
      memcpy(out, t[k].a, (size_t)g->ld1 * g->ld2 * 8);
      return HYO_OK;
    }
  return HYO_ERR_ARG;
}

/* ------------------------------------------------------------------ */
/* section-edge zeroing of a u-face / v-face array                      */
/* (mod_tsadvc.F90:738-758 and the copies at :299-321, :835-855, ...)  */
/* ------------------------------------------------------------------ */
static void zero_sections(const hyo_grid *g, double *fx, double *fy, int margin) {
  const int ii = g->ii, jj = g->jj;
  for (int j = 1 - margin; j <= jj + margin; j++) {
    int ns = g->isp[j + g->nbdy - 1];
    for (int l = 1; l <= ns; l++) {
      int f = g->ifp[SJ(g, j, l)], la = g->ilp[SJ(g, j, l)];
      if (f >= 1 - margin) fx[P(g, f, j)] = 0.0;
      if (la < ii + margin) fx[P(g, la + 1, j)] = 0.0;
    }
  }
  for (int i = 1 - margin; i <= ii + margin; i++) {
    int ns = g->jsp[i + g->nbdy - 1];
    for (int l = 1; l <= ns; l++) {
      int f = g->jfp[SI(g, i, l)], la = g->jlp[SI(g, i, l)];
      if (f >= 1 - margin) fy[P(g, i, f)] = 0.0;
      if (la < jj + margin) fy[P(g, i, la + 1)] = 0.0;
    }
  }
}

/* ------------------------------------------------------------------ */
/* advem_fct2: mod_tsadvc.F90:645-997                                   */
/* ------------------------------------------------------------------ */
static void advem_fct2(hyo_grid *g, double *fld, const double *fldc, const double *u, const double *v,
                       const double *fco, const double *fcn, const double *scal, const double *scali, double dt2) {
  const int ii = g->ii, jj = g->jj, ld = g->ld1;
  const int mbdy_a = 5;
  int margin;
  double *fmx = g->fmx, *fmn = g->fmn, *flx = g->flx, *fly = g->fly, *fldlo = g->fldlo, *fmxlo = g->fmxlo,
         *fmnlo = g->fmnlo, *fax = g->fax, *fay = g->fay, *rp = g->rp, *rm = g->rm, *flxdiv = g->flxdiv,
         *fldao = g->fldao, *fldan = g->fldan;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;

  margin = mbdy_a - 1; /* :686-720 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double q;
      if (iu[c] != 0) {
        if (u[c] >= 0.0) q = fld[c - 1];
        else q = fld[c];
        flx[c] = u[c] * q;
      }
      if (iv[c] != 0) {
        if (v[c] >= 0.0) q = fld[c - ld];
        else q = fld[c];
        fly[c] = v[c] * q;
      }
      if (ip[c] != 0) {
        int ia = g->ipim1[c], ib = g->ipip1[c], ja = g->ipjm1[c], jb = g->ipjp1[c];
        double a0 = fld[c], a1 = fld[P(g, ia, j)], a2 = fld[P(g, ib, j)], a3 = fld[P(g, i, ja)],
               a4 = fld[P(g, i, jb)];
        fmx[c] = mx5(a0, a1, a2, a3, a4);
        fmn[c] = mn5(a0, a1, a2, a3, a4);
      }
    }
  zero_sections(g, flx, fly, margin); /* :738-758 */

  margin = mbdy_a - 2; /* :778-797 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        flxdiv[c] = ((flx[c + 1] - flx[c]) + (fly[c + ld] - fly[c])) * dt2 * scali[c];
        double q = fld[c] * (fco[c] + ONEMU) - flxdiv[c];
        fldlo[c] = mx2(fmn[c], mn2(fmx[c], q / (fcn[c] + ONEMU)));
        fmxlo[c] = mx3(fld[c], fldc[c], fldlo[c]);
        fmnlo[c] = mn3(fld[c], fldc[c], fldlo[c]);
      }
    }

  margin = mbdy_a - 2; /* :817-833 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (iu[c] != 0) {
        double fhx = u[c] * 0.5 * (fldc[c] + fldc[c - 1]);
        fax[c] = fhx - flx[c];
      }
      if (iv[c] != 0) {
        double fhy = v[c] * 0.5 * (fldc[c] + fldc[c - ld]);
        fay[c] = fhy - fly[c];
      }
    }
  zero_sections(g, fax, fay, margin); /* :835-855 */

  margin = mbdy_a - 3; /* :863-909 */
  const double qdt2 = 1.0 / dt2;
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        int ia = g->ipim1[c], ib = g->ipip1[c], ja = g->ipjm1[c], jb = g->ipjp1[c];
        double fqmax = mx5(fmxlo[c], fmxlo[P(g, ia, j)], fmxlo[P(g, ib, j)], fmxlo[P(g, i, ja)], fmxlo[P(g, i, jb)]);
        double fqmin = mn5(fmnlo[c], fmnlo[P(g, ia, j)], fmnlo[P(g, ib, j)], fmnlo[P(g, i, ja)], fmnlo[P(g, i, jb)]);
        double faxb = fax[P(g, ib, j)], fayb = fay[P(g, i, jb)];
        double famax = mx2(0.0, fax[c]) - mn2(0.0, faxb) + mx2(0.0, fay[c]) - mn2(0.0, fayb);
        double famin = mx2(0.0, faxb) - mn2(0.0, fax[c]) + mx2(0.0, fayb) - mn2(0.0, fay[c]);
        if (famax > 0.0) {
          double qp = (fqmax - fldlo[c]) * fcn[c] * scal[c] * qdt2;
          rp[c] = (qp < famax) ? qp / famax : 1.0;
        } else {
          rp[c] = 0.0;
        }
        if (famin > 0.0) {
          double qm = (fldlo[c] - fqmin) * fcn[c] * scal[c] * qdt2;
          rm[c] = (qm < famin) ? qm / famin : 1.0;
        } else {
          rm[c] = 0.0;
        }
        fmx[c] = fqmax;
        fmn[c] = fqmin;
      }
    }

  margin = mbdy_a - 4; /* :922-946 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double fact;
      if (iu[c] != 0) {
        if (fax[c] < 0.0) fact = mn2(rp[c - 1], rm[c]);
        else fact = mn2(rp[c], rm[c - 1]);
        fax[c] = fact * fax[c];
      }
      if (iv[c] != 0) {
        if (fay[c] < 0.0) fact = mn2(rp[c - ld], rm[c]);
        else fact = mn2(rp[c], rm[c - ld]);
        fay[c] = fact * fay[c];
      }
    }

  margin = mbdy_a - 5; /* :962-982 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        fldao[c] = fld[c] * fco[c] * scal[c];
        flxdiv[c] = ((fax[c + 1] - fax[c]) + (fay[c + ld] - fay[c])) * dt2 * scali[c];
        fld[c] = mx2(fmn[c], mn2(fmx[c], fldlo[c] - flxdiv[c] / (fcn[c] + ONEMU)));
        fldan[c] = fld[c] * fcn[c] * scal[c];
      }
    }
}

/* ------------------------------------------------------------------ */
/* advem_fct4: mod_tsadvc.F90:1370-1706                                 */
/* ------------------------------------------------------------------ */
static void advem_fct4(hyo_grid *g, double *fld, const double *fldc, const double *u, const double *v,
                       const double *fco, const double *fcn, const double *scal, const double *scali, double dt2) {
  const int ii = g->ii, jj = g->jj, ld = g->ld1;
  const int mbdy_a = 5;
  const double ft14 = 7.0 / 12.0, ft24 = -1.0 / 12.0; /* :1398-1399 */
  int margin;
  double *fmx = g->fmx, *fmn = g->fmn, *flx = g->flx, *fly = g->fly, *fldlo = g->fldlo, *fmxlo = g->fmxlo,
         *fmnlo = g->fmnlo, *fax = g->fax, *fay = g->fay, *rp = g->rp, *rm = g->rm, *flxdiv = g->flxdiv,
         *fldao = g->fldao, *fldan = g->fldan;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;

  margin = mbdy_a - 1; /* :1414-1448 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double q;
      if (iu[c] != 0) {
        if (u[c] >= 0.0) q = fld[c - 1];
        else q = fld[c];
        flx[c] = u[c] * q;
      }
      if (iv[c] != 0) {
        if (v[c] >= 0.0) q = fld[c - ld];
        else q = fld[c];
        fly[c] = v[c] * q;
      }
      if (ip[c] != 0) {
        int ia = g->ipim1[c], ib = g->ipip1[c], ja = g->ipjm1[c], jb = g->ipjp1[c];
        double a0 = fld[c], a1 = fld[P(g, ia, j)], a2 = fld[P(g, ib, j)], a3 = fld[P(g, i, ja)],
               a4 = fld[P(g, i, jb)];
        fmx[c] = mx5(a0, a1, a2, a3, a4);
        fmn[c] = mn5(a0, a1, a2, a3, a4);
      }
    }
  zero_sections(g, flx, fly, margin);

  margin = mbdy_a - 2; /* :1497-1516 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        flxdiv[c] = ((flx[c + 1] - flx[c]) + (fly[c + ld] - fly[c])) * dt2 * scali[c];
        double q = fld[c] * (fco[c] + ONEMU) - flxdiv[c];
        fldlo[c] = mx2(fmn[c], mn2(fmx[c], q / (fcn[c] + ONEMU)));
        fmxlo[c] = mx3(fld[c], fldc[c], fldlo[c]);
        fmnlo[c] = mn3(fld[c], fldc[c], fldlo[c]);
      }
    }

  margin = mbdy_a - 2; /* :1528-1558 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double fhx, fhy;
      if (iu[c] != 0) {
        if (iu[c - 1] == 0 || iu[c + 1] == 0)
          fhx = u[c] * 0.5 * (fldc[c] + fldc[c - 1]);
        else
          fhx = u[c] * (ft14 * (fldc[c] + fldc[c - 1]) + ft24 * (fldc[c + 1] + fldc[c - 2]));
        fax[c] = fhx - flx[c];
      }
      if (iv[c] != 0) {
        if (iv[c - ld] == 0 || iv[c + ld] == 0)
          fhy = v[c] * 0.5 * (fldc[c] + fldc[c - ld]);
        else
          fhy = v[c] * (ft14 * (fldc[c] + fldc[c - ld]) + ft24 * (fldc[c + ld] + fldc[c - 2 * ld]));
        fay[c] = fhy - fly[c];
      }
    }
  zero_sections(g, fax, fay, margin);

  margin = mbdy_a - 3; /* :1588-1634 */
  const double qdt2 = 1.0 / dt2;
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        int ia = g->ipim1[c], ib = g->ipip1[c], ja = g->ipjm1[c], jb = g->ipjp1[c];
        double fqmax = mx5(fmxlo[c], fmxlo[P(g, ia, j)], fmxlo[P(g, ib, j)], fmxlo[P(g, i, ja)], fmxlo[P(g, i, jb)]);
        double fqmin = mn5(fmnlo[c], fmnlo[P(g, ia, j)], fmnlo[P(g, ib, j)], fmnlo[P(g, i, ja)], fmnlo[P(g, i, jb)]);
        double faxb = fax[P(g, ib, j)], fayb = fay[P(g, i, jb)];
        double famax = mx2(0.0, fax[c]) - mn2(0.0, faxb) + mx2(0.0, fay[c]) - mn2(0.0, fayb);
        double famin = mx2(0.0, faxb) - mn2(0.0, fax[c]) + mx2(0.0, fayb) - mn2(0.0, fay[c]);
        if (famax > 0.0) {
          double qp = (fqmax - fldlo[c]) * fcn[c] * scal[c] * qdt2;
          rp[c] = (qp < famax) ? qp / famax : 1.0;
        } else {
          rp[c] = 0.0;
        }
        if (famin > 0.0) {
          double qm = (fldlo[c] - fqmin) * fcn[c] * scal[c] * qdt2;
          rm[c] = (qm < famin) ? qm / famin : 1.0;
        } else {
          rm[c] = 0.0;
        }
        fmx[c] = fqmax;
        fmn[c] = fqmin;
      }
    }

  margin = mbdy_a - 4; /* :1639-1663 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double fact;
      if (iu[c] != 0) {
        if (fax[c] < 0.0) fact = mn2(rp[c - 1], rm[c]);
        else fact = mn2(rp[c], rm[c - 1]);
        fax[c] = fact * fax[c];
      }
      if (iv[c] != 0) {
        if (fay[c] < 0.0) fact = mn2(rp[c - ld], rm[c]);
        else fact = mn2(rp[c], rm[c - ld]);
        fay[c] = fact * fay[c];
      }
    }

  margin = mbdy_a - 5; /* :1679-1699 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        fldao[c] = fld[c] * fco[c] * scal[c];
        flxdiv[c] = ((fax[c + 1] - fax[c]) + (fay[c + ld] - fay[c])) * dt2 * scali[c];
        fld[c] = mx2(fmn[c], mn2(fmx[c], fldlo[c] - flxdiv[c] / (fcn[c] + ONEMU)));
        fldan[c] = fld[c] * fcn[c] * scal[c];
      }
    }
}

/* ------------------------------------------------------------------ */
/* advem_pcm: mod_tsadvc.F90:495-643                                    */
/* ------------------------------------------------------------------ */
static void advem_pcm(hyo_grid *g, double *fld, const double *u, const double *v, const double *fco,
                      const double *fcn, const double *scal, const double *scali, double dt2) {
  const int ii = g->ii, jj = g->jj, ld = g->ld1;
  const int mbdy_a = 2;
  int margin;
  double *fmx = g->fmx, *fmn = g->fmn, *flx = g->flx, *fly = g->fly, *flxdiv = g->flxdiv, *fldao = g->fldao,
         *fldan = g->fldan;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;

  margin = mbdy_a - 1; /* :529-563 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double q;
      if (iu[c] != 0) {
        if (u[c] >= 0.0) q = fld[c - 1];
        else q = fld[c];
        flx[c] = u[c] * q;
      }
      if (iv[c] != 0) {
        if (v[c] >= 0.0) q = fld[c - ld];
        else q = fld[c];
        fly[c] = v[c] * q;
      }
      if (ip[c] != 0) {
        int ia = g->ipim1[c], ib = g->ipip1[c], ja = g->ipjm1[c], jb = g->ipjp1[c];
        double a0 = fld[c], a1 = fld[P(g, ia, j)], a2 = fld[P(g, ib, j)], a3 = fld[P(g, i, ja)],
               a4 = fld[P(g, i, jb)];
        fmx[c] = mx5(a0, a1, a2, a3, a4);
        fmn[c] = mn5(a0, a1, a2, a3, a4);
      }
    }
  zero_sections(g, flx, fly, margin); /* :571-591 */

  margin = mbdy_a - 2; /* :610-630 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        fldao[c] = fld[c] * fco[c] * scal[c];
        flxdiv[c] = ((flx[c + 1] - flx[c]) + (fly[c + ld] - fly[c])) * dt2 * scali[c];
        double q = fld[c] * (fco[c] + ONEMU) - flxdiv[c];
        fld[c] = mx2(fmn[c], mn2(fmx[c], q / (fcn[c] + ONEMU)));
        fldan[c] = fld[c] * fcn[c] * scal[c];
      }
    }
}

/* ------------------------------------------------------------------ */
/* advem_mpdata: mod_tsadvc.F90:207-493                                 */
/* ------------------------------------------------------------------ */
static void advem_mpdata(hyo_grid *g, double *fld, const double *u, const double *v, const double *fco,
                         const double *fcn, double posdef, const double *scal, const double *scali, double dt2) {
  const int ii = g->ii, jj = g->jj, ld = g->ld1, nbdy = g->nbdy;
  const int mbdy_a = 5;
  int margin;
  double *fmx = g->fmx, *fmn = g->fmn, *flx = g->flx, *fly = g->fly, *fldlo = g->fldlo, *rp = g->rp,
         *rm = g->rm, *flxdiv = g->flxdiv, *tx1 = g->tx1, *ty1 = g->ty1, *fldao = g->fldao, *fldan = g->fldan;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;

  margin = mbdy_a - 1; /* :248-284 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double q;
      if (iu[c] != 0) {
        tx1[c] = .5 * fabs(u[c]) * (fld[c] - fld[c - 1]);
        if (u[c] >= 0.0) q = fld[c - 1];
        else q = fld[c];
        flx[c] = u[c] * (q + posdef);
      }
      if (iv[c] != 0) {
        ty1[c] = .5 * fabs(v[c]) * (fld[c] - fld[c - ld]);
        if (v[c] >= 0.0) q = fld[c - ld];
        else q = fld[c];
        fly[c] = v[c] * (q + posdef);
      }
      if (ip[c] != 0) {
        int ia = g->ipim1[c], ib = g->ipip1[c], ja = g->ipjm1[c], jb = g->ipjp1[c];
        double a0 = fld[c], a1 = fld[P(g, ia, j)], a2 = fld[P(g, ib, j)], a3 = fld[P(g, i, ja)],
               a4 = fld[P(g, i, jb)];
        fmx[c] = mx5(a0, a1, a2, a3, a4) + posdef;
        fmn[c] = mn5(a0, a1, a2, a3, a4) + posdef;
      }
    }
  zero_sections(g, flx, fly, margin); /* :299-321 */

  margin = mbdy_a - 2; /* :340-357 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        flxdiv[c] = ((flx[c + 1] - flx[c]) + (fly[c + ld] - fly[c])) * dt2 * scali[c];
        double q = (fld[c] + posdef) * (fco[c] + ONEMU) - flxdiv[c];
        fldlo[c] = mx2(fmn[c], mn2(fmx[c], q / (fcn[c] + ONEMU)));
      }
    }

  margin = mbdy_a - 2; /* :369-392 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++) {
    double fco2 = 0.0, fcn2 = 0.0;
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (iu[c] != 0) {
        fco2 = fco[c] + fco[c - 1];
        fcn2 = fcn[c] + fcn[c - 1];
        flx[c] = tx1[c] - u[c] * (flxdiv[c] + flxdiv[c - 1]) / ((fco2 + fcn2) + ONEMU);
      }
      if (iv[c] != 0) {
        fco2 = fco[c] + fco[c - ld];
        fcn2 = fcn[c] + fcn[c - ld];
        fly[c] = ty1[c] - v[c] * (flxdiv[c] + flxdiv[c - ld]) / ((fco2 + fcn2) + ONEMU);
      }
    }
    if (fco2 * fcn2 == 1.e30) flx[P(g, 1 - nbdy, j)] = 0.0; /* :390, ordering guard */
  }

  margin = mbdy_a - 3; /* :405-423 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        double flxdp = mn2(0.0, flx[c + 1]) - mx2(0.0, flx[c]);
        double flxdn = mx2(0.0, flx[c + 1]) - mn2(0.0, flx[c]);
        double flydp = mn2(0.0, fly[c + ld]) - mx2(0.0, fly[c]);
        double flydn = mx2(0.0, fly[c + ld]) - mn2(0.0, fly[c]);
        rp[c] = (fmx[c] - fldlo[c]) * (fcn[c] * scal[c]) / ((ONEMU - (flxdp + flydp)) * dt2);
        rm[c] = (fldlo[c] - fmn[c]) * (fcn[c] * scal[c]) / ((ONEMU + (flxdn + flydn)) * dt2);
      }
    }

  margin = mbdy_a - 4; /* :433-449 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (iu[c] != 0) {
        flx[c] = mx2(0.0, flx[c]) * mn3(1.0, rp[c], rm[c - 1]) + mn2(0.0, flx[c]) * mn3(1.0, rp[c - 1], rm[c]);
      }
      if (iv[c] != 0) {
        fly[c] = mx2(0.0, fly[c]) * mn3(1.0, rp[c], rm[c - ld]) + mn2(0.0, fly[c]) * mn3(1.0, rp[c - ld], rm[c]);
      }
    }

  margin = mbdy_a - 5; /* :465-486 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        fldao[c] = fld[c] * fco[c] * scal[c];
        flxdiv[c] = ((flx[c + 1] - flx[c]) + (fly[c + ld] - fly[c])) * dt2 * scali[c];
        fld[c] = mx2(fmn[c], mn2(fmx[c], fldlo[c] - flxdiv[c] / (fcn[c] + ONEMU)));
        fld[c] = fld[c] - posdef;
        fldan[c] = fld[c] * fcn[c] * scal[c];
      }
    }
}

/* ------------------------------------------------------------------ */
/* advem_fct2c: mod_tsadvc.F90:999-1368 (btrmas, sub-cycled donor cell) */
/* ------------------------------------------------------------------ */
static void advem_fct2c(hyo_grid *g, double *fld, const double *fldc, const double *u, const double *v,
                        const double *fco, const double *fcn, const double *scal, const double *scali, double dt2) {
  const int ii = g->ii, jj = g->jj, ld = g->ld1;
  const int mbdy_a = 5;
  const size_t n2 = (size_t)g->ld1 * g->ld2;
  int margin;
  (void)fcn;
  double *fmx = g->fmx, *fmn = g->fmn, *flx = g->flx, *fly = g->fly, *fldlo = g->fldlo, *fax = g->fax,
         *fay = g->fay, *rp = g->rp, *rm = g->rm, *flxdiv = g->flxdiv;
  double *uloc = g->uloc, *vloc = g->vloc, *hloc = g->hloc, *dtloc = g->dtloc, *ucumdt = g->ucumdt,
         *vcumdt = g->vcumdt, *flxcum = g->flxcum, *flycum = g->flycum;
  unsigned char *lcalc = g->lcalc;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;

  /* :1068-1081 whole-array initialisation */
  for (size_t c = 0; c < n2; c++) {
    lcalc[c] = 1;
    flxcum[c] = 0.0;
    flycum[c] = 0.0;
    dtloc[c] = 0.0;
    hloc[c] = fco[c];
    fldlo[c] = fld[c];
    ucumdt[c] = 0.0;
    vcumdt[c] = 0.0;
    uloc[c] = 0.0;
    vloc[c] = 0.0;
    flx[c] = 0.0;
    fly[c] = 0.0;
  }

  for (int iter = 1; iter <= 5; iter++) { /* :1083-1192 */
    margin = mbdy_a;
#pragma omp parallel for schedule(static) num_threads(nthr(g))
    for (int j = 1 - margin; j <= jj + margin; j++)
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] != 0) {
          double q = mx2(u[c + 1], 0.0) - mn2(u[c], 0.0) + mx2(v[c + ld], 0.0) - mn2(v[c], 0.0);
          if (q > 0.0) dtloc[c] = mn2(dt2, hloc[c] / (q * scali[c]));
          else dtloc[c] = dt2;
        }
      }
    margin = mbdy_a - 1;
#pragma omp parallel for schedule(static) num_threads(nthr(g))
    for (int j = 1 - margin; j <= jj + margin; j++)
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (iu[c] != 0) {
          if (ucumdt[c] != dt2) {
            if (u[c] >= 0) {
              uloc[c] = mn2(dt2 - ucumdt[c], dtloc[c - 1]) * u[c];
              flx[c] = fldlo[c - 1] * uloc[c];
              ucumdt[c] = ucumdt[c] + mn2(dt2 - ucumdt[c], dtloc[c - 1]);
            } else {
              uloc[c] = mn2(dt2 - ucumdt[c], dtloc[c]) * u[c];
              flx[c] = fldlo[c] * uloc[c];
              ucumdt[c] = ucumdt[c] + mn2(dt2 - ucumdt[c], dtloc[c]);
            }
            flxcum[c] = flxcum[c] + flx[c];
          } else {
            uloc[c] = 0.0;
            flx[c] = 0.0;
          }
        }
        if (iv[c] != 0) {
          if (vcumdt[c] != dt2) {
            if (v[c] >= 0) {
              vloc[c] = mn2(dt2 - vcumdt[c], dtloc[c - ld]) * v[c];
              fly[c] = fldlo[c - ld] * vloc[c];
              vcumdt[c] = vcumdt[c] + mn2(dt2 - vcumdt[c], dtloc[c - ld]);
            } else {
              vloc[c] = mn2(dt2 - vcumdt[c], dtloc[c]) * v[c];
              fly[c] = fldlo[c] * vloc[c];
              vcumdt[c] = vcumdt[c] + mn2(dt2 - vcumdt[c], dtloc[c]);
            }
            flycum[c] = flycum[c] + fly[c];
          } else {
            vloc[c] = 0.0;
            fly[c] = 0.0;
          }
        }
      }
    margin = mbdy_a - 2;
#pragma omp parallel for schedule(static) num_threads(nthr(g))
    for (int j = 1 - margin; j <= jj + margin; j++)
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] != 0) {
          if (lcalc[c]) {
            double qp = hloc[c] - (uloc[c + 1] - uloc[c] + vloc[c + ld] - vloc[c]) * scali[c];
            if (qp > 0.0) {
              fldlo[c] = ((EPSIL + hloc[c]) * fldlo[c] - (flx[c + 1] - flx[c] + fly[c + ld] - fly[c]) * scali[c]) /
                         (EPSIL + qp);
            }
            hloc[c] = qp;
            lcalc[c] = ucumdt[c + 1] != dt2 || ucumdt[c] != dt2 || vcumdt[c + ld] != dt2 || vcumdt[c] != dt2;
          }
        }
      }
    hyo_xctilr(g, hloc, 1, mbdy_a, mbdy_a);  /* :1181 */
    hyo_xctilr(g, fldlo, 1, mbdy_a, mbdy_a); /* :1182 */
  }

  margin = mbdy_a - 2; /* :1199-1215 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (iu[c] != 0) {
        double fhx = u[c] * 0.5 * (fldc[c] + fldc[c - 1]);
        fax[c] = fhx - flxcum[c] / dt2;
      }
      if (iv[c] != 0) {
        double fhy = v[c] * 0.5 * (fldc[c] + fldc[c - ld]);
        fay[c] = fhy - flycum[c] / dt2;
      }
    }
  zero_sections(g, fax, fay, margin); /* :1223-1243 */

  margin = mbdy_a - 3; /* :1257-1303 */
  const double qdt2 = 1.0 / dt2;
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        int ia = i - 1;
        if (ip[P(g, ia, j)] == 0) ia = i;
        int ib = i + 1;
        if (ip[P(g, ib, j)] == 0) ib = i;
        int ja = j - 1;
        if (ip[P(g, i, ja)] == 0) ja = j;
        int jb = j + 1;
        if (ip[P(g, i, jb)] == 0) jb = j;
        double fqmax = mx5(fldlo[c], fldlo[P(g, ia, j)], fldlo[P(g, ib, j)], fldlo[P(g, i, ja)], fldlo[P(g, i, jb)]);
        double fqmin = mn5(fldlo[c], fldlo[P(g, ia, j)], fldlo[P(g, ib, j)], fldlo[P(g, i, ja)], fldlo[P(g, i, jb)]);
        double famax = mx2(0.0, fax[c]) - mn2(0.0, fax[c + 1]) + mx2(0.0, fay[c]) - mn2(0.0, fay[c + ld]);
        double famin = mx2(0.0, fax[c + 1]) - mn2(0.0, fax[c]) + mx2(0.0, fay[c + ld]) - mn2(0.0, fay[c]);
        if (famax > EPSIL) {
          double qp = (fqmax - fldlo[c]) * hloc[c] * scal[c] * qdt2;
          rp[c] = (qp < famax) ? qp / famax : 1.0;
        } else {
          rp[c] = 0.0;
        }
        if (famin > EPSIL) {
          double qm = (fldlo[c] - fqmin) * hloc[c] * scal[c] * qdt2;
          rm[c] = (qm < famin) ? qm / famin : 1.0;
        } else {
          rm[c] = 0.0;
        }
        fmx[c] = fqmax;
        fmn[c] = fqmin;
      }
    }

  margin = mbdy_a - 4; /* :1308-1332 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      double fact;
      if (iu[c] != 0) {
        if (fax[c] < 0.0) fact = mn2(rp[c - 1], rm[c]);
        else fact = mn2(rp[c], rm[c - 1]);
        fax[c] = fact * fax[c];
      }
      if (iv[c] != 0) {
        if (fay[c] < 0.0) fact = mn2(rp[c - ld], rm[c]);
        else fact = mn2(rp[c], rm[c - ld]);
        fay[c] = fact * fay[c];
      }
    }

  margin = mbdy_a - 5; /* :1340-1359 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        flxdiv[c] = ((fax[c + 1] - fax[c]) + (fay[c + ld] - fay[c])) * dt2 * scali[c];
        if (hloc[c] > 0.)
          fld[c] = ((EPSIL + hloc[c]) * fldlo[c] - flxdiv[c]) / (EPSIL + hloc[c]);
        else
          fld[c] = fldlo[c];
      }
    }
}

double hyo_xcsum(const hyo_grid *g, const double *a, const int32_t *mask);

/* ------------------------------------------------------------------ */
/* advem: mod_tsadvc.F90:69-205; with lconserve (:32, .false. as       */
/* shipped) the rescale of :168-203 follows the scheme                 */
/* ------------------------------------------------------------------ */
int hyo_advem(hyo_grid *g, int advtyp, double *fld, const double *fldc, const double *u, const double *v,
              const double *fco, const double *fcn, double posdef, const double *scal, const double *scali,
              double dt2, int btrmas) {
  if (advtyp == 0)
    advem_pcm(g, fld, u, v, fco, fcn, scal, scali, dt2);
  else if (advtyp == 1)
    advem_mpdata(g, fld, u, v, fco, fcn, posdef, scal, scali, dt2);
  else if (advtyp == 2 && btrmas)
    advem_fct2c(g, fld, fldc, u, v, fco, fcn, scal, scali, dt2);
  else if (advtyp == 2)
    advem_fct2(g, fld, fldc, u, v, fco, fcn, scal, scali, dt2);
  else if (advtyp == 4)
    advem_fct4(g, fld, fldc, u, v, fco, fcn, scal, scali, dt2);
  else
    return HYO_ERR_ADVTYP;
  if (g->lconserve) { /* :168-188; ipa = ip without ice shelf or tripole (geopar.F90:427-437) */
    const double sumold = hyo_xcsum(g, g->fldao, g->ip);
    const double sumnew = hyo_xcsum(g, g->fldan, g->ip);
    const double offset = sumnew != 0.0 ? (sumold - sumnew) / sumnew : 0.0;
    for (int j = 1; j <= g->jj; j++)
      for (int i = 1; i <= g->ii; i++) {
        const size_t c = P(g, i, j);
        if (g->ip[c] != 0) fld[c] = fld[c] * (1.0 + offset);
      }
  }
  return HYO_OK;
}

/* ------------------------------------------------------------------ */
/* tsadvc: mod_tsadvc.F90:1708-2132, advection part (temdf2 = 0)        */
/* ------------------------------------------------------------------ */
typedef struct hyo_tsparams {
  int kdm, advtyp, advflg, btrmas, ntracr, nhybrd, isopyc, hybrid, mxlmy, nstep, diagno;
  double delt1;
  const int32_t *trcflg; /* ntracr entries */
} hyo_tsparams;

/*
 * Fields (reference layout, mod_cb_arrays.F90):
 *   temp, saln, th3d : (ld1,ld2,kdm,2)
 *   tracer           : (ld1,ld2,kdm,2,ntracr)  (may be NULL if ntracr=0)
 *   uflx, vflx       : (ld1,ld2,kdm)
 *   dp               : (ld1,ld2,kdm,2)
 *   oneta            : (ld1,ld2,2)             (only read if btrmas)
 *   q2, q2l          : (ld1,ld2,0:kdm+1,2)     (only if mxlmy)
 * xmin/xmax (kdm) receive the salinity range diagnostic when it runs.
 * m, n are the reference's 1-based time-level indices.
 */
int hyo_tsadvc(hyo_grid *g, const hyo_tsparams *p, int m, int n, double *temp, double *saln, double *th3d,
               double *tracer, double *uflx, double *vflx, const double *dp, const double *oneta, double *q2,
               double *q2l, double *xmin, double *xmax) {
  static const int mbdy_advtyp[5] = {2, 5, 5, 0, 5}; /* :24-29 */
  const double pdzero = 0.0, pdtemp = 256.0, pdth3d = 32.0, pdq2 = 1.0;
  const int ii = g->ii, jj = g->jj, kk = p->kdm, ld = g->ld1;
  const size_t sl = (size_t)g->ld1 * g->ld2;
  if (m < 1 || m > 2 || n < 1 || n > 2 || kk < 1) return HYO_ERR_ARG;
  int at = p->advtyp < 0 ? -p->advtyp : p->advtyp;
  if (at > 4 || at == 3) return HYO_ERR_ADVTYP;
  int mbdy = mbdy_advtyp[at];
  if (g->nbdy < mbdy) return HYO_ERR_NBDY; /* :1817-1825 */
  double *util1 = g->util1, *util2 = g->util2, *uflux = g->uflux, *vflux = g->vflux;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;
  const double *scp2 = g->scp2, *scp2i = g->scp2i;
  const int mm = m - 1, nn = n - 1;

  for (size_t c = 0; c < sl; c++) { /* :1812-1813 */
    uflux[c] = 0.0;
    vflux[c] = 0.0;
  }
  /* :1829-1840 halo refresh */
  int l = mbdy;
  hyo_xctilr(g, saln, 2 * kk, l, l);
  hyo_xctilr(g, temp, 2 * kk, l, l);
  hyo_xctilr(g, th3d, 2 * kk, l, l);
  hyo_xctilr(g, uflx, kk, l, l);
  hyo_xctilr(g, vflx, kk, l, l);
  for (int ktr = 0; ktr < p->ntracr; ktr++) hyo_xctilr(g, tracer + (size_t)ktr * 2 * kk * sl, 2 * kk, l, l);
  if (p->mxlmy) {
    hyo_xctilr(g, q2, 2 * kk + 4, l, l);
    hyo_xctilr(g, q2l, 2 * kk + 4, l, l);
  }
  const int diag = (p->nstep % 3 == 0) || p->diagno;
#define F3(a, k, t) ((a) + ((size_t)(k) + (size_t)(t) * kk) * sl)         /* (…,k,t), k 0-based */
#define Q3(a, k, t) ((a) + ((size_t)(k) + (size_t)(t) * (kk + 2)) * sl) /* q2(…,0:kk+1,t), k 1-based */
  for (int k = 1; k <= kk; k++) {
    int latemp = k <= p->nhybrd && p->advflg == 0;
    int lath3d = (k <= p->nhybrd && p->advflg == 1) || (k == 1 && p->isopyc);
    const double *uk = F3(uflx, k - 1, 0), *vk = F3(vflx, k - 1, 0);
    if (p->isopyc && k == 1) { /* :1860-1897 */
      int margin = mbdy - 1;
      for (int j = 1 - margin; j <= jj + margin; j++)
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (iv[c] != 0) {
            double vfa = (iv[c - 1] != 0) ? vk[c - 1] : vk[c];
            double vfb = (iv[c + 1] != 0) ? vk[c + 1] : vk[c];
            vflux[c] = .5 * vk[c] + .25 * (vfa + vfb);
          }
          if (iu[c] != 0) {
            double ufa = (iu[c - ld] != 0) ? uk[c - ld] : uk[c];
            double ufb = (iu[c + ld] != 0) ? uk[c + ld] : uk[c];
            uflux[c] = .5 * uk[c] + .25 * (ufa + ufb);
          }
        }
    }
    const double *dpn = F3(dp, k - 1, nn);
    const int usesm = p->isopyc && k == 1;
    {
      int margin = mbdy - 1; /* :1905-1942 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
      for (int j = 1 - margin; j <= jj + margin; j++)
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (ip[c] != 0) {
            double flxdiv;
            if (usesm)
              flxdiv = ((uflux[c + 1] - uflux[c]) + (vflux[c + ld] - vflux[c])) * p->delt1 * scp2i[c];
            else
              flxdiv = ((uk[c + 1] - uk[c]) + (vk[c + ld] - vk[c])) * p->delt1 * scp2i[c];
            double ota = p->btrmas ? oneta[c + (size_t)nn * sl] : 1.0; /* onetamas(m), :1804-1810 */
            util1[c] = mx2(ota * dpn[c] + flxdiv, 0.0);
            util2[c] = mx2(ota * dpn[c], 0.0);
          }
        }
    }
    const double *ua = usesm ? uflux : uk, *va = usesm ? vflux : vk;
    int rc = HYO_OK;
    if (latemp) {
      rc |= hyo_advem(g, p->advtyp, F3(temp, k - 1, nn), F3(temp, k - 1, mm), uk, vk, util1, util2, pdtemp, scp2,
                      scp2i, p->delt1, p->btrmas);
      rc |= hyo_advem(g, p->advtyp, F3(saln, k - 1, nn), F3(saln, k - 1, mm), uk, vk, util1, util2, pdzero, scp2,
                      scp2i, p->delt1, p->btrmas);
    } else if (lath3d && p->hybrid) {
      rc |= hyo_advem(g, p->advtyp, F3(th3d, k - 1, nn), F3(th3d, k - 1, mm), uk, vk, util1, util2, pdth3d, scp2,
                      scp2i, p->delt1, p->btrmas);
      rc |= hyo_advem(g, p->advtyp, F3(saln, k - 1, nn), F3(saln, k - 1, mm), uk, vk, util1, util2, pdzero, scp2,
                      scp2i, p->delt1, p->btrmas);
    } else if (lath3d && p->isopyc) {
      rc |= hyo_advem(g, p->advtyp, F3(th3d, k - 1, nn), F3(th3d, k - 1, mm), ua, va, util1, util2, pdth3d, scp2,
                      scp2i, p->delt1, p->btrmas);
      rc |= hyo_advem(g, p->advtyp, F3(saln, k - 1, nn), F3(saln, k - 1, mm), ua, va, util1, util2, pdzero, scp2,
                      scp2i, p->delt1, p->btrmas);
    } else {
      rc |= hyo_advem(g, p->advtyp, F3(saln, k - 1, nn), F3(saln, k - 1, mm), uk, vk, util1, util2, pdzero, scp2,
                      scp2i, p->delt1, p->btrmas);
    }
    for (int ktr = 0; ktr < p->ntracr; ktr++) {
      double *tr = tracer + (size_t)ktr * 2 * kk * sl;
      double pd = (p->trcflg && p->trcflg[ktr] == 2) ? pdtemp : pdzero;
      rc |= hyo_advem(g, p->advtyp, F3(tr, k - 1, nn), F3(tr, k - 1, mm), uk, vk, util1, util2, pd, scp2, scp2i,
                      p->delt1, p->btrmas);
    }
    if (p->mxlmy) {
      rc |= hyo_advem(g, p->advtyp, Q3(q2, k, nn), Q3(q2, k, mm), uk, vk, util1, util2, pdq2, scp2, scp2i, p->delt1,
                      p->btrmas);
      rc |= hyo_advem(g, p->advtyp, Q3(q2l, k, nn), Q3(q2l, k, mm), uk, vk, util1, util2, pdq2, scp2, scp2i,
                      p->delt1, p->btrmas);
    }
    if (rc != HYO_OK) return HYO_ERR_ADVTYP;
    if (diag && xmin && xmax) { /* :2065-2084 */
      const double onemm = ONEM * 0.001; /* onemm, mod_cb_arrays.F90:851 */
      double smin = 999., smax = -999.;
      const double *sk = F3(saln, k - 1, nn), *dk = F3(dp, k - 1, nn);
      for (int j = 1; j <= jj; j++) {
        double sminy = 999., smaxy = -999.;
        for (int i = 1; i <= ii; i++) {
          size_t c = P(g, i, j);
          if (ip[c] != 0 && dk[c] > onemm) {
            sminy = mn2(sminy, sk[c]);
            smaxy = mx2(smaxy, sk[c]);
          }
        }
        smin = mn2(smin, sminy);
        smax = mx2(smax, smaxy);
      }
      xmin[k - 1] = smin;
      xmax[k - 1] = smax;
    }
  }
#undef F3
#undef Q3
  return HYO_OK;
}

/* xcsum: mod_xc_sm.h:900-963 (row sums in 2*nbdy+1 strips, then serial) */
double hyo_xcsum(const hyo_grid *g, const double *a, const int32_t *mask) {
  const int idm = g->ii, jdm = g->jj, w = 2 * g->nbdy + 1;
  if (jdm < 1) return 0.0;
  double *sj = (double *)calloc((size_t)jdm, sizeof(double));
  if (!sj) return NAN;
  for (int j = 1; j <= jdm; j++) {
    double s8 = 0.0;
    for (int i1 = 1; i1 <= idm; i1 += w) {
      double s8p = 0.0;
      int ie = i1 + w - 1 < idm ? i1 + w - 1 : idm;
      for (int i = i1; i <= ie; i++)
        if (mask[P(g, i, j)] == 1) s8p = s8p + a[P(g, i, j)];
      s8 = s8 + s8p;
    }
    sj[j - 1] = s8;
  }
  double s = sj[0];
  for (int j = 2; j <= jdm; j++) s = s + sj[j - 1];
  free(sj);
  return s;
}

/* ------------------------------------------------------------------ */
/* Lateral diffusion at the end of tsadvc: mod_tsadvc.F90:2138-2230,   */
/* tsdff_2x :2262-2350, tsdff_1x :2352-2492, with the 17-term equation */
/* of state for sigma-2 (stmt_fns.h:174-263, :496-515; EOS_17T with    */
/* EOS_SIG2, the configuration the reference's relo builds use).       */
/* ------------------------------------------------------------------ */
/* stmt_fns.h:183-218 (the coefficients of the 17-term equation of state) */
static const double c001 = 9.9984085444849347e+02, c002 = 7.3471625860981584e+00, c003 = -5.3211231792841769e-02,
                    c004 = 3.6492439109814549e-04, c005 = 2.5880571023991390e+00, c006 = 6.7168282786692355e-03,
                    c007 = 1.9203202055760151e-03, c008 = 1.0000000000000000e+00, c009 = 7.2815210113327091e-03,
                    c010 = -4.4787265461983921e-05, c011 = 3.3851002965802430e-07, c012 = 1.3651202389758572e-10,
                    c013 = 1.7632126669040377e-03, c014 = 8.8066583251206474e-06, c015 = 1.8832689434804897e-10,
                    c016 = 5.7463776745432097e-06, c017 = 1.4716275472242334e-09, c018 = 1.1798263740430364e-02,
                    c019 = 9.8920219266399117e-08, c020 = 4.6996642771754730e-06, c021 = 2.5862187075154352e-08,
                    c022 = 3.2921414007960662e-12, c023 = 6.7103246285651894e-06, c024 = 2.4461698007024582e-17,
                    c025 = 9.1534417604289062e-18;

/* sigma-2 reference pressure in dbar and the pressure-folded coefficients,
   stmt_fns.h:249-263 (constants folded in double, left to right) */
static double eos_rpdb(void) { return 2000.e4 * 1.e-4; }
double hyo_sig(double t, double s) {
  const double rpdb = eos_rpdb();
  const double c101 = c001 + (c018 - c021 * rpdb) * rpdb, c103 = c003 + (c019 - c022 * rpdb) * rpdb,
               c105 = c005 + c020 * rpdb, c108 = c008 + c023 * rpdb, c109 = c009 - c025 * (rpdb * rpdb * rpdb),
               c111 = c011 - c024 * (rpdb * rpdb);
  /* stmt_fns.h:497-502 */
  const double sn = c101 + t * (c002 + t * (c103 + t * c004)) + s * (c105 - t * c006 + s * c007);
  const double sd = c108 + t * (c109 + t * (c010 + t * (c111 + t * c012))) +
                    s * (c013 - t * (c014 + t * t * c015) + sqrt(mx2(0.0, s)) * (c016 + t * t * c017));
  const double sq = 1.0 / sd;
  return sn * sq - 1000.0;
}
/* stmt_fns.h:516: no inverse for the 17-term equation of state */
static double tofsig17(double r, double s) {
  (void)r;
  (void)s;
  return 99.0;
}

/* harmonc, mod_tsadvc.F90:1770-1771 */
static inline double harmonz(double a, double b) { return 2.0 * a * b / mx2((a + b), 2.0 * 1.0e-20); }
static inline double harmonc(double aa, double bb) { return harmonz(mx2(aa, 0.0), mx2(bb, 0.0)); }

/* tsdff_1x / tsdff_2x on layer slices f1 (and f2), dp(:,:,k,n), onetamas(:,:,n) */
static void tsdff_nx(hyo_grid *g, double *f1, double *f2, const double *dpk, const double *ota, double temdf2,
                     double delt1, const double *aspux, const double *aspvy, const double *scuy,
                     const double *scvx) {
  const int ii = g->ii, jj = g->jj, ld = g->ld1;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;
  double *uflux = g->uflux, *vflux = g->vflux, *uflux2 = g->uflux2, *vflux2 = g->vflux2;
  double *util1 = g->util1, *util2 = g->util2;
  int margin = 1; /* :2270-2291 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (iu[c] != 0) {
        double factor = temdf2 * aspux[c] * scuy[c] * harmonc(dpk[c - 1] * ota[c - 1], dpk[c] * ota[c]);
        uflux[c] = factor * (f1[c - 1] - f1[c]);
        if (f2) uflux2[c] = factor * (f2[c - 1] - f2[c]);
      }
      if (iv[c] != 0) {
        double factor = temdf2 * aspvy[c] * scvx[c] * harmonc(dpk[c - ld] * ota[c - ld], dpk[c] * ota[c]);
        vflux[c] = factor * (f1[c - ld] - f1[c]);
        if (f2) vflux2[c] = factor * (f2[c - ld] - f2[c]);
      }
    }
  margin = 0; /* :2329-2343 */
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (ip[c] != 0) {
        double factor = -delt1 / (g->scp2[c] * mx2(dpk[c] * ota[c], 1.0e-20));
        util1[c] = ((uflux[c + 1] - uflux[c]) + (vflux[c + ld] - vflux[c])) * factor;
        f1[c] = f1[c] + util1[c];
        if (f2) {
          util2[c] = ((uflux2[c + 1] - uflux2[c]) + (vflux2[c + ld] - vflux2[c])) * factor;
          f2[c] = f2[c] + util2[c];
        }
      }
    }
}

/*
 * The diffusion block of tsadvc(m,n) (temdf2 > 0), run after the advection
 * (hyo_tsadvc) on the same fields; oneta (ld1,ld2,2) is onetamas(:,:,n) for
 * diffusion (:1804-1810); aspux, aspvy, scuy, scvx are the grid's arrays.
 * Layers beyond nhybrd (exactly isopycnal, needing theta) are not restated;
 * q2, q2l (ld1,ld2,0:kdm+1,2) are read only when mxlmy.
 */
int hyo_tsdff(hyo_grid *g, const hyo_tsparams *p, double temdf2, double temdfc, double thbase, int m, int n,
              double *temp, double *saln, double *th3d, double *tracer, double *q2, double *q2l, const double *dp,
              const double *oneta,
              const double *aspux, const double *aspvy, const double *scuy, const double *scvx) {
  const int ii = g->ii, jj = g->jj, kk = p->kdm;
  const size_t sl = (size_t)g->ld1 * g->ld2;
  (void)m;
  if (n < 1 || n > 2 || kk < 1 || !oneta || !aspux || !aspvy || !scuy || !scvx) return HYO_ERR_ARG;
  if (p->nhybrd < kk || (p->mxlmy && (!q2 || !q2l))) return HYO_ERR_ARG;
  if (!(temdf2 > 0.0)) return HYO_OK; /* :2138 */
  const int nn = n - 1;
  for (size_t c = 0; c < sl; c++) { /* :1812-1813, the land values of the diffusive fluxes */
    g->uflux[c] = 0.0;
    g->vflux[c] = 0.0;
  }
  const int mdf = 2; /* :2139-2152, level n of every diffused field */
  hyo_xctilr(g, saln + (size_t)nn * kk * sl, kk, mdf, mdf);
  hyo_xctilr(g, temp + (size_t)nn * kk * sl, kk, mdf, mdf);
  hyo_xctilr(g, th3d + (size_t)nn * kk * sl, kk, mdf, mdf);
  if (p->mxlmy) {
    hyo_xctilr(g, q2 + (size_t)nn * (kk + 2) * sl, kk + 2, mdf, mdf);
    hyo_xctilr(g, q2l + (size_t)nn * (kk + 2) * sl, kk + 2, mdf, mdf);
  }
  for (int ktr = 0; ktr < p->ntracr; ktr++) hyo_xctilr(g, tracer + ((size_t)ktr * 2 * kk + (size_t)nn * kk) * sl, kk, mdf, mdf);
  const double *ota = oneta + (size_t)nn * sl;
#define FN(a, k) ((a) + ((size_t)(k) + (size_t)nn * kk) * sl) /* (…,k,n), k 0-based */
  for (int k = 1; k <= kk; k++) { /* :2153-2198 */
    const int ldtemp = k <= p->nhybrd && temdfc > 0.0;
    const int ldth3d = (k <= p->nhybrd && temdfc < 1.0) || (k == 1 && p->isopyc);
    const double *dpk = dp + ((size_t)(k - 1) + (size_t)nn * kk) * sl;
    if (ldtemp && ldth3d) {
      tsdff_nx(g, FN(th3d, k - 1), FN(temp, k - 1), dpk, ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
      tsdff_nx(g, FN(saln, k - 1), NULL, dpk, ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
    } else if (ldtemp) {
      tsdff_nx(g, FN(temp, k - 1), FN(saln, k - 1), dpk, ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
    } else if (ldth3d) {
      tsdff_nx(g, FN(th3d, k - 1), FN(saln, k - 1), dpk, ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
    } else {
      tsdff_nx(g, FN(saln, k - 1), NULL, dpk, ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
    }
    if (p->mxlmy) /* q2(…,k,n), k 1-based in 0:kk+1 */
      tsdff_nx(g, q2 + ((size_t)k + (size_t)nn * (kk + 2)) * sl, q2l + ((size_t)k + (size_t)nn * (kk + 2)) * sl, dpk,
               ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
    for (int ktr = 0; ktr < p->ntracr; ktr += 2) {
      double *t1 = tracer + ((size_t)ktr * 2 * kk + (size_t)nn * kk + (size_t)(k - 1)) * sl;
      double *t2 = ktr + 1 < p->ntracr ? tracer + ((size_t)(ktr + 1) * 2 * kk + (size_t)nn * kk + (size_t)(k - 1)) * sl
                                        : NULL;
      tsdff_nx(g, t1, t2, dpk, ota, temdf2, p->delt1, aspux, aspvy, scuy, scvx);
    }
  }
  for (int j = 1; j <= jj; j++) /* :2199-2229, margin 0 */
    for (int k = 1; k <= kk; k++) {
      const int ldtemp = k <= p->nhybrd && temdfc > 0.0;
      const int ldth3d = (k <= p->nhybrd && temdfc < 1.0) || (k == 1 && p->isopyc);
      double *tk = FN(temp, k - 1), *sk = FN(saln, k - 1), *hk = FN(th3d, k - 1);
      for (int i = 1; i <= ii; i++) {
        size_t c = P(g, i, j);
        if (g->ip[c] == 0) continue;
        if (ldtemp && ldth3d) {
          double th3d_t = hyo_sig(tk[c], sk[c]) - thbase;
          hk[c] = (1.0 - temdfc) * hk[c] + temdfc * th3d_t;
          tk[c] = tofsig17(hk[c] + thbase, sk[c]);
        } else if (ldtemp) {
          hk[c] = hyo_sig(tk[c], sk[c]) - thbase;
        } else if (ldth3d) {
          tk[c] = tofsig17(hk[c] + thbase, sk[c]);
        }
      }
    }
#undef FN
  return HYO_OK;
}


/* ------------------------------------------------------------------ */
/* Robert-Asselin time filter of the scalar fields, mod_asselin.F90:   */
/* asselin_save :28-82 (start of the step) and asselin_filter :84-268  */
/* (end of the step), with the 17-term equation of state for th3d.     */
/* ------------------------------------------------------------------ */
/*
 * Arrays (reference layout), passed in a[HYO_A_N]:
 *   temp, saln, th3d (ld1,ld2,kdm,2); tracer (ld1,ld2,kdm,2,ntracr);
 *   q2, q2l (ld1,ld2,0:kdm+1,2); dp, dpo (ld1,ld2,kdm,2);
 *   oneta, onetao (ld1,ld2,2); pbavg (ld1,ld2,3); pbot (ld1,ld2);
 *   otemp, osaln, oth3d (ld1,ld2,kdm); otracer (ld1,ld2,kdm,ntracr);
 *   oq2, oq2l (ld1,ld2,0:kdm+1).
 * Entries not used by the switches may be NULL.
 */
enum {
  HYO_A_TEMP, HYO_A_SALN, HYO_A_TH3D, HYO_A_TRACER, HYO_A_Q2, HYO_A_Q2L, HYO_A_DP, HYO_A_DPO, HYO_A_ONETA,
  HYO_A_ONETAO, HYO_A_PBAVG, HYO_A_PBOT, HYO_A_OTEMP, HYO_A_OSALN, HYO_A_OTH3D, HYO_A_OTRACER, HYO_A_OQ2,
  HYO_A_OQ2L, HYO_A_N
};

/* asselin_save(m,n): oneta and onetao of both levels from pbavg/pbot at sea
   points, level n of every scalar into the t-1 copies (all interior points),
   then the halo of oneta/onetao (:45-80). */
int hyo_asselin_save(hyo_grid *g, const hyo_tsparams *p, double oneta0, int m, int n, double *const *a) {
  const int ii = g->ii, jj = g->jj, kk = p->kdm;
  const size_t sl = (size_t)g->ld1 * g->ld2;
  if (m < 1 || m > 2 || n < 1 || n > 2 || kk < 1) return HYO_ERR_ARG;
  if (!a[HYO_A_TEMP] || !a[HYO_A_SALN] || !a[HYO_A_TH3D] || !a[HYO_A_ONETA] || !a[HYO_A_ONETAO] ||
      !a[HYO_A_PBAVG] || !a[HYO_A_PBOT] || !a[HYO_A_OTEMP] || !a[HYO_A_OSALN] || !a[HYO_A_OTH3D] ||
      (p->ntracr > 0 && (!a[HYO_A_TRACER] || !a[HYO_A_OTRACER])) ||
      (p->mxlmy && (!a[HYO_A_Q2] || !a[HYO_A_Q2L] || !a[HYO_A_OQ2] || !a[HYO_A_OQ2L])))
    return HYO_ERR_ARG;
  const int mm = m - 1, nn = n - 1;
  double *oneta = a[HYO_A_ONETA], *onetao = a[HYO_A_ONETAO];
  const double *pbavg = a[HYO_A_PBAVG], *pbot = a[HYO_A_PBOT];
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1; j <= jj; j++) {
    for (int i = 1; i <= ii; i++) {
      size_t c = P(g, i, j);
      if (g->ip[c] != 0) {
        oneta[c + nn * sl] = mx2(oneta0, 1.0 + pbavg[c + nn * sl] / pbot[c]);
        oneta[c + mm * sl] = mx2(oneta0, 1.0 + pbavg[c + mm * sl] / pbot[c]);
        onetao[c + nn * sl] = oneta[c + nn * sl];
        onetao[c + mm * sl] = oneta[c + mm * sl];
      }
    }
    for (int k = 0; k < kk; k++)
      for (int i = 1; i <= ii; i++) {
        size_t c = P(g, i, j), lk = (size_t)k * sl, ln = ((size_t)k + (size_t)nn * kk) * sl;
        a[HYO_A_OTEMP][lk + c] = a[HYO_A_TEMP][ln + c];
        a[HYO_A_OSALN][lk + c] = a[HYO_A_SALN][ln + c];
        a[HYO_A_OTH3D][lk + c] = a[HYO_A_TH3D][ln + c];
        for (int t = 0; t < p->ntracr; t++)
          a[HYO_A_OTRACER][((size_t)t * kk) * sl + lk + c] = a[HYO_A_TRACER][((size_t)t * 2 * kk) * sl + ln + c];
      }
    if (p->mxlmy)
      for (int k = 1; k <= kk; k++)
        for (int i = 1; i <= ii; i++) {
          size_t c = P(g, i, j);
          a[HYO_A_OQ2][(size_t)k * sl + c] = a[HYO_A_Q2][((size_t)k + (size_t)nn * (kk + 2)) * sl + c];
          a[HYO_A_OQ2L][(size_t)k * sl + c] = a[HYO_A_Q2L][((size_t)k + (size_t)nn * (kk + 2)) * sl + c];
        }
  }
  hyo_xctilr(g, oneta, 2, 6, 6);
  hyo_xctilr(g, onetao, 2, 6, 6);
  return HYO_OK;
}

/* one scalar of asselin_filter, the version that conserves a constant field
   (:147-155): returns the filtered level-m value */
static inline double ra_scalar(double fo, double fm, double fn, double dpold, double dpmid, double dpnew,
                               double ra2fac, double qdpmidn) {
  const double smin = mn3(fo, fm, fn);
  const double dpsold = dpold * (fo - smin), dpsmid = dpmid * (fm - smin), dpsnew = dpnew * (fn - smin);
  const double q = 0.5 * ra2fac * (dpsold + dpsnew - 2.0 * dpsmid);
  return smin + (dpsmid + q) * qdpmidn;
}

/* asselin_filter(m,n) for hybrid layers advecting temperature (advflg=0,
   nhybrd >= kdm: the 17-term equation of state has no tofsig, so the th3d
   branch and the exactly isopycnal layers are not restated). */
int hyo_asselin_filter(hyo_grid *g, const hyo_tsparams *p, double ra2fac, double oneta0, double thbase, int m, int n,
                       double *const *a) {
  const int ii = g->ii, jj = g->jj, kk = p->kdm;
  const size_t sl = (size_t)g->ld1 * g->ld2;
  if (m < 1 || m > 2 || n < 1 || n > 2 || kk < 1) return HYO_ERR_ARG;
  if (p->advflg != 0 || p->nhybrd < kk || p->isopyc) return HYO_ERR_ARG;
  if (!a[HYO_A_TEMP] || !a[HYO_A_SALN] || !a[HYO_A_TH3D] || !a[HYO_A_DP] || !a[HYO_A_DPO] || !a[HYO_A_ONETA] ||
      !a[HYO_A_ONETAO] || !a[HYO_A_PBAVG] || !a[HYO_A_PBOT] || !a[HYO_A_OTEMP] || !a[HYO_A_OSALN] ||
      (p->ntracr > 0 && (!a[HYO_A_TRACER] || !a[HYO_A_OTRACER])) ||
      (p->mxlmy && (!a[HYO_A_Q2] || !a[HYO_A_Q2L] || !a[HYO_A_OQ2] || !a[HYO_A_OQ2L])))
    return HYO_ERR_ARG;
  const double onezm = 9806.e-20; /* :95 */
  const int mm = m - 1, nn = n - 1;
  double *oneta = a[HYO_A_ONETA];
  const double *onetao = a[HYO_A_ONETAO], *pbavg = a[HYO_A_PBAVG], *pbot = a[HYO_A_PBOT];
  double *dp = a[HYO_A_DP];
  const double *dpo = a[HYO_A_DPO];
#pragma omp parallel for schedule(static) num_threads(nthr(g))
  for (int j = 1; j <= jj; j++) {
    for (int i = 1; i <= ii; i++) { /* :112-117 */
      size_t c = P(g, i, j);
      if (g->ip[c] != 0) {
        oneta[c + nn * sl] = mx2(oneta0, 1.0 + pbavg[c + nn * sl] / pbot[c]);
        oneta[c + mm * sl] = mx2(oneta0, 1.0 + pbavg[c + mm * sl] / pbot[c]);
      }
    }
    for (int k = 0; k < kk; k++)
      for (int i = 1; i <= ii; i++) {
        size_t c = P(g, i, j);
        if (g->ip[c] == 0) continue;
        const size_t lk = (size_t)k * sl, lm = ((size_t)k + (size_t)mm * kk) * sl,
                     ln = ((size_t)k + (size_t)nn * kk) * sl;
        const double dpold = dpo[ln + c] * onetao[c + nn * sl]; /* :128-135 */
        const double dpmid = dpo[lm + c] * onetao[c + mm * sl];
        const double dpnew = dp[ln + c] * oneta[c + nn * sl];
        const double q = 0.5 * ra2fac * (dpold + dpnew - 2.0 * dpmid);
        const double dpmidn = dpmid + q;
        dp[lm + c] = dpmidn / oneta[c + mm * sl];
        if (!(dpmidn > onezm)) continue;
        const double qdpmidn = 1.0 / dpmidn;
        double *s = a[HYO_A_SALN], *t = a[HYO_A_TEMP];
        s[lm + c] = ra_scalar(a[HYO_A_OSALN][lk + c], s[lm + c], s[ln + c], dpold, dpmid, dpnew, ra2fac, qdpmidn);
        t[lm + c] = ra_scalar(a[HYO_A_OTEMP][lk + c], t[lm + c], t[ln + c], dpold, dpmid, dpnew, ra2fac, qdpmidn);
        a[HYO_A_TH3D][lm + c] = hyo_sig(t[lm + c], s[lm + c]) - thbase; /* :175-176 */
        for (int tr = 0; tr < p->ntracr; tr++) { /* :189-221 */
          double *f = a[HYO_A_TRACER] + (size_t)tr * 2 * kk * sl;
          const double *fo = a[HYO_A_OTRACER] + (size_t)tr * kk * sl;
          f[lm + c] = ra_scalar(fo[lk + c], f[lm + c], f[ln + c], dpold, dpmid, dpnew, ra2fac, qdpmidn);
        }
        if (p->mxlmy) { /* :222-233, q2(…,k,·) with k 1-based in 0:kk+1 */
          const size_t qm = ((size_t)(k + 1) + (size_t)mm * (kk + 2)) * sl,
                       qn = ((size_t)(k + 1) + (size_t)nn * (kk + 2)) * sl, qo = (size_t)(k + 1) * sl;
          double *q2 = a[HYO_A_Q2], *q2l = a[HYO_A_Q2L];
          double so = dpold * a[HYO_A_OQ2][qo + c], sm = dpmid * q2[qm + c], sn = dpnew * q2[qn + c];
          double qq = 0.5 * ra2fac * (so + sn - 2.0 * sm);
          q2[qm + c] = (sm + qq) * qdpmidn;
          so = dpold * a[HYO_A_OQ2L][qo + c];
          sm = dpmid * q2l[qm + c];
          sn = dpnew * q2l[qn + c];
          qq = 0.5 * ra2fac * (so + sn - 2.0 * sm);
          q2l[qm + c] = (sm + qq) * qdpmidn;
        }
      }
  }
  return HYO_OK;
}

/* ------------------------------------------------------------------ */
/* Continuity equation, cnuity.F90:14-1419 (flux-corrected transport   */
/* of the layer thicknesses): loop 76 (low-order fluxes, FCT limiter,  */
/* antidiffusive fluxes), the negative-thickness check, loop 77 and    */
/* the bottom-pressure restoring (not btrmas), biharmonic (loop 13) or */
/* Laplacian (loop 113) interface-depth diffusion, the cumulative      */
/* fluxes, the btrmas restoring and the Robert-Asselin filter of dp.   */
/* Not restated: open boundaries (iuopn/ivopn), STOKES drift, isopyc   */
/* (dpmixl), the Kraus-Turner mixed-layer base advection (mxlkta) and  */
/* the float vertical velocity (synflt).                               */
/* ------------------------------------------------------------------ */
typedef struct hyo_cnparams {
  int kdm, nstep, btrmas;
  int thkdf4, thkdf2; /* nonzero: that thickness diffusion runs, with the coefficients thkdfu/thkdfv
                         (the reference's thkdf4u/thkdf4v, which hold thkdf2's in the Laplacian case) */
  double delt1, ra2fac;
} hyo_cnparams;

enum {
  HYO_C_DP, HYO_C_DPO, HYO_C_DPU, HYO_C_DPV, HYO_C_U, HYO_C_V, HYO_C_UBAVG, HYO_C_VBAVG, HYO_C_PBOT, HYO_C_DEPTHU,
  HYO_C_DEPTHV, HYO_C_ONETA, HYO_C_SCUY, HYO_C_SCVX, HYO_C_THKDFU, HYO_C_THKDFV, HYO_C_P, HYO_C_UFLX, HYO_C_VFLX,
  HYO_C_UFLXAV, HYO_C_VFLXAV, HYO_C_DPAV, HYO_C_ONETACNT, HYO_C_N
};
#define HYO_ERR_NEGDP (-9)

/* ipim1x etc. (bigrid.F90:343-368): W (E, S, N) if sea, else the opposite
   neighbour if sea, else the point itself */
static inline int nbx(const hyo_grid *g, int i, int j, int di, int dj) {
  if (g->ip[P(g, i + di, j + dj)] != 0) return 1;
  if (g->ip[P(g, i - di, j - dj)] != 0) return -1;
  return 0;
}

int hyo_cnuity(hyo_grid *g, const hyo_cnparams *p, int m, int n, double *const *a, double *dpkmin_out) {
  const int ii = g->ii, jj = g->jj, kk = p->kdm, ld = g->ld1;
  const size_t sl = (size_t)g->ld1 * g->ld2;
  if (m < 1 || m > 2 || n < 1 || n > 2 || kk < 1 || g->nbdy < 6) return HYO_ERR_ARG;
  for (int q = 0; q < HYO_C_N; q++)
    if (!a[q] && q != HYO_C_UFLXAV && q != HYO_C_VFLXAV && q != HYO_C_DPAV && q != HYO_C_ONETA &&
        q != HYO_C_ONETACNT && q != HYO_C_THKDFU && q != HYO_C_THKDFV)
      return HYO_ERR_ARG;
  if (p->btrmas && (!a[HYO_C_ONETA] || !a[HYO_C_ONETACNT])) return HYO_ERR_ARG;
  if ((p->thkdf4 || p->thkdf2) && (!a[HYO_C_THKDFU] || !a[HYO_C_THKDFV])) return HYO_ERR_ARG;
  const int mm = m - 1, nn = n - 1;
  const int32_t *ip = g->ip, *iu = g->iu, *iv = g->iv;
  const double *scp2 = g->scp2, *scp2i = g->scp2i;
  double *dp = a[HYO_C_DP], *dpo = a[HYO_C_DPO], *pp = a[HYO_C_P], *uflx = a[HYO_C_UFLX], *vflx = a[HYO_C_VFLX];
  const double *dpu = a[HYO_C_DPU], *dpv = a[HYO_C_DPV], *u = a[HYO_C_U], *v = a[HYO_C_V];
  const double *ubavg = a[HYO_C_UBAVG], *vbavg = a[HYO_C_VBAVG], *pbot = a[HYO_C_PBOT];
  const double *depthu = a[HYO_C_DEPTHU], *depthv = a[HYO_C_DEPTHV], *scuy = a[HYO_C_SCUY], *scvx = a[HYO_C_SCVX];
  const double onem = ONEM, onecm = ONEM * 0.01, epsil = 1.0e-11, dpfatal = -10.0, epsil_cnuity = 1.e-14;
  double *uflux = g->uflux, *vflux = g->vflux, *uflux2 = g->uflux2, *vflux2 = g->vflux2;
  double *w = (double *)calloc(sl * 12, sizeof(double));
  if (!w) return HYO_ERR_ARG;
  double *utotm = w, *vtotm = w + sl, *utotn = w + 2 * sl, *vtotn = w + 3 * sl, *util1 = w + 4 * sl,
         *util2 = w + 5 * sl, *util3 = w + 6 * sl, *pold = w + 7 * sl, *oneta_u = w + 8 * sl,
         *oneta_v = w + 9 * sl, *om = w + 10 * sl; /* onetamas(:,:,1:2) */
#define DPK(k, t) (dp + ((size_t)(k) + (size_t)(t) * kk) * sl) /* k 0-based */
#define PK(k) (pp + (size_t)(k) * sl)                          /* p(:,:,k+1), k 0-based */
  double *dpkmin = (double *)malloc(sizeof(double) * 2 * kk);
  /* uflux/vflux hold 0 on faces that are not sea faces when cnuity runs:
     geopar zeroes them next to the sea (geopar.F90:826-836), tsadvc zeroes
     the whole array every step (mod_tsadvc.F90:1812-1813), and momtum,
     cnuity and tsdff write sea faces only */
  for (size_t c = 0; c < sl; c++) {
    if (iu[c] == 0) uflux[c] = 0.0;
    if (iv[c] == 0) vflux[c] = 0.0;
  }
  int mbdy = 6;
  /* halos (:100-107); dpmixl is not restated */
  hyo_xctilr(g, dp, 2 * kk, 6, 6);
  hyo_xctilr(g, (double *)dpu + (size_t)mm * kk * sl, kk, 6, 6);
  hyo_xctilr(g, (double *)dpv + (size_t)mm * kk * sl, kk, 6, 6);
  hyo_xctilr(g, (double *)u + (size_t)mm * kk * sl, kk, 6, 6);
  hyo_xctilr(g, (double *)v + (size_t)mm * kk * sl, kk, 6, 6);
  hyo_xctilr(g, (double *)ubavg + (size_t)mm * sl, 1, 6, 6);
  hyo_xctilr(g, (double *)vbavg + (size_t)mm * sl, 1, 6, 6);
  int margin = mbdy; /* :112-157 */
  for (int j = 1 - margin; j <= jj + margin; j++)
    for (int i = 1 - margin; i <= ii + margin; i++) {
      size_t c = P(g, i, j);
      if (p->btrmas) {
        const double *oneta = a[HYO_C_ONETA];
        om[c] = oneta[c];
        om[c + sl] = oneta[c + sl];
        /* the outermost halo column/row has no west/south neighbour (the
           reference reads outside the array there); those factors are never read */
        if (iu[c] != 0 && i > 1 - g->nbdy) {
          if (pbot[c] == pbot[c - 1]) oneta_u[c] = 0.5 * (om[c + mm * sl] + om[c - 1 + mm * sl]);
          else if (pbot[c] == depthu[c]) oneta_u[c] = om[c + mm * sl];
          else oneta_u[c] = om[c - 1 + mm * sl];
        }
        if (iv[c] != 0 && j > 1 - g->nbdy) {
          if (pbot[c] == pbot[c - ld]) oneta_v[c] = 0.5 * (om[c + mm * sl] + om[c - ld + mm * sl]);
          else if (pbot[c] == depthv[c]) oneta_v[c] = om[c + mm * sl];
          else oneta_v[c] = om[c - ld + mm * sl];
        }
      } else {
        om[c] = 1.0;
        om[c + sl] = 1.0;
        oneta_u[c] = 1.0;
        oneta_v[c] = 1.0;
      }
      utotn[c] = 0.0;
      vtotn[c] = 0.0;
      util3[c] = 0.0;
      for (int k = 0; k < kk; k++) dpo[((size_t)k + (size_t)nn * kk) * sl + c] = DPK(k, nn)[c]; /* t-1 */
    }
  const double *omn = om + (size_t)nn * sl;
  for (int k = 0; k < kk; k++) { /* loop 76 */
    double *dk = DPK(k, nn);
    const double *uk = u + ((size_t)k + (size_t)mm * kk) * sl, *vk = v + ((size_t)k + (size_t)mm * kk) * sl;
    const double *dpuk = dpu + ((size_t)k + (size_t)mm * kk) * sl, *dpvk = dpv + ((size_t)k + (size_t)mm * kk) * sl;
    double *uflxk = uflx + (size_t)k * sl, *vflxk = vflx + (size_t)k * sl;
    margin = mbdy - 1; /* :240-285 (open-boundary loops :160-234 do nothing without iuopn/ivopn) */
    for (int j = 1 - margin; j <= jj + margin; j++) {
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (iu[c] == 0) continue;
        utotm[c] = (uk[c] + ubavg[c + mm * sl]) * scuy[c];
        double q;
        if (utotm[c] >= 0.) q = mn2(dk[c - 1], mx2(0., depthu[c] - util3[c - 1])) * omn[c - 1];
        else q = mn2(dk[c], mx2(0., depthu[c] - util3[c])) * omn[c];
        uflux[c] = utotm[c] * q;
        uflux2[c] = utotm[c] * dpuk[c] * oneta_u[c] - uflux[c];
        uflxk[c] = uflux[c];
      }
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (iv[c] == 0) continue;
        vtotm[c] = (vk[c] + vbavg[c + mm * sl]) * scvx[c];
        double q;
        if (vtotm[c] >= 0.) q = mn2(dk[c - ld], mx2(0., depthv[c] - util3[c - ld])) * omn[c - ld];
        else q = mn2(dk[c], mx2(0., depthv[c] - util3[c])) * omn[c];
        vflux[c] = vtotm[c] * q;
        vflux2[c] = vtotm[c] * dpvk[c] * oneta_v[c] - vflux[c];
        vflxk[c] = vflux[c];
      }
    }
    margin = mbdy - 2; /* loop 19, :294-315 */
    double dmin = 999.;
    for (int j = 1 - margin; j <= jj + margin; j++) {
      double dpmin = 999.;
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] == 0) continue;
        util3[c] = util3[c] + dk[c];
        dk[c] = dk[c] * omn[c] - ((uflux[c + 1] - uflux[c]) + (vflux[c + ld] - vflux[c])) * p->delt1 * scp2i[c];
        dpo[((size_t)k + (size_t)mm * kk) * sl + c] = dk[c];
        dpmin = mn2(dpmin, dk[c]);
      }
      if (j >= 1 && j <= jj) dmin = mn2(dmin, dpmin);
    }
    dpkmin[k] = dmin;
    margin = mbdy - 2; /* :400-430 */
    for (int j = 1 - margin; j <= jj + margin; j++)
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] == 0) continue;
        const size_t ca = P(g, g->ipim1[c], j), cb = P(g, g->ipip1[c], j), cja = P(g, i, g->ipjm1[c]),
                     cjb = P(g, i, g->ipjp1[c]);
        double u1 = mx5(dk[c], dk[ca], dk[cb], dk[cja], dk[cjb]);
        double u2 = mx2(0., mn2(mn2(mn2(mn2(dk[c], dk[ca]), dk[cb]), dk[cja]), dk[cjb]));
        util1[c] = (u1 - dk[c]) / ((((mx2(0., uflux2[c]) - mn2(0., uflux2[c + 1])) +
                                     (mx2(0., vflux2[c]) - mn2(0., vflux2[c + ld]))) + epsil) *
                                   p->delt1 * scp2i[c]);
        util2[c] = (u2 - dk[c]) / ((((mn2(0., uflux2[c]) - mx2(0., uflux2[c + 1])) +
                                     (mn2(0., vflux2[c]) - mx2(0., vflux2[c + ld]))) - epsil) *
                                   p->delt1 * scp2i[c]);
      }
    margin = mbdy - 3; /* :442-472 */
    for (int j = 1 - margin; j <= jj + margin; j++) {
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (iu[c] == 0) continue;
        double clip = uflux2[c] >= 0. ? mn2(mn2(1., util1[c]), util2[c - 1]) : mn2(mn2(1., util2[c]), util1[c - 1]);
        utotn[c] = utotn[c] + uflux2[c] * (1. - clip);
        uflux[c] = uflux2[c] * clip;
        uflxk[c] = uflxk[c] + uflux[c];
      }
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (iv[c] == 0) continue;
        double clip =
            vflux2[c] >= 0. ? mn2(mn2(1., util1[c]), util2[c - ld]) : mn2(mn2(1., util2[c]), util1[c - ld]);
        vtotn[c] = vtotn[c] + vflux2[c] * (1. - clip);
        vflux[c] = vflux2[c] * clip;
        vflxk[c] = vflxk[c] + vflux[c];
      }
    }
    margin = mbdy - 4; /* loop 15, :480-498 */
    dmin = 999.;
    for (int j = 1 - margin; j <= jj + margin; j++) {
      double dpmin = 999.;
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] == 0) continue;
        dk[c] = dk[c] - ((uflux[c + 1] - uflux[c]) + (vflux[c + ld] - vflux[c])) * p->delt1 * scp2i[c];
        PK(k + 1)[c] = PK(k)[c] + dk[c];
        dpmin = mn2(dpmin, dk[c]);
      }
      if (j >= 1 && j <= jj) dmin = mn2(dmin, dpmin);
    }
    dpkmin[k + kk] = dmin;
  }
  int rc = HYO_OK;
  if (p->nstep % 3 == 0) { /* :520-580: only the fatal part changes the run */
    double mn = dpkmin[kk];
    for (int k = kk + 1; k < 2 * kk; k++) mn = mn2(mn, dpkmin[k]);
    if (mn < dpfatal * onem) rc = HYO_ERR_NEGDP;
  }
  if (dpkmin_out) memcpy(dpkmin_out, dpkmin, sizeof(double) * 2 * kk);
  if (rc == HYO_OK && !p->btrmas) {
    for (int k = 0; k < kk; k++) { /* loop 77 */
      double *dk = DPK(k, nn), *uflxk = uflx + (size_t)k * sl, *vflxk = vflx + (size_t)k * sl;
      margin = mbdy - 5;
      for (int j = 1 - margin; j <= jj + margin; j++) {
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (iu[c] == 0) continue;
          double q = utotn[c] >= 0. ? dk[c - 1] / PK(kk)[c - 1] : dk[c] / PK(kk)[c];
          uflux[c] = utotn[c] * q;
          uflxk[c] = uflxk[c] + uflux[c];
        }
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (iv[c] == 0) continue;
          double q = vtotn[c] >= 0. ? dk[c - ld] / PK(kk)[c - ld] : dk[c] / PK(kk)[c];
          vflux[c] = vtotn[c] * q;
          vflxk[c] = vflxk[c] + vflux[c];
        }
      }
      margin = mbdy - 6;
      for (int j = 1 - margin; j <= jj + margin; j++)
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (ip[c] == 0) continue;
          dk[c] = dk[c] - ((uflux[c + 1] - uflux[c]) + (vflux[c + ld] - vflux[c])) * p->delt1 * scp2i[c];
          PK(k + 1)[c] = PK(k)[c] + dk[c];
        }
    }
    margin = mbdy - 6; /* bottom-pressure restoring, :709-735 */
    for (int j = 1 - margin; j <= jj + margin; j++)
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] == 0) continue;
        double q = pbot[c] / PK(kk)[c];
        for (int k = 0; k < kk; k++) {
          DPK(k, nn)[c] = DPK(k, nn)[c] * q;
          PK(k + 1)[c] = PK(k)[c] + DPK(k, nn)[c];
        }
      }
  }
  if (rc == HYO_OK && (p->thkdf4 || p->thkdf2)) { /* loops 13 (biharmonic) and 113 (Laplacian) */
    const double *thu = a[HYO_C_THKDFU], *thv = a[HYO_C_THKDFV];
    for (int pass = 0; pass < 2; pass++) {
      const int bih = pass == 0;
      if (bih ? !p->thkdf4 : !p->thkdf2) continue;
      hyo_xctilr(g, dp + (size_t)nn * kk * sl, kk, 6, 6);
      hyo_xctilr(g, pp + sl, kk, 6, 6);
      const double dtinv = 1. / p->delt1;
      const int iflip = p->nstep % 2;
      margin = mbdy;
      for (int j = 1 - margin; j <= jj + margin; j++)
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (iu[c] != 0) uflux[c] = 0.;
          if (iv[c] != 0) vflux[c] = 0.;
          if (ip[c] != 0) {
            if (!bih) vflux[c] = 0.; /* :1005 */
            pold[c] = iflip == 1 ? PK(kk)[c] : 0.;
          }
        }
      const int k0 = bih ? (iflip ? kk : 2) : 2, k1 = bih ? (iflip ? 2 : kk) : kk, dk_ = bih ? (iflip ? -1 : 1) : 1;
      for (int k = k0;; k += dk_) { /* k 1-based; p(:,:,k) = PK(k-1) */
        const double *pk = PK(k - 1), *ptop = PK(kk);
        const double *dk = DPK(k - 1, nn), *dkm = DPK(k - 2, nn);
        if (bih) {
          margin = mbdy - 1; /* :790-830 */
          for (int j = 1 - margin; j <= jj + margin; j++)
            for (int i = 1 - margin; i <= ii + margin; i++) {
              size_t c = P(g, i, j);
              if (ip[c] == 0) continue;
              if (mn2(dk[c], dkm[c]) < onecm) {
                util1[c] = 0.0;
                util2[c] = 0.0;
              } else {
                const size_t ca = c + nbx(g, i, j, -1, 0) * -1, cb = c + nbx(g, i, j, 1, 0),
                             cja = c + (size_t)(nbx(g, i, j, 0, -1) * -ld), cjb = c + (size_t)(nbx(g, i, j, 0, 1) * ld);
                util1[c] = pk[c] - .5 * (pk[ca] + pk[cb]);
                util2[c] = pk[c] - .5 * (pk[cja] + pk[cjb]);
                if (util1[c] > 0.0) {
                  if (mn2(dk[ca], dk[cb]) < onecm) util1[c] = 0.0;
                } else {
                  if (mn2(dkm[ca], dkm[cb]) < onecm) util1[c] = 0.0;
                }
                if (util2[c] > 0.0) {
                  if (mn2(dk[cja], dk[cjb]) < onecm) util2[c] = 0.0;
                } else {
                  if (mn2(dkm[cja], dkm[cjb]) < onecm) util2[c] = 0.0;
                }
              }
            }
        }
        margin = mbdy - 2; /* :838-900 and :1030-1060 */
        double *uk1 = uflx + (size_t)(k - 2) * sl, *uk = uflx + (size_t)(k - 1) * sl;
        double *vk1 = vflx + (size_t)(k - 2) * sl, *vk = vflx + (size_t)(k - 1) * sl;
        for (int j = 1 - margin; j <= jj + margin; j++) {
          for (int i = 1 - margin; i <= ii + margin; i++) {
            size_t c = P(g, i, j);
            if (iu[c] == 0) continue;
            double flxhi = .25 * (ptop[c] - pk[c]) * scp2[c];
            double flxlo = -.25 * (ptop[c - 1] - pk[c - 1]) * scp2[c - 1];
            if (bih) {
              if (iflip == 0) {
                flxhi = mn2(flxhi, uflux[c] + .25 * (pk[c - 1] - pold[c - 1]) * scp2[c - 1]);
                flxlo = mx2(flxlo, uflux[c] - .25 * (pk[c] - pold[c]) * scp2[c]);
              } else {
                flxhi = mn2(flxhi, uflux[c] + .25 * (pold[c] - pk[c]) * scp2[c]);
                flxlo = mx2(flxlo, uflux[c] - .25 * (pold[c - 1] - pk[c - 1]) * scp2[c - 1]);
              }
              const double thkdfu = p->delt1 * thu[c];
              uflux[c] = mn2(flxhi, mx2(flxlo, thkdfu * (util1[c - 1] - util1[c])));
            } else {
              const double thkdfu = p->delt1 * thu[c];
              uflux[c] = mn2(flxhi, mx2(flxlo, thkdfu * (pk[c - 1] - pk[c])));
            }
            uk1[c] = uk1[c] + uflux[c] * dtinv;
            uk[c] = uk[c] - uflux[c] * dtinv;
          }
          for (int i = 1 - margin; i <= ii + margin; i++) {
            size_t c = P(g, i, j);
            if (iv[c] == 0) continue;
            double flxhi = .25 * (ptop[c] - pk[c]) * scp2[c];
            double flxlo = -.25 * (ptop[c - ld] - pk[c - ld]) * scp2[c - ld];
            if (bih) {
              if (iflip == 0) {
                flxhi = mn2(flxhi, vflux[c] + .25 * (pk[c - ld] - pold[c - ld]) * scp2[c - ld]);
                flxlo = mx2(flxlo, vflux[c] - .25 * (pk[c] - pold[c]) * scp2[c]);
              } else {
                flxhi = mn2(flxhi, vflux[c] + .25 * (pold[c] - pk[c]) * scp2[c]);
                flxlo = mx2(flxlo, vflux[c] - .25 * (pold[c - ld] - pk[c - ld]) * scp2[c - ld]);
              }
              const double thkdfv = p->delt1 * thv[c];
              vflux[c] = mn2(flxhi, mx2(flxlo, thkdfv * (util2[c - ld] - util2[c])));
            } else {
              const double thkdfv = p->delt1 * thv[c];
              vflux[c] = mn2(flxhi, mx2(flxlo, thkdfv * (pk[c - ld] - pk[c])));
            }
            vk1[c] = vk1[c] + vflux[c] * dtinv;
            vk[c] = vk[c] - vflux[c] * dtinv;
          }
        }
        margin = mbdy - 2; /* :905-920 */
        double *pkw = PK(k - 1);
        for (int j = 1 - margin; j <= jj + margin; j++)
          for (int i = 1 - margin; i <= ii + margin; i++) {
            size_t c = P(g, i, j);
            if (ip[c] == 0) continue;
            pold[c] = pkw[c];
            pkw[c] = pkw[c] - ((uflux[c + 1] - uflux[c]) + (vflux[c + ld] - vflux[c])) * scp2i[c];
          }
        if (k == k1) break;
      }
      margin = mbdy - 2; /* :925-950 */
      for (int j = 1 - margin; j <= jj + margin; j++)
        for (int k = 0; k < kk; k++)
          for (int i = 1 - margin; i <= ii + margin; i++) {
            size_t c = P(g, i, j);
            if (ip[c] == 0) continue;
            if (PK(k + 1)[c] < PK(k)[c]) PK(k + 1)[c] = PK(k)[c];
            DPK(k, nn)[c] = PK(k + 1)[c] - PK(k)[c];
          }
    }
  }
  if (rc == HYO_OK) {
    if (a[HYO_C_UFLXAV] && a[HYO_C_VFLXAV] && a[HYO_C_DPAV]) /* cumulative fluxes, :1326-1348 */
      for (int j = 1; j <= jj; j++)
        for (int k = 0; k < kk; k++)
          for (int i = 1; i <= ii; i++) {
            size_t c = P(g, i, j), ck = (size_t)k * sl + c;
            if (iu[c] != 0) a[HYO_C_UFLXAV][ck] = a[HYO_C_UFLXAV][ck] + uflx[ck];
            if (iv[c] != 0) a[HYO_C_VFLXAV][ck] = a[HYO_C_VFLXAV][ck] + vflx[ck];
            if (ip[c] != 0) a[HYO_C_DPAV][ck] = a[HYO_C_DPAV][ck] + DPK(k, nn)[c];
          }
    if (p->btrmas) { /* :1350-1385 */
      double *onetacnt = a[HYO_C_ONETACNT];
      margin = 1;
      for (int j = 1 - margin; j <= jj + margin; j++)
        for (int i = 1 - margin; i <= ii + margin; i++) {
          size_t c = P(g, i, j);
          if (ip[c] == 0) continue;
          onetacnt[c] = PK(kk)[c] / pbot[c];
          if (onetacnt[c] > epsil_cnuity) {
            const double q = 1.0 / onetacnt[c];
            for (int k = 0; k < kk; k++) {
              DPK(k, nn)[c] = DPK(k, nn)[c] * q;
              PK(k + 1)[c] = PK(k)[c] + DPK(k, nn)[c];
            }
          } else {
            DPK(0, nn)[c] = pbot[c];
            PK(1)[c] = PK(0)[c] + DPK(0, nn)[c];
            for (int k = 1; k < kk; k++) {
              DPK(k, nn)[c] = 0.0;
              PK(k + 1)[c] = PK(k)[c] + DPK(k, nn)[c];
            }
          }
        }
    }
    hyo_xctilr(g, dp + (size_t)nn * kk * sl, kk, 6, 6); /* Robert-Asselin filter of dp, :1387-1410 */
    margin = mbdy;
    for (int j = 1 - margin; j <= jj + margin; j++)
      for (int i = 1 - margin; i <= ii + margin; i++) {
        size_t c = P(g, i, j);
        if (ip[c] == 0) continue;
        for (int k = 0; k < kk; k++) {
          const double dpold = dpo[((size_t)k + (size_t)nn * kk) * sl + c], dpmid = DPK(k, mm)[c],
                       dpnew = DPK(k, nn)[c];
          const double q = 0.5 * p->ra2fac * (dpold + dpnew - 2.0 * dpmid);
          dpo[((size_t)k + (size_t)mm * kk) * sl + c] = DPK(k, mm)[c];
          DPK(k, mm)[c] = dpmid + q;
        }
      }
  }
#undef DPK
#undef PK
  free(dpkmin);
  free(w);
  return rc;
}
