/* CPU oracle for the Athena++ MHD stage update — TEST INFRASTRUCTURE ONLY.
 *
 * Plain C99, FP64 throughout.  Every routine restates one reference routine and keeps
 * its floating-point association (operand order and grouping) so that results can be
 * compared bit for bit; comments give the reference file:line followed.  Compile with
 * -ffp-contract=off (no FMA contraction), without -ffast-math.
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.
 */
#include "athena_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* std::min / std::max semantics (return the first argument unless the second is
 * strictly smaller / larger) */
static inline double smin(double a, double b) { return (b < a) ? b : a; }
static inline double smax(double a, double b) { return (a < b) ? b : a; }
#define SQR(x) ((x) * (x))
#define SIGN(x) (((x) < 0.0) ? -1.0 : 1.0)

enum { IDN = 0, IVX = 1, IVY = 2, IVZ = 3, IPR = 4, IBY = 5, IBZ = 6, NWAVE = 7 };
enum { NHYDRO = 5 };

struct orc_mesh {
  orc_params p;
  int nb, nc1, nc2, nc3, is, ie, js, je, ks, ke;
  long ncell, nf1, nf2, nf3; /* per-block array sizes (one variable) */
  /* per block state, AthenaArray layout */
  double *u, *u1, *w, *w1, *bcc, *b1, *b2, *b3, *bb1, *bb2, *bb3;
  double *x1f, *dx1f, *x2f, *dx2f, *x3f, *dx3f; /* per block */
  double *x1v, *x2v, *x3v;
  double *e1, *e2, *e3;  /* per block edge EMFs before the shared-edge averaging */
  long ne1, ne2, ne3;
  double dt, time;
  long c2p_fail;
  /* multi-level mesh (athena_oracle_ml.c), NULL for a uniform mesh */
  struct orc_ml *ml;
  const int *ml_nblev;  /* its [nb][27] neighbour-level table */
  int integ;            /* time/integrator: ORC_VL2, ORC_RK2 or ORC_RK1 */
};

/* The stage weights of TimeIntegratorTaskList (time_integrator.cpp:111-236 vl2,
 * :338-465 rk2; rk1 one stage with beta = delta = 1): beta scales dt in the flux
 * divergence and CT, delta the first register average (u1 += delta*u), and
 * gamma = (g1, g2, 0) the second, a register swap when (0, 1, 0) (:1814-1821). */
typedef struct {
  double beta, delta, g1, g2;
  int order;  /* reconstruction: donor cell on the first vl2 stage (:1700-1703) */
  int swap;   /* gamma = (0, 1, 0) */
} stage_w;

struct orc_ml;
static stage_w stage_weights(const orc_mesh *m, int stage);
static void ml_stage(orc_mesh *m, int stage);
static void ml_initialize(orc_mesh *m);
static void ml_free(struct orc_ml *ml, int nb);

/* ------------------------------------------------------------------------------------
 * indexing helpers (athena_arrays.hpp:140-143)
 */
#define CIDX(m, n, k, j, i) ((((long)(n) * (m)->nc3 + (k)) * (m)->nc2 + (j)) * (m)->nc1 + (i))
#define F1IDX(m, k, j, i) ((((long)(k)) * (m)->nc2 + (j)) * ((m)->nc1 + 1) + (i))
#define F2IDX(m, k, j, i) ((((long)(k)) * ((m)->nc2 + 1) + (j)) * (m)->nc1 + (i))
#define F3IDX(m, k, j, i) ((((long)(k)) * (m)->nc2 + (j)) * (m)->nc1 + (i))

/* per-block scratch used within one stage (the reference keeps these per object,
 * hydro.cpp:31-148, field.cpp:27-105) */
typedef struct {
  double *flx1, *flx2, *flx3;          /* NHYDRO x face arrays */
  double *e3x1, *e2x1, *w1f;           /* x1 faces */
  double *e1x2, *e3x2, *w2f;           /* x2 faces */
  double *e1x3, *e2x3, *w3f;           /* x3 faces */
  double *e1, *e2, *e3;                /* edges */
  double *cce;                         /* 3 x cells */
} scratch;

static void scratch_alloc(const orc_mesh *m, scratch *s) {
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1);
  long n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1;
  long n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  s->flx1 = calloc(NHYDRO * n1, sizeof(double));
  s->flx2 = calloc(NHYDRO * n2, sizeof(double));
  s->flx3 = calloc(NHYDRO * n3, sizeof(double));
  s->e3x1 = calloc(n1, sizeof(double)); s->e2x1 = calloc(n1, sizeof(double));
  s->w1f = calloc(n1, sizeof(double));
  s->e1x2 = calloc(n2, sizeof(double)); s->e3x2 = calloc(n2, sizeof(double));
  s->w2f = calloc(n2, sizeof(double));
  s->e1x3 = calloc(n3, sizeof(double)); s->e2x3 = calloc(n3, sizeof(double));
  s->w3f = calloc(n3, sizeof(double));
  /* edges: x1e (nc3+1, nc2+1, nc1), x2e (nc3+1, nc2, nc1+1), x3e (nc3, nc2+1, nc1+1)
   * (athena.hpp:141-148) */
  s->e1 = calloc((long)(m->nc3 + 1) * (m->nc2 + 1) * m->nc1, sizeof(double));
  s->e2 = calloc((long)(m->nc3 + 1) * m->nc2 * (m->nc1 + 1), sizeof(double));
  s->e3 = calloc((long)m->nc3 * (m->nc2 + 1) * (m->nc1 + 1), sizeof(double));
  s->cce = calloc(3 * m->ncell, sizeof(double));
}

static void scratch_free(scratch *s) {
  free(s->flx1); free(s->flx2); free(s->flx3); free(s->e3x1); free(s->e2x1);
  free(s->w1f); free(s->e1x2); free(s->e3x2); free(s->w2f); free(s->e1x3);
  free(s->e2x3); free(s->w3f); free(s->e1); free(s->e2); free(s->e3); free(s->cce);
}

#define E1IDX(m, k, j, i) ((((long)(k)) * ((m)->nc2 + 1) + (j)) * (m)->nc1 + (i))
#define E2IDX(m, k, j, i) ((((long)(k)) * (m)->nc2 + (j)) * ((m)->nc1 + 1) + (i))
#define E3IDX(m, k, j, i) ((((long)(k)) * ((m)->nc2 + 1) + (j)) * ((m)->nc1 + 1) + (i))

/* ------------------------------------------------------------------------------------
 * EOS pieces (eos/adiabatic_mhd.cpp)
 */

/* FastMagnetosonicSpeed, adiabatic_mhd.cpp:149-156 */
static double fast_ms(double gamma, const double prim[NWAVE], double bx) {
  double asq = gamma * prim[IPR];
  double vaxsq = bx * bx;
  double ct2 = (prim[IBY] * prim[IBY] + prim[IBZ] * prim[IBZ]);
  double qsq = vaxsq + ct2 + asq;
  double tmp = vaxsq + ct2 - asq;
  return sqrt(0.5 * (qsq + sqrt(tmp * tmp + 4.0 * asq * ct2)) / prim[IDN]);
}

/* Hydro::GetWeightForCT, hydro.cpp:154-158 */
static double weight_for_ct(double dflx, double rhol, double rhor, double dx, double dt) {
  double v_over_c = (1024.0) * dt * dflx / (dx * (rhol + rhor));
  double tmp_min = smin(0.5, v_over_c);
  return 0.5 + smax(-0.5, tmp_min);
}

/* ------------------------------------------------------------------------------------
 * Riemann solvers.  wl/wr are in the solver's local order (IDN, normal v, two
 * transverse v, p, IBY, IBZ) as loaded in hlld.cpp:59-75.  out: f[0..4] = mass,
 * normal/transverse momentum, energy fluxes in that local order, f[5] = F(By),
 * f[6] = F(Bz).
 */

/* HLLD, hydro/rsolvers/mhd/hlld.cpp:36-376 (Miyoshi & Kusano 2005) */
typedef struct { double d, mx, my, mz, e, by, bz; } cons1d;

/* ld = 0: HLLD.  ld = 1: the low-dissipation HLLD of Minoshima et al. 2021,
 * hydro/rsolvers/mhd/lhlld.cpp:33-380, which differs in the middle speed (the pressure
 * jump scaled by the shock detector th from the face's velocity differences dvn, dvt,
 * :157-163), the star total pressure (the low-Mach factor phi, :184-188) and the grouping
 * of a few products (sdld = sdl*ul.d, :153-154, :192-234). */
static void hlld_core(double gamma, const double *wli, const double *wri, double bxi,
                      int ld, double dvn, double dvt, double *flxi) {
  const double SMALL_NUMBER = 1.0e-4;
  double igm1 = 1.0 / (gamma - 1.0);
  cons1d ul, ur, ulst, uldst, urdst, urst, fl, fr;
  double spd[5];

  double bxsq = bxi * bxi;
  double pbl = 0.5 * (bxsq + (SQR(wli[IBY]) + SQR(wli[IBZ])));
  double pbr = 0.5 * (bxsq + (SQR(wri[IBY]) + SQR(wri[IBZ])));
  double kel = 0.5 * wli[IDN] * (SQR(wli[IVX]) + (SQR(wli[IVY]) + SQR(wli[IVZ])));
  double ker = 0.5 * wri[IDN] * (SQR(wri[IVX]) + (SQR(wri[IVY]) + SQR(wri[IVZ])));

  ul.d = wli[IDN];
  ul.mx = wli[IVX] * ul.d;
  ul.my = wli[IVY] * ul.d;
  ul.mz = wli[IVZ] * ul.d;
  ul.e = wli[IPR] * igm1 + kel + pbl;
  ul.by = wli[IBY];
  ul.bz = wli[IBZ];

  ur.d = wri[IDN];
  ur.mx = wri[IVX] * ur.d;
  ur.my = wri[IVY] * ur.d;
  ur.mz = wri[IVZ] * ur.d;
  ur.e = wri[IPR] * igm1 + ker + pbr;
  ur.by = wri[IBY];
  ur.bz = wri[IBZ];

  /* eqn (67) wave speeds, hlld.cpp:104-108 */
  double cfl = fast_ms(gamma, wli, bxi);
  double cfr = fast_ms(gamma, wri, bxi);
  spd[0] = smin(wli[IVX] - cfl, wri[IVX] - cfr);
  spd[4] = smax(wli[IVX] + cfl, wri[IVX] + cfr);

  /* L/R fluxes, hlld.cpp:121-142 */
  double ptl = wli[IPR] + pbl;
  double ptr = wri[IPR] + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[IVX] + ptl - bxsq;
  fl.my = ul.my * wli[IVX] - bxi * ul.by;
  fl.mz = ul.mz * wli[IVX] - bxi * ul.bz;
  fl.e = wli[IVX] * (ul.e + ptl - bxsq) - bxi * (wli[IVY] * ul.by + wli[IVZ] * ul.bz);
  fl.by = ul.by * wli[IVX] - bxi * wli[IVY];
  fl.bz = ul.bz * wli[IVX] - bxi * wli[IVZ];

  fr.d = ur.mx;
  fr.mx = ur.mx * wri[IVX] + ptr - bxsq;
  fr.my = ur.my * wri[IVX] - bxi * ur.by;
  fr.mz = ur.mz * wri[IVX] - bxi * ur.bz;
  fr.e = wri[IVX] * (ur.e + ptr - bxsq) - bxi * (wri[IVY] * ur.by + wri[IVZ] * ur.bz);
  fr.by = ur.by * wri[IVX] - bxi * wri[IVY];
  fr.bz = ur.bz * wri[IVX] - bxi * wri[IVZ];

  /* middle and Alfven speeds, hlld.cpp:144-171 */
  double sdl = spd[0] - wli[IVX];
  double sdr = spd[4] - wri[IVX];
  double sdld = sdl * ul.d, sdrd = sdr * ur.d;
  double cfmax = smax(cfl, cfr);
  if (ld) {
    /* shock detector, lhlld.cpp:158-163 */
    double th1 = smin(1.0, (cfmax - smin(dvn, 0.0)) / (cfmax - smin(dvt, 0.0)));
    double th = th1 * th1 * th1 * th1;
    spd[2] = (sdr * ur.mx - sdl * ul.mx + th * (ptl - ptr)) / (sdrd - sdld);
  } else {
    spd[2] = (sdr * ur.mx - sdl * ul.mx + (ptl - ptr)) / (sdr * ur.d - sdl * ul.d);
  }
  double sdml = spd[0] - spd[2];
  double sdmr = spd[4] - spd[2];
  double sdml_inv = 1.0 / sdml;
  double sdmr_inv = 1.0 / sdmr;
  ulst.d = ul.d * sdl * sdml_inv;
  urst.d = ur.d * sdr * sdmr_inv;
  double ulst_d_inv = 1.0 / ulst.d;
  double urst_d_inv = 1.0 / urst.d;
  double sqrtdl = sqrt(ulst.d);
  double sqrtdr = sqrt(urst.d);
  spd[1] = spd[2] - fabs(bxi) / sqrtdl;
  spd[3] = spd[2] + fabs(bxi) / sqrtdr;

  /* intermediate states, hlld.cpp:173-300 */
  double ptst;
  if (ld) {  /* lhlld.cpp:184-188 */
    double clsq = ((pbl + kel) + sqrt(SQR(pbl + kel) - 2.0 * kel * bxsq)) / ul.d;
    double crsq = ((pbr + ker) + sqrt(SQR(pbr + ker) - 2.0 * ker * bxsq)) / ur.d;
    double chi = smin(1.0, sqrt(smax(clsq, crsq)) / cfmax);
    double phi = chi * (2.0 - chi);
    ptst = (sdrd * ptl - sdld * ptr + phi * sdrd * sdld * (wri[IVX] - wli[IVX])) /
           (sdrd - sdld);
  } else {
    double ptstl = ptl + ul.d * sdl * (spd[2] - wli[IVX]);
    double ptstr = ptr + ur.d * sdr * (spd[2] - wri[IVX]);
    ptst = 0.5 * (ptstr + ptstl);
  }

  ulst.mx = ulst.d * spd[2];
  if (fabs(ul.d * sdl * sdml - bxsq) < (SMALL_NUMBER)*ptst) {
    ulst.my = ulst.d * wli[IVY];
    ulst.mz = ulst.d * wli[IVZ];
    ulst.by = ul.by;
    ulst.bz = ul.bz;
  } else {
    double tmp = bxi * (sdl - sdml) / (ul.d * sdl * sdml - bxsq);
    ulst.my = ulst.d * (wli[IVY] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[IVZ] - ul.bz * tmp);
    tmp = (ld ? sdld * sdl - bxsq : ul.d * SQR(sdl) - bxsq) / (ul.d * sdl * sdml - bxsq);
    ulst.by = ul.by * tmp;
    ulst.bz = ul.bz * tmp;
  }
  double vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) * ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[IVX] + ptst * spd[2] +
            bxi * (wli[IVX] * bxi + (wli[IVY] * ul.by + wli[IVZ] * ul.bz) - vbstl)) *
           sdml_inv;

  urst.mx = urst.d * spd[2];
  if (fabs(ur.d * sdr * sdmr - bxsq) < (SMALL_NUMBER)*ptst) {
    urst.my = urst.d * wri[IVY];
    urst.mz = urst.d * wri[IVZ];
    urst.by = ur.by;
    urst.bz = ur.bz;
  } else {
    double tmp = bxi * (sdr - sdmr) / (ur.d * sdr * sdmr - bxsq);
    urst.my = urst.d * (wri[IVY] - ur.by * tmp);
    urst.mz = urst.d * (wri[IVZ] - ur.bz * tmp);
    tmp = (ld ? sdrd * sdr - bxsq : ur.d * SQR(sdr) - bxsq) / (ur.d * sdr * sdmr - bxsq);
    urst.by = ur.by * tmp;
    urst.bz = ur.bz * tmp;
  }
  double vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) * urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[IVX] + ptst * spd[2] +
            bxi * (wri[IVX] * bxi + (wri[IVY] * ur.by + wri[IVZ] * ur.bz) - vbstr)) *
           sdmr_inv;

  double invsumd = 1.0 / (sqrtdl + sqrtdr);
  double bxsig = (bxi > 0.0 ? 1.0 : -1.0);
  uldst.d = ulst.d;
  urdst.d = urst.d;
  uldst.mx = ulst.mx;
  urdst.mx = urst.mx;
  double tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) + sqrtdr * (urst.my * urst_d_inv) +
                          bxsig * (urst.by - ulst.by));
  uldst.my = uldst.d * tmp;
  urdst.my = urdst.d * tmp;
  tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) + sqrtdr * (urst.mz * urst_d_inv) +
                   bxsig * (urst.bz - ulst.bz));
  uldst.mz = uldst.d * tmp;
  urdst.mz = urdst.d * tmp;
  tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                   bxsig * sqrtdl * sqrtdr * ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
  uldst.by = urdst.by = tmp;
  tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                   bxsig * sqrtdl * sqrtdr * ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
  uldst.bz = urdst.bz = tmp;
  tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
  uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
  urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);

  /* jumps across the waves, hlld.cpp:302-332 */
#define JUMP(dst, a, b, s)                     \
  do {                                         \
    dst.d = (s) * (a.d - b.d);                 \
    dst.mx = (s) * (a.mx - b.mx);              \
    dst.my = (s) * (a.my - b.my);              \
    dst.mz = (s) * (a.mz - b.mz);              \
    dst.e = (s) * (a.e - b.e);                 \
    dst.by = (s) * (a.by - b.by);              \
    dst.bz = (s) * (a.bz - b.bz);              \
  } while (0)
  JUMP(uldst, uldst, ulst, spd[1]);
  JUMP(ulst, ulst, ul, spd[0]);
  JUMP(urdst, urdst, urst, spd[3]);
  JUMP(urst, urst, ur, spd[4]);
#undef JUMP

  /* upwind selection, hlld.cpp:334-370 */
  cons1d f;
  if (spd[0] >= 0.0) {
    f = fl;
  } else if (spd[4] <= 0.0) {
    f = fr;
  } else if (spd[1] >= 0.0) {
    f.d = fl.d + ulst.d; f.mx = fl.mx + ulst.mx; f.my = fl.my + ulst.my;
    f.mz = fl.mz + ulst.mz; f.e = fl.e + ulst.e; f.by = fl.by + ulst.by;
    f.bz = fl.bz + ulst.bz;
  } else if (spd[3] <= 0.0) {
    f.d = fr.d + urst.d; f.mx = fr.mx + urst.mx; f.my = fr.my + urst.my;
    f.mz = fr.mz + urst.mz; f.e = fr.e + urst.e; f.by = fr.by + urst.by;
    f.bz = fr.bz + urst.bz;
  } else if (spd[2] >= 0.0) {
    f.d = fl.d + ulst.d + uldst.d; f.mx = fl.mx + ulst.mx + uldst.mx;
    f.my = fl.my + ulst.my + uldst.my; f.mz = fl.mz + ulst.mz + uldst.mz;
    f.e = fl.e + ulst.e + uldst.e; f.by = fl.by + ulst.by + uldst.by;
    f.bz = fl.bz + ulst.bz + uldst.bz;
  } else {
    f.d = fr.d + urst.d + urdst.d; f.mx = fr.mx + urst.mx + urdst.mx;
    f.my = fr.my + urst.my + urdst.my; f.mz = fr.mz + urst.mz + urdst.mz;
    f.e = fr.e + urst.e + urdst.e; f.by = fr.by + urst.by + urdst.by;
    f.bz = fr.bz + urst.bz + urdst.bz;
  }
  flxi[0] = f.d; flxi[1] = f.mx; flxi[2] = f.my; flxi[3] = f.mz; flxi[4] = f.e;
  flxi[5] = f.by; flxi[6] = f.bz;
}

static void hlld(double gamma, const double *wli, const double *wri, double bxi,
                 double *flxi) {
  hlld_core(gamma, wli, wri, bxi, 0, 0.0, 0.0, flxi);
}

/* HLLE, hydro/rsolvers/mhd/hlle_mhd.cpp:25-182 */
static void hlle(double gamma, const double *wli, const double *wri, double bxi,
                 double *flxi) {
  double gm1 = gamma - 1.0;
  double fl[NWAVE], fr[NWAVE];
  double sqrtdl = sqrt(wli[IDN]);
  double sqrtdr = sqrt(wri[IDN]);
  double isdlpdr = 1.0 / (sqrtdl + sqrtdr);
  double wroe_d = sqrtdl * sqrtdr;
  double wroe_vx = (sqrtdl * wli[IVX] + sqrtdr * wri[IVX]) * isdlpdr;
  double wroe_vy = (sqrtdl * wli[IVY] + sqrtdr * wri[IVY]) * isdlpdr;
  double wroe_vz = (sqrtdl * wli[IVZ] + sqrtdr * wri[IVZ]) * isdlpdr;
  double wroe_by = (sqrtdr * wli[IBY] + sqrtdl * wri[IBY]) * isdlpdr;
  double wroe_bz = (sqrtdr * wli[IBZ] + sqrtdl * wri[IBZ]) * isdlpdr;
  double x = 0.5 * (SQR(wli[IBY] - wri[IBY]) + SQR(wli[IBZ] - wri[IBZ])) /
             (SQR(sqrtdl + sqrtdr));
  double y = 0.5 * (wli[IDN] + wri[IDN]) / wroe_d;

  double pbl = 0.5 * (bxi * bxi + SQR(wli[IBY]) + SQR(wli[IBZ]));
  double pbr = 0.5 * (bxi * bxi + SQR(wri[IBY]) + SQR(wri[IBZ]));
  double el = wli[IPR] / gm1 +
              0.5 * wli[IDN] * (SQR(wli[IVX]) + SQR(wli[IVY]) + SQR(wli[IVZ])) + pbl;
  double er = wri[IPR] / gm1 +
              0.5 * wri[IDN] * (SQR(wri[IVX]) + SQR(wri[IVY]) + SQR(wri[IVZ])) + pbr;
  double hroe = ((el + wli[IPR] + pbl) / sqrtdl + (er + wri[IPR] + pbr) / sqrtdr) * isdlpdr;

  double cl = fast_ms(gamma, wli, bxi);
  double cr = fast_ms(gamma, wri, bxi);

  double btsq = SQR(wroe_by) + SQR(wroe_bz);
  double vaxsq = bxi * bxi / wroe_d;
  double bt_starsq = (gm1 - (gm1 - 1.0) * y) * btsq;
  double hp = hroe - (vaxsq + btsq / wroe_d);
  double vsq = SQR(wroe_vx) + SQR(wroe_vy) + SQR(wroe_vz);
  double twid_asq = smax((gm1 * (hp - 0.5 * vsq) - (gm1 - 1.0) * x), 0.0);
  double ct2 = bt_starsq / wroe_d;
  double tsum = vaxsq + ct2 + twid_asq;
  double tdif = vaxsq + ct2 - twid_asq;
  double cf2_cs2 = sqrt(tdif * tdif + 4.0 * twid_asq * ct2);
  double cfsq = 0.5 * (tsum + cf2_cs2);
  double a = sqrt(cfsq);

  double al = smin((wroe_vx - a), (wli[IVX] - cl));
  double ar = smax((wroe_vx + a), (wri[IVX] + cr));
  double bp = ar > 0.0 ? ar : 0.0;
  double bm = al < 0.0 ? al : 0.0;

  double vxl = wli[IVX] - bm;
  double vxr = wri[IVX] - bp;
  fl[IDN] = wli[IDN] * vxl;
  fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl + pbl - SQR(bxi);
  fr[IVX] = wri[IDN] * wri[IVX] * vxr + pbr - SQR(bxi);
  fl[IVY] = wli[IDN] * wli[IVY] * vxl - bxi * wli[IBY];
  fr[IVY] = wri[IDN] * wri[IVY] * vxr - bxi * wri[IBY];
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl - bxi * wli[IBZ];
  fr[IVZ] = wri[IDN] * wri[IVZ] * vxr - bxi * wri[IBZ];
  fl[IVX] += wli[IPR];
  fr[IVX] += wri[IPR];
  fl[IPR] = el * vxl + wli[IVX] * (wli[IPR] + pbl - bxi * bxi);
  fr[IPR] = er * vxr + wri[IVX] * (wri[IPR] + pbr - bxi * bxi);
  fl[IPR] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IPR] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * vxl - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * vxr - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * vxl - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * vxr - bxi * wri[IVZ];

  double tmp = 0.0;
  if (bp != bm) tmp = 0.5 * (bp + bm) / (bp - bm);
  for (int n = 0; n < NWAVE; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

/* FastMagnetosonicSpeedsGR with the SR metric (g00, g01, g11) = (-1, 0, 1),
 * adiabatic_mhd_sr.cpp:350-370 */
static void sr_fast_speeds(double gamma_adi, double wgas, double pgas, double u0, double u1,
                           double b_sq, double *lp, double *lm) {
  const double g00 = -1.0, g01 = 0.0, g11 = 1.0;
  double cs_sq = gamma_adi * pgas / wgas;
  double va_sq = b_sq / (b_sq + wgas);
  double cms_sq = cs_sq + va_sq - cs_sq * va_sq;
  double a = SQR(u0) - (g00 + SQR(u0)) * cms_sq;
  double b = -2.0 * (u0 * u1 - (g01 + u0 * u1) * cms_sq);
  double c = SQR(u1) - (g11 + SQR(u1)) * cms_sq;
  double a1 = b / a;
  double a0 = c / a;
  double s = sqrt(smax(SQR(a1) - 4.0 * a0, 0.0));
  *lp = (a1 >= 0.0) ? -2.0 * a0 / (a1 + s) : (-a1 + s) / 2.0;
  *lm = (a1 >= 0.0) ? (-a1 - s) / 2.0 : -2.0 * a0 / (a1 - s);
}

/* local Lax-Friedrichs, hydro/rsolvers/mhd/llf_mhd.cpp:29-153 (adiabatic).  Local order
 * as for hlld(). */
static void llf(double gamma, const double *wli, const double *wri, double bxi,
                double *flxi) {
  double gm1 = gamma - 1.0;
  double fl[NWAVE], fr[NWAVE], du[NWAVE];
  double cfl = fast_ms(gamma, wli, bxi);
  double cfr = fast_ms(gamma, wri, bxi);
  double a = 0.5 * smax(fabs(wli[IVX]) + cfl, fabs(wri[IVX]) + cfr);
  double mxl = wli[IDN] * wli[IVX];
  double mxr = wri[IDN] * wri[IVX];
  double pbl = 0.5 * (bxi * bxi + SQR(wli[IBY]) + SQR(wli[IBZ]));
  double pbr = 0.5 * (bxi * bxi + SQR(wri[IBY]) + SQR(wri[IBZ]));
  fl[IDN] = mxl;
  fr[IDN] = mxr;
  fl[IVX] = mxl * wli[IVX] + pbl - SQR(bxi);
  fr[IVX] = mxr * wri[IVX] + pbr - SQR(bxi);
  fl[IVY] = mxl * wli[IVY] - bxi * wli[IBY];
  fr[IVY] = mxr * wri[IVY] - bxi * wri[IBY];
  fl[IVZ] = mxl * wli[IVZ] - bxi * wli[IBZ];
  fr[IVZ] = mxr * wri[IVZ] - bxi * wri[IBZ];
  double el = wli[IPR] / gm1 +
              0.5 * wli[IDN] * (SQR(wli[IVX]) + SQR(wli[IVY]) + SQR(wli[IVZ])) + pbl;
  double er = wri[IPR] / gm1 +
              0.5 * wri[IDN] * (SQR(wri[IVX]) + SQR(wri[IVY]) + SQR(wri[IVZ])) + pbr;
  fl[IVX] += wli[IPR];
  fr[IVX] += wri[IPR];
  fl[IPR] = (el + wli[IPR] + pbl - bxi * bxi) * wli[IVX];
  fr[IPR] = (er + wri[IPR] + pbr - bxi * bxi) * wri[IVX];
  fl[IPR] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IPR] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * wli[IVX] - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * wri[IVX] - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * wli[IVX] - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * wri[IVX] - bxi * wri[IVZ];
  du[IDN] = wri[IDN] - wli[IDN];
  du[IVX] = wri[IDN] * wri[IVX] - wli[IDN] * wli[IVX];
  du[IVY] = wri[IDN] * wri[IVY] - wli[IDN] * wli[IVY];
  du[IVZ] = wri[IDN] * wri[IVZ] - wli[IDN] * wli[IVZ];
  du[IPR] = er - el;
  du[IBY] = wri[IBY] - wli[IBY];
  du[IBZ] = wri[IBZ] - wli[IBZ];
  for (int n = 0; n < NWAVE; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) - a * du[n];
}

/* Roe's linearised solver for adiabatic MHD, hydro/rsolvers/mhd/roe_mhd.cpp:45-221 (the
 * driver) and :223-460 (RoeFlux: the eigensystem of Stone et al. 2008, ApJS 178, 137,
 * appendix B, eqs. B17-B29).  The sums over waves follow the reference's order term by
 * term, which fixes the rounding.  Upwind fluxes replace the Roe flux outside the fan; the
 * LLF flux replaces the hydro components (not the field ones) when an intermediate density
 * of the fan is negative. */
static void roe(double gamma, const double *wli, const double *wri, double bxi,
                double *flxi) {
  const double gm1 = gamma - 1.0;
  double fl[NWAVE], fr[NWAVE], du[NWAVE], ev[NWAVE], a[NWAVE], cf_[NWAVE];
  /* Roe averages (density-weighted velocity, inverse-weighted transverse field, enthalpy) */
  double sl = sqrt(wli[IDN]), sr = sqrt(wri[IDN]);
  double isum = 1.0 / (sl + sr);
  double d = sl * sr;
  double v1 = (sl * wli[IVX] + sr * wri[IVX]) * isum;
  double v2 = (sl * wli[IVY] + sr * wri[IVY]) * isum;
  double v3 = (sl * wli[IVZ] + sr * wri[IVZ]) * isum;
  double b2 = (sr * wli[IBY] + sl * wri[IBY]) * isum;
  double b3 = (sr * wli[IBZ] + sl * wri[IBZ]) * isum;
  double x = 0.5 * (SQR(wli[IBY] - wri[IBY]) + SQR(wli[IBZ] - wri[IBZ])) / SQR(sl + sr);
  double y = 0.5 * (wli[IDN] + wri[IDN]) / d;
  double pbl = 0.5 * (bxi * bxi + SQR(wli[IBY]) + SQR(wli[IBZ]));
  double pbr = 0.5 * (bxi * bxi + SQR(wri[IBY]) + SQR(wri[IBZ]));
  double el = wli[IPR] / gm1 +
              0.5 * wli[IDN] * (SQR(wli[IVX]) + SQR(wli[IVY]) + SQR(wli[IVZ])) + pbl;
  double er = wri[IPR] / gm1 +
              0.5 * wri[IDN] * (SQR(wri[IVX]) + SQR(wri[IVY]) + SQR(wri[IVZ])) + pbr;
  double h = ((el + wli[IPR] + pbl) / sl + (er + wri[IPR] + pbr) / sr) * isum;
  /* left and right physical fluxes */
  double mxl = wli[IDN] * wli[IVX], mxr = wri[IDN] * wri[IVX];
  fl[IDN] = mxl;
  fr[IDN] = mxr;
  fl[IVX] = mxl * wli[IVX] + pbl - SQR(bxi);
  fr[IVX] = mxr * wri[IVX] + pbr - SQR(bxi);
  fl[IVY] = mxl * wli[IVY] - bxi * wli[IBY];
  fr[IVY] = mxr * wri[IVY] - bxi * wri[IBY];
  fl[IVZ] = mxl * wli[IVZ] - bxi * wli[IBZ];
  fr[IVZ] = mxr * wri[IVZ] - bxi * wri[IBZ];
  fl[IVX] += wli[IPR];
  fr[IVX] += wri[IPR];
  fl[IPR] = (el + wli[IPR] + pbl - bxi * bxi) * wli[IVX];
  fr[IPR] = (er + wri[IPR] + pbr - bxi * bxi) * wri[IVX];
  fl[IPR] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IPR] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * wli[IVX] - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * wri[IVX] - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * wli[IVX] - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * wri[IVX] - bxi * wri[IVZ];
  /* jump in the conserved variables */
  du[IDN] = wri[IDN] - wli[IDN];
  du[IVX] = wri[IDN] * wri[IVX] - wli[IDN] * wli[IVX];
  du[IVY] = wri[IDN] * wri[IVY] - wli[IDN] * wli[IVY];
  du[IVZ] = wri[IDN] * wri[IVZ] - wli[IDN] * wli[IVZ];
  du[IPR] = er - el;
  du[IBY] = wri[IBY] - wli[IBY];
  du[IBZ] = wri[IBZ] - wli[IBZ];
  for (int n = 0; n < NWAVE; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]);

  /* wave speeds of the Roe matrix (eq. B17-B18) */
  double di = 1.0 / d;
  double btsq = b2 * b2 + b3 * b3;
  double vaxsq = bxi * bxi * di;
  double vsq = v1 * v1 + v2 * v2 + v3 * v3;
  double hp = h - (vaxsq + btsq * di);
  double ystar = gm1 - (gm1 - 1.0) * y;
  double bt_starsq = ystar * btsq;
  double csq = smax((gm1 * (hp - 0.5 * vsq) - (gm1 - 1.0) * x), 1.0e-20);
  double ct2 = bt_starsq * di;
  double tsum = vaxsq + ct2 + csq;
  double tdif = vaxsq + ct2 - csq;
  double root = sqrt(tdif * tdif + 4.0 * csq * ct2);
  double cfsq = 0.5 * (tsum + root);
  double cf = sqrt(cfsq);
  double cssq = csq * vaxsq / cfsq;
  double cs = sqrt(cssq);
  /* transverse-field directions (eq. A17, B20, B28) */
  double bt = sqrt(btsq), bt_star = sqrt(bt_starsq);
  double be2 = 0.0, be3 = 0.0;
  if (bt != 0.0) {
    be2 = b2 / bt;
    be3 = b3 / bt;
  }
  double be2s = be2 / sqrt(ystar);
  double be3s = be3 / sqrt(ystar);
  double bes_sq = be2s * be2s + be3s * be3s;
  double vbet = v2 * be2s + v3 * be3s;
  double q2s = 0.0, q3s = 0.0;
  if (bes_sq != 0.0) {
    q2s = be2s / bes_sq;
    q3s = be3s / bes_sq;
  }
  /* fast/slow normalisations (eq. A16), with their degenerate limits */
  double af_, as_;
  if ((cfsq - cssq) <= 0.0) { af_ = 1.0; as_ = 0.0; }
  else if ((csq - cssq) <= 0.0) { af_ = 0.0; as_ = 1.0; }
  else if ((cfsq - csq) <= 0.0) { af_ = 1.0; as_ = 0.0; }
  else {
    af_ = sqrt((csq - cssq) / (cfsq - cssq));
    as_ = sqrt((cfsq - csq) / (cfsq - cssq));
  }
  double sqd = sqrt(d), isqd = 1.0 / sqd;
  double sgn = (bxi < 0.0) ? -1.0 : 1.0;
  double c = sqrt(csq);
  double qf = cf * af_ * sgn, qs = cs * as_ * sgn;
  double afp = c * af_ * isqd, asp = c * as_ * isqd;
  double afpbb = afp * bt_star * bes_sq, aspbb = asp * bt_star * bes_sq;
  double vq = (v2 * q2s + v3 * q3s);
  double vax = sqrt(vaxsq);
  double nrm = 0.5 / csq;
  double cff = nrm * af_ * cf, css = nrm * as_ * cs;
  double qfh = qf * nrm, qsh = qs * nrm;
  double afd = nrm * afp * d, asd = nrm * asp * d;
  double afpb = nrm * afp * bt_star, aspb = nrm * asp * bt_star;
  ev[0] = v1 - cf;
  ev[1] = v1 - vax;
  ev[2] = v1 - cs;
  ev[3] = v1;
  ev[4] = v1 + cs;
  ev[5] = v1 + vax;
  ev[6] = v1 + cf;
  /* projection of du on the left eigenvectors (eq. B29), term by term */
  double afb = af_ * gm1 * nrm, asb = as_ * gm1 * nrm;
  double gm1a = gm1 / csq;
  a[0] = du[0] * (afb * (vsq - hp) + cff * (cf + v1) - qsh * vq - aspb);
  a[0] -= du[1] * (afb * v1 + cff);
  a[0] -= du[2] * (afb * v2 - qsh * q2s);
  a[0] -= du[3] * (afb * v3 - qsh * q3s);
  a[0] += du[4] * afb;
  a[0] += du[5] * (asd * q2s - afb * b2);
  a[0] += du[6] * (asd * q3s - afb * b3);
  a[1] = du[0] * (v2 * be3 - v3 * be2);
  a[1] -= du[2] * be3;
  a[1] += du[3] * be2;
  a[1] -= du[5] * sqd * be3 * sgn;
  a[1] += du[6] * sqd * be2 * sgn;
  a[1] *= 0.5;
  a[2] = du[0] * (asb * (vsq - hp) + css * (cs + v1) + qfh * vq + afpb);
  a[2] -= du[1] * (asb * v1 + css);
  a[2] -= du[2] * (asb * v2 + qfh * q2s);
  a[2] -= du[3] * (asb * v3 + qfh * q3s);
  a[2] += du[4] * asb;
  a[2] -= du[5] * (afd * q2s + asb * b2);
  a[2] -= du[6] * (afd * q3s + asb * b3);
  a[3] = du[0] * (1.0 - gm1a * (0.5 * vsq - (gm1 - 1.0) * x / gm1));
  a[3] += du[1] * gm1a * v1;
  a[3] += du[2] * gm1a * v2;
  a[3] += du[3] * gm1a * v3;
  a[3] -= du[4] * gm1a;
  a[3] += du[5] * gm1a * b2;
  a[3] += du[6] * gm1a * b3;
  a[4] = du[0] * (asb * (vsq - hp) + css * (cs - v1) - qfh * vq + afpb);
  a[4] -= du[1] * (asb * v1 - css);
  a[4] -= du[2] * (asb * v2 - qfh * q2s);
  a[4] -= du[3] * (asb * v3 - qfh * q3s);
  a[4] += du[4] * asb;
  a[4] -= du[5] * (afd * q2s + asb * b2);
  a[4] -= du[6] * (afd * q3s + asb * b3);
  a[5] = du[0] * (v3 * be2 - v2 * be3);
  a[5] += du[2] * be3;
  a[5] -= du[3] * be2;
  a[5] -= du[5] * sqd * be3 * sgn;
  a[5] += du[6] * sqd * be2 * sgn;
  a[5] *= 0.5;
  a[6] = du[0] * (afb * (vsq - hp) + cff * (cf - v1) + qsh * vq - aspb);
  a[6] -= du[1] * (afb * v1 - cff);
  a[6] -= du[2] * (afb * v2 + qsh * q2s);
  a[6] -= du[3] * (afb * v3 + qsh * q3s);
  a[6] += du[4] * afb;
  a[6] += du[5] * (asd * q2s - afb * b2);
  a[6] += du[6] * (asd * q3s - afb * b3);
  for (int n = 0; n < NWAVE; ++n) cf_[n] = -0.5 * fabs(ev[n]) * a[n];
  /* density of the intermediate states left to right (first row of the right
   * eigenvectors): a negative one selects the LLF flux below */
  int neg = 0;
  double dens = wli[IDN] + a[0] * af_;
  neg |= dens < 0.0;
  dens += a[2] * as_;
  neg |= dens < 0.0;
  dens += a[3];
  neg |= dens < 0.0;
  dens += a[4] * as_;
  neg |= dens < 0.0;
  /* dissipation: sum of the waves times the right eigenvectors (eq. B21) */
  flxi[0] += cf_[0] * af_;
  flxi[0] += cf_[2] * as_;
  flxi[0] += cf_[3];
  flxi[0] += cf_[4] * as_;
  flxi[0] += cf_[6] * af_;
  flxi[1] += cf_[0] * (af_ * (v1 - cf));
  flxi[1] += cf_[2] * (as_ * (v1 - cs));
  flxi[1] += cf_[3] * v1;
  flxi[1] += cf_[4] * (as_ * (v1 + cs));
  flxi[1] += cf_[6] * (af_ * (v1 + cf));
  flxi[2] += cf_[0] * (af_ * v2 + qs * be2s);
  flxi[2] -= cf_[1] * be3;
  flxi[2] += cf_[2] * (as_ * v2 - qf * be2s);
  flxi[2] += cf_[3] * v2;
  flxi[2] += cf_[4] * (as_ * v2 + qf * be2s);
  flxi[2] += cf_[5] * be3;
  flxi[2] += cf_[6] * (af_ * v2 - qs * be2s);
  flxi[3] += cf_[0] * (af_ * v3 + qs * be3s);
  flxi[3] += cf_[1] * be2;
  flxi[3] += cf_[2] * (as_ * v3 - qf * be3s);
  flxi[3] += cf_[3] * v3;
  flxi[3] += cf_[4] * (as_ * v3 + qf * be3s);
  flxi[3] -= cf_[5] * be2;
  flxi[3] += cf_[6] * (af_ * v3 - qs * be3s);
  flxi[4] += cf_[0] * (af_ * (hp - v1 * cf) + qs * vbet + aspbb);
  flxi[4] -= cf_[1] * (v2 * be3 - v3 * be2);
  flxi[4] += cf_[2] * (as_ * (hp - v1 * cs) - qf * vbet - afpbb);
  flxi[4] += cf_[3] * (0.5 * vsq + (gm1 - 1.0) * x / gm1);
  flxi[4] += cf_[4] * (as_ * (hp + v1 * cs) + qf * vbet - afpbb);
  flxi[4] += cf_[5] * (v1 * be3 - v3 * be2);
  flxi[4] += cf_[6] * (af_ * (hp + v1 * cf) - qs * vbet + aspbb);
  flxi[5] += cf_[0] * asp * be2s;
  flxi[5] -= cf_[1] * be3 * sgn * isqd;
  flxi[5] -= cf_[2] * afp * be2s;
  flxi[5] -= cf_[4] * afp * be2s;
  flxi[5] -= cf_[5] * be3 * sgn * isqd;
  flxi[5] += cf_[6] * asp * be2s;
  flxi[6] += cf_[0] * asp * be3s;
  flxi[6] += cf_[1] * be2 * sgn * isqd;
  flxi[6] -= cf_[2] * afp * be3s;
  flxi[6] -= cf_[4] * afp * be3s;
  flxi[6] += cf_[5] * be2 * sgn * isqd;
  flxi[6] += cf_[6] * asp * be3s;
  /* supersonic: the upwind flux */
  if (ev[0] >= 0.0)
    for (int n = 0; n < NWAVE; ++n) flxi[n] = fl[n];
  if (ev[NWAVE - 1] <= 0.0)
    for (int n = 0; n < NWAVE; ++n) flxi[n] = fr[n];
  if (neg) {
    double cl = fast_ms(gamma, wli, bxi), cr = fast_ms(gamma, wri, bxi);
    double s = 0.5 * smax((fabs(wli[IVX]) + cl), (fabs(wri[IVX]) + cr));
    for (int n = 0; n < NHYDRO; ++n) flxi[n] = 0.5 * (fl[n] + fr[n]) - s * du[n];
  }
}

/* The L and R states of the SR frame-transforming solvers (hlle_mhd_rel.cpp:160-260,
 * llf_mhd_rel.cpp:136-220, the same operations): conserved state and flux (MUB 8, 15) of
 * each side and its fast speeds.  Local order as for hlld(); velocities are the spatial
 * 4-velocity u^i. */
static void sr_states(double gamma_adi, const double *wli, const double *wri, double bb1,
                      double *cl, double *cr, double *fl, double *fr, double *lml,
                      double *lpl, double *lmr, double *lpr) {
  const double *wv[2] = {wli, wri};
  double *cv[2] = {cl, cr}, *fv[2] = {fl, fr}, *lm[2] = {lml, lmr}, *lp[2] = {lpl, lpr};
  for (int s = 0; s < 2; ++s) {
    const double *w = wv[s];
    double rho = w[IDN], pgas = w[IPR];
    double u[4];
    u[0] = sqrt(1.0 + SQR(w[IVX]) + SQR(w[IVY]) + SQR(w[IVZ]));
    u[1] = w[IVX]; u[2] = w[IVY]; u[3] = w[IVZ];
    double bb2 = w[IBY], bb3 = w[IBZ];
    double b[4];
    b[0] = bb1 * u[1] + bb2 * u[2] + bb3 * u[3];
    b[1] = (bb1 + b[0] * u[1]) / u[0];
    b[2] = (bb2 + b[0] * u[2]) / u[0];
    b[3] = (bb3 + b[0] * u[3]) / u[0];
    double b_sq = -SQR(b[0]) + SQR(b[1]) + SQR(b[2]) + SQR(b[3]);
    double wgas = rho + gamma_adi / (gamma_adi - 1.0) * pgas;
    sr_fast_speeds(gamma_adi, wgas, pgas, u[0], u[1], b_sq, lp[s], lm[s]);
    double wtot = wgas + b_sq, ptot = pgas + 0.5 * b_sq;
    double *c = cv[s], *f = fv[s];
    /* local slots: 0 mass, 1..3 momenta (normal, t1, t2), 4 energy, 5/6 fields */
    c[0] = rho * u[0];
    c[4] = wtot * u[0] * u[0] - b[0] * b[0] - ptot;
    c[1] = wtot * u[1] * u[0] - b[1] * b[0];
    c[2] = wtot * u[2] * u[0] - b[2] * b[0];
    c[3] = wtot * u[3] * u[0] - b[3] * b[0];
    c[5] = b[2] * u[0] - b[0] * u[2];
    c[6] = b[3] * u[0] - b[0] * u[3];
    f[0] = rho * u[1];
    f[4] = wtot * u[0] * u[1] - b[0] * b[1];
    f[1] = wtot * u[1] * u[1] - b[1] * b[1] + ptot;
    f[2] = wtot * u[2] * u[1] - b[2] * b[1];
    f[3] = wtot * u[3] * u[1] - b[3] * b[1];
    f[5] = b[2] * u[1] - b[1] * u[2];
    f[6] = b[3] * u[1] - b[1] * u[3];
  }
}

/* SR frame-transforming HLLE, hydro/rsolvers/mhd/hlle_mhd_rel.cpp:103-330 (SR branch) */
static void hlle_sr(double gamma_adi, const double *wli, const double *wri, double bb1,
                    double *f) {
  double cl[NWAVE], cr[NWAVE], fl[NWAVE], fr[NWAVE];
  double lml, lpl, lmr, lpr;
  sr_states(gamma_adi, wli, wri, bb1, cl, cr, fl, fr, &lml, &lpl, &lmr, &lpr);
  double lambda_l = smin(lml, lmr);
  double lambda_r = smax(lpl, lpr);
  double lambda_diff_inv = 1.0 / (lambda_r - lambda_l);
  const double v_interface = 0.0;
  for (int n = 0; n < NWAVE; ++n) {
    if (lambda_l >= v_interface) f[n] = fl[n];
    else if (lambda_r <= v_interface) f[n] = fr[n];
    else f[n] = (lambda_r * fl[n] - lambda_l * fr[n] + lambda_l * lambda_r * (cr[n] - cl[n])) *
                lambda_diff_inv;
  }
}

/* SR frame-transforming LLF, hydro/rsolvers/mhd/llf_mhd_rel.cpp:101-280 (SR branch):
 * lambda = max(lambda_r, -lambda_l) (MB 55), F = (F_l + F_r - lambda (U_r - U_l)) / 2 */
static void llf_sr(double gamma_adi, const double *wli, const double *wri, double bb1,
                   double *f) {
  double cl[NWAVE], cr[NWAVE], fl[NWAVE], fr[NWAVE];
  double lml, lpl, lmr, lpr;
  sr_states(gamma_adi, wli, wri, bb1, cl, cr, fl, fr, &lml, &lpl, &lmr, &lpr);
  double lambda_l = smin(lml, lmr);
  double lambda_r = smax(lpl, lpr);
  double lambda = smax(lambda_r, -lambda_l);
  for (int n = 0; n < NWAVE; ++n) f[n] = 0.5 * (fl[n] + fr[n] - lambda * (cr[n] - cl[n]));
}

/* 1/3 as the reference writes it (defs.hpp.in:144, ONE_3RD); the nearest double to 1/3 */
#define ORC_ONE_3RD 0.33333333333333333

/* the enthalpy residual and its derivative of the HLL state's total-pressure estimate
 * (Mignone & McKinney 2007 A1, A3, A11, A14-A18), hlld_rel.cpp:928-975 */
static double hlldsr_eres(double w_guess, double dd, double ee, double m_sq, double bb_sq, double ss_sq,
                    double gamma_prime) {
  double v_sq = (m_sq + ss_sq / SQR(w_guess) * (2.0 * w_guess + bb_sq)) / SQR(w_guess + bb_sq);
  double gamma_sq = 1.0 / (1.0 - v_sq);
  double gamma_lorentz = sqrt(gamma_sq);
  double chi = (1.0 - v_sq) * (w_guess - gamma_lorentz * dd);
  double pgas = chi / gamma_prime;
  double ee_calc = w_guess - pgas + 0.5 * bb_sq * (1.0 + v_sq) -
                 ss_sq / (2.0 * SQR(w_guess));
  return ee_calc - ee;
}

static double hlldsr_eres_prime(double w_guess, double dd, double m_sq, double bb_sq, double ss_sq,
                          double gamma_prime) {
  double v_sq = (m_sq + ss_sq / SQR(w_guess) * (2.0 * w_guess + bb_sq)) / SQR(w_guess + bb_sq);
  double gamma_sq = 1.0 / (1.0 - v_sq);
  double gamma_lorentz = sqrt(gamma_sq);
  double chi = (1.0 - v_sq) * (w_guess - gamma_lorentz * dd);
  double w_cu = SQR(w_guess) * w_guess;
  double w_b_cu = SQR(w_guess + bb_sq) * (w_guess + bb_sq);
  double dv_sq_dw = -2.0 / (w_cu * w_b_cu) *
                  (ss_sq * (3.0 * w_guess * (w_guess + bb_sq) + SQR(bb_sq)) + m_sq * w_cu);
  double dchi_dw = 1.0 - v_sq - gamma_lorentz / 2.0 * (dd + 2.0 * gamma_lorentz * chi) *
                                     dv_sq_dw;
  double drho_dw = -gamma_lorentz * dd / 2.0 * dv_sq_dw;
  double dpgas_dchi = 1.0 / gamma_prime;
  double dpgas_drho = 0.0;
  double dpgas_dw = dpgas_dchi * dchi_dw + dpgas_drho * drho_dw;
  return 1.0 - dpgas_dw + 0.5 * bb_sq * dv_sq_dw + ss_sq / w_cu;
}

/* the Alfven-region states of one total pressure ptot (MUB 21-49): the normal velocities
 * vx, vy, vz and transverse fields of the aL and aR regions, eta, K and the residual of
 * the contact condition (MUB 48), hlld_rel.cpp:437-517 (repeated at :521-598, :618-697) */
typedef struct {
  double vx_al, vy_al, vz_al, vx_ar, vy_ar, vz_ar;
  double kx_l, ky_l, kz_l, kx_r, ky_r, kz_r, eta_l, eta_r;
  double by_al, bz_al, by_ar, bz_ar, lambda_al, lambda_ar;
} hlldsr_alfven;

static double hlldsr_residual(double ptot, double bbx, double lambda_l, double lambda_r, const double *r_l,
                        const double *r_r, hlldsr_alfven *s) {
  const double delta_kx_aug = 1.0e-12;
  double al = r_l[1] - lambda_l * r_l[4] + ptot * (1.0 - SQR(lambda_l));
  double gl = SQR(r_l[5]) + SQR(r_l[6]);
  double cl = r_l[2] * r_l[5] + r_l[3] * r_l[6];
  double ql = -al - gl + SQR(bbx) * (1.0 - SQR(lambda_l));
  double xl_inv = 1.0 / (bbx * (al * lambda_l * bbx + cl) - (al + gl) * (lambda_l * ptot + r_l[4]));
  s->vx_al = (bbx * (al * bbx + lambda_l * cl) - (al + gl) * (ptot + r_l[1])) * xl_inv;
  s->vy_al = (ql * r_l[2] + r_l[5] * (cl + bbx * (lambda_l * r_l[1] - r_l[4]))) * xl_inv;
  s->vz_al = (ql * r_l[3] + r_l[6] * (cl + bbx * (lambda_l * r_l[1] - r_l[4]))) * xl_inv;
  double ar = r_r[1] - lambda_r * r_r[4] + ptot * (1.0 - SQR(lambda_r));
  double gr = SQR(r_r[5]) + SQR(r_r[6]);
  double cr = r_r[2] * r_r[5] + r_r[3] * r_r[6];
  double qr = -ar - gr + SQR(bbx) * (1.0 - SQR(lambda_r));
  double xr_inv = 1.0 / (bbx * (ar * lambda_r * bbx + cr) - (ar + gr) * (lambda_r * ptot + r_r[4]));
  s->vx_ar = (bbx * (ar * bbx + lambda_r * cr) - (ar + gr) * (ptot + r_r[1])) * xr_inv;
  s->vy_ar = (qr * r_r[2] + r_r[5] * (cr + bbx * (lambda_r * r_r[1] - r_r[4]))) * xr_inv;
  s->vz_ar = (qr * r_r[3] + r_r[6] * (cr + bbx * (lambda_r * r_r[1] - r_r[4]))) * xr_inv;
  s->by_al = (r_l[5] - bbx * s->vy_al) / (lambda_l - s->vx_al);
  s->bz_al = (r_l[6] - bbx * s->vz_al) / (lambda_l - s->vx_al);
  s->by_ar = (r_r[5] - bbx * s->vy_ar) / (lambda_r - s->vx_ar);
  s->bz_ar = (r_r[6] - bbx * s->vz_ar) / (lambda_r - s->vx_ar);
  double v_rm_l = s->vx_al * r_l[1] + s->vy_al * r_l[2] + s->vz_al * r_l[3];
  double wtot_al = ptot + (r_l[4] - v_rm_l) / (lambda_l - s->vx_al);
  double v_rm_r = s->vx_ar * r_r[1] + s->vy_ar * r_r[2] + s->vz_ar * r_r[3];
  double wtot_ar = ptot + (r_r[4] - v_rm_r) / (lambda_r - s->vx_ar);
  s->eta_l = -copysign(sqrt(wtot_al), bbx);
  s->eta_r = copysign(sqrt(wtot_ar), bbx);
  double denom_al_inv = 1.0 / (lambda_l * ptot + r_l[4] + bbx * s->eta_l);
  s->kx_l = (r_l[1] + ptot + lambda_l * bbx * s->eta_l) * denom_al_inv;
  s->ky_l = (r_l[2] + r_l[5] * s->eta_l) * denom_al_inv;
  s->kz_l = (r_l[3] + r_l[6] * s->eta_l) * denom_al_inv;
  double denom_ar_inv = 1.0 / (lambda_r * ptot + r_r[4] + bbx * s->eta_r);
  s->kx_r = (r_r[1] + ptot + lambda_r * bbx * s->eta_r) * denom_ar_inv;
  s->ky_r = (r_r[2] + r_r[5] * s->eta_r) * denom_ar_inv;
  s->kz_r = (r_r[3] + r_r[6] * s->eta_r) * denom_ar_inv;
  s->lambda_al = s->kx_l;
  s->lambda_ar = s->kx_r;
  double delta_kx = s->kx_r - s->kx_l + delta_kx_aug;
  double bbx_c_delta_kx = bbx * delta_kx;
  double by_c_delta_kx = s->by_ar * (s->lambda_ar - s->vx_ar) - s->by_al * (s->lambda_al - s->vx_al) +
                       bbx * (s->vy_ar - s->vy_al);
  double bz_c_delta_kx = s->bz_ar * (s->lambda_ar - s->vx_ar) - s->bz_al * (s->lambda_al - s->vx_al) +
                       bbx * (s->vz_ar - s->vz_al);
  double k_sq_l = SQR(s->kx_l) + SQR(s->ky_l) + SQR(s->kz_l);
  double k_dot_bc_delta_kx = s->kx_l * bbx_c_delta_kx + s->ky_l * by_c_delta_kx +
                           s->kz_l * bz_c_delta_kx;
  double y_l = (1.0 - k_sq_l) / (s->eta_l * delta_kx - k_dot_bc_delta_kx);
  double k_sq_r = SQR(s->kx_r) + SQR(s->ky_r) + SQR(s->kz_r);
  k_dot_bc_delta_kx = s->kx_r * bbx_c_delta_kx + s->ky_r * by_c_delta_kx +
                      s->kz_r * bz_c_delta_kx;
  double y_r = (1.0 - k_sq_r) / (s->eta_r * delta_kx - k_dot_bc_delta_kx);
  return delta_kx * (1.0 - bbx * (y_r - y_l));
}

/* SR frame-transforming HLLD (Mignone, Ugliano & Bodo 2009), hydro/rsolvers/mhd/
 * hlld_rel.cpp:116-890 (SR branch): L, R and HLL states, the HLL total pressure from two
 * Newton steps on the enthalpy (MM A26-A27), the initial total pressure (MUB 53-55), four
 * secant steps on the contact condition, the aL, aR and contact states, the region of the
 * fan at the interface, HLL where anything is not finite. */
static void hlld_sr(double gamma_adi, const double *wli, const double *wri, double bbx, double *f) {
  const double p_transition = 0.01, vc_extension = 1.0e-6;
  const double delta_kx_aug = 1.0e-12;
  const double gamma_prime = gamma_adi / (gamma_adi - 1.0);
  const int num_secant = 4;
  const double initial_offset = 1.0e-5, tol_res = 1.0e-12;
  double cons_l[7], flux_l[7], cons_r[7], flux_r[7], r_l[7], r_r[7], cons_hll[7], flux_hll[7];
  double cons_al[7], flux_al[7], cons_ar[7], flux_ar[7], cons_c[7], flux_c[7];
  double lml, lpl, lmr, lpr;
  sr_states(gamma_adi, wli, wri, bbx, cons_l, cons_r, flux_l, flux_r, &lml, &lpl, &lmr, &lpr);
  const double lambda_l = smin(lml, lmr);
  const double lambda_r = smax(lpl, lpr);
  for (int n = 0; n < 7; ++n) r_l[n] = lambda_l * cons_l[n] - flux_l[n];
  for (int n = 0; n < 7; ++n) r_r[n] = lambda_r * cons_r[n] - flux_r[n];
  double lambda_diff_inv = 1.0 / (lambda_r - lambda_l);
  for (int n = 0; n < 7; ++n) cons_hll[n] = (r_r[n] - r_l[n]) * lambda_diff_inv;
  for (int n = 0; n < 7; ++n) flux_hll[n] = (lambda_l * r_r[n] - lambda_r * r_l[n]) * lambda_diff_inv;
  /* total pressure of the HLL state */
  double ptot_hll;
  {
    double m_sq = SQR(cons_hll[1]) + SQR(cons_hll[2]) + SQR(cons_hll[3]);
    double bb_sq = SQR(bbx) + SQR(cons_hll[5]) + SQR(cons_hll[6]);
    double m_dot_bb = cons_hll[1] * bbx + cons_hll[2] * cons_hll[5] + cons_hll[3] * cons_hll[6];
    double ss_sq = SQR(m_dot_bb);
    double a1 = 4.0 / 3.0 * (bb_sq - cons_hll[4]);
    double a0 = ORC_ONE_3RD * (m_sq + bb_sq * (bb_sq - 2.0 * cons_hll[4]));
    double s2 = SQR(a1) - 4.0 * a0;
    double s = (s2 < 0.0) ? 0.0 : sqrt(s2);
    double w_init = (s2 >= 0.0 && a1 >= 0.0) ? -2.0 * a0 / (a1 + s) : 0.5 * (-a1 + s);
    double w_new = w_init;
    double res_new = hlldsr_eres(w_new, cons_hll[0], cons_hll[4], m_sq, bb_sq, ss_sq, gamma_prime);
    for (int n = 0; n < 2; ++n) {
      double w_old = w_new;
      double res_old = res_new;
      double derivative = hlldsr_eres_prime(w_old, cons_hll[0], m_sq, bb_sq, ss_sq, gamma_prime);
      double delta = -res_old / derivative;
      w_new = w_old + delta;
      res_new = hlldsr_eres(w_new, cons_hll[0], cons_hll[4], m_sq, bb_sq, ss_sq, gamma_prime);
    }
    double w = w_new;
    double v_sq = (m_sq + ss_sq / SQR(w) * (2.0 * w + bb_sq)) / SQR(w + bb_sq);
    double gamma_lor_sq = 1.0 / (1.0 - v_sq);
    double gamma_lor = sqrt(gamma_lor_sq);
    double chi = (1.0 - v_sq) * (w - gamma_lor * cons_hll[0]);
    double pgas = 1.0 / gamma_prime * chi;
    double vx = (cons_hll[1] + m_dot_bb / w * bbx) / (w + bb_sq);
    double vy = (cons_hll[2] + m_dot_bb / w * cons_hll[5]) / (w + bb_sq);
    double vz = (cons_hll[3] + m_dot_bb / w * cons_hll[6]) / (w + bb_sq);
    double v_bb = vx * bbx + vy * cons_hll[5] + vz * cons_hll[6];
    double b_sq = bb_sq / gamma_lor_sq + SQR(v_bb);
    ptot_hll = pgas + 0.5 * b_sq;
  }
  double ptot_init;
  if (SQR(bbx) / ptot_hll < p_transition) {  /* weak field (MUB 55) */
    double a1 = cons_hll[4] - flux_hll[1];
    double a0 = cons_hll[1] * flux_hll[4] - flux_hll[1] * cons_hll[4];
    double s2 = SQR(a1) - 4.0 * a0;
    double s = (s2 < 0.0) ? 0.0 : sqrt(s2);
    ptot_init = (s2 >= 0.0 && a1 >= 0.0) ? -2.0 * a0 / (a1 + s) : (-a1 + s) / 2.0;
  } else {
    ptot_init = ptot_hll;
  }
  int switch_to_hlle = 0;
  if (!isfinite(ptot_init) || ptot_init <= 0.0) switch_to_hlle = 1;
  /* secant iteration on the total pressure (MUB 48) */
  hlldsr_alfven st;
  double ptot_0 = ptot_init;
  double res_0 = hlldsr_residual(ptot_0, bbx, lambda_l, lambda_r, r_l, r_r, &st);
  double ptot_1 = ptot_init * (1.0 + initial_offset);
  double res_1 = hlldsr_residual(ptot_1, bbx, lambda_l, lambda_r, r_l, r_r, &st);
  double ptot_last = ptot_0, ptot_n = ptot_1, res_last = res_0, res_n = res_1;
  const double tol_ptot = 1.0e-8 * ptot_init;
  for (int n = 0; n < num_secant; ++n) {
    double ptot_old = ptot_last;
    ptot_last = ptot_n;
    double res_old = res_last;
    res_last = res_n;
    int need_to_iterate = fabs(res_last) > tol_res && fabs(ptot_last - ptot_old) > tol_ptot;
    if (need_to_iterate)
      ptot_n = (res_last * ptot_old - res_old * ptot_last) / (res_last - res_old);
    else
      ptot_n = ptot_last;
    res_n = hlldsr_residual(ptot_n, bbx, lambda_l, lambda_r, r_l, r_r, &st);
  }
  const double ptot_c = ptot_n;
  const double lambda_al = st.lambda_al, lambda_ar = st.lambda_ar;
  if (!isfinite(lambda_al) || !isfinite(lambda_ar) || !isfinite(ptot_c) || ptot_c <= 0.0)
    switch_to_hlle = 1;
  const double vx_al = st.vx_al, vy_al = st.vy_al, vz_al = st.vz_al;
  const double vx_ar = st.vx_ar, vy_ar = st.vy_ar, vz_ar = st.vz_ar;
  cons_al[5] = st.by_al;
  cons_al[6] = st.bz_al;
  cons_ar[5] = st.by_ar;
  cons_ar[6] = st.bz_ar;
  /* the aL and aR states (MUB 32-34) */
  double v_bb_al = vx_al * bbx + vy_al * cons_al[5] + vz_al * cons_al[6];
  cons_al[0] = r_l[0] / (lambda_l - vx_al);
  cons_al[4] = (r_l[4] + ptot_c * vx_al - v_bb_al * bbx) / (lambda_l - vx_al);
  cons_al[1] = (cons_al[4] + ptot_c) * vx_al - v_bb_al * bbx;
  cons_al[2] = (cons_al[4] + ptot_c) * vy_al - v_bb_al * cons_al[5];
  cons_al[3] = (cons_al[4] + ptot_c) * vz_al - v_bb_al * cons_al[6];
  double v_bb_ar = vx_ar * bbx + vy_ar * cons_ar[5] + vz_ar * cons_ar[6];
  cons_ar[0] = r_r[0] / (lambda_r - vx_ar);
  cons_ar[4] = (r_r[4] + ptot_c * vx_ar - v_bb_ar * bbx) / (lambda_r - vx_ar);
  cons_ar[1] = (cons_ar[4] + ptot_c) * vx_ar - v_bb_ar * bbx;
  cons_ar[2] = (cons_ar[4] + ptot_c) * vy_ar - v_bb_ar * cons_ar[5];
  cons_ar[3] = (cons_ar[4] + ptot_c) * vz_ar - v_bb_ar * cons_ar[6];
  for (int n = 0; n < 7; ++n) flux_al[n] = lambda_l * cons_al[n] - r_l[n];
  for (int n = 0; n < 7; ++n) flux_ar[n] = lambda_r * cons_ar[n] - r_r[n];
  /* the contact state (MUB 45, 47, 50-52) */
  double denom_c_inv = 1.0 / (lambda_ar - lambda_al + delta_kx_aug);
  double numer_al = cons_al[5] * (lambda_al - vx_al) + bbx * vy_al;
  double numer_ar = cons_ar[5] * (lambda_ar - vx_ar) + bbx * vy_ar;
  cons_c[5] = (numer_ar - numer_al) * denom_c_inv;
  numer_al = cons_al[6] * (lambda_al - vx_al) + bbx * vz_al;
  numer_ar = cons_ar[6] * (lambda_ar - vx_ar) + bbx * vz_ar;
  cons_c[6] = (numer_ar - numer_al) * denom_c_inv;
  const double kx_l = st.kx_l, ky_l = st.ky_l, kz_l = st.kz_l, eta_l = st.eta_l;
  const double kx_r = st.kx_r, ky_r = st.ky_r, kz_r = st.kz_r, eta_r = st.eta_r;
  double k_sq_l = SQR(kx_l) + SQR(ky_l) + SQR(kz_l);
  double k_bc_l = kx_l * bbx + ky_l * cons_c[5] + kz_l * cons_c[6];
  double vx_cl = kx_l - bbx * (1.0 - k_sq_l) / (eta_l - k_bc_l);
  double vy_cl = ky_l - cons_c[5] * (1.0 - k_sq_l) / (eta_l - k_bc_l);
  double vz_cl = kz_l - cons_c[6] * (1.0 - k_sq_l) / (eta_l - k_bc_l);
  double k_sq_r = SQR(kx_r) + SQR(ky_r) + SQR(kz_r);
  double k_bc_r = kx_r * bbx + ky_r * cons_c[5] + kz_r * cons_c[6];
  double vx_cr = kx_r - bbx * (1.0 - k_sq_r) / (eta_r - k_bc_r);
  double vy_cr = ky_r - cons_c[5] * (1.0 - k_sq_r) / (eta_r - k_bc_r);
  double vz_cr = kz_r - cons_c[6] * (1.0 - k_sq_r) / (eta_r - k_bc_r);
  double vx_c = 0.5 * (vx_cl + vx_cr);
  double vy_c = 0.5 * (vy_cl + vy_cr);
  double vz_c = 0.5 * (vz_cl + vz_cr);
  double v_bb_c = vx_c * bbx + vy_c * cons_c[5] + vz_c * cons_c[6];
  if (vx_c >= 0.0) {
    cons_c[0] = cons_al[0] * (lambda_al - vx_al) / (lambda_al - vx_c);
    cons_c[4] = (lambda_al * cons_al[4] - cons_al[1] + ptot_c * vx_c - v_bb_c * bbx) /
                (lambda_al - vx_c);
  } else {
    cons_c[0] = cons_ar[0] * (lambda_ar - vx_ar) / (lambda_ar - vx_c);
    cons_c[4] = (lambda_ar * cons_ar[4] - cons_ar[1] + ptot_c * vx_c - v_bb_c * bbx) /
                (lambda_ar - vx_c);
  }
  cons_c[1] = (cons_c[4] + ptot_c) * vx_c - v_bb_c * bbx;
  cons_c[2] = (cons_c[4] + ptot_c) * vy_c - v_bb_c * cons_c[5];
  cons_c[3] = (cons_c[4] + ptot_c) * vz_c - v_bb_c * cons_c[6];
  for (int n = 0; n < 7; ++n) {
    if (vx_c >= 0.0)
      flux_c[n] = flux_al[n] + lambda_al * (cons_c[n] - cons_al[n]);
    else
      flux_c[n] = flux_ar[n] + lambda_ar * (cons_c[n] - cons_ar[n]);
  }
  /* the region of the fan at the interface (v_interface = 0 in SR) */
  const double v_interface = 0.0;
  const double *ci, *fi;
  if (lambda_l >= v_interface) { ci = cons_l; fi = flux_l; }
  else if (lambda_r <= v_interface) { ci = cons_r; fi = flux_r; }
  else if (switch_to_hlle) { ci = cons_hll; fi = flux_hll; }
  else if (lambda_al >= v_interface - vc_extension) { ci = cons_al; fi = flux_al; }
  else if (lambda_ar <= v_interface + vc_extension) { ci = cons_ar; fi = flux_ar; }
  else { ci = cons_c; fi = flux_c; }
  if (!switch_to_hlle) {
    for (int n = 0; n < 7; ++n)
      if (!isfinite(ci[n]) || !isfinite(fi[n])) switch_to_hlle = 1;
    if (switch_to_hlle) { ci = cons_hll; fi = flux_hll; }
  }
  for (int n = 0; n < 7; ++n) f[n] = fi[n];
}

/* ------------------------------------------------------------------------------------
 * Reconstruction of one cell along a direction: given the 7-component wave vector of the
 * cell and its neighbours, return the value at its upper face (qlp, becomes wl of the
 * next face) and at its lower face (qrm, becomes wr of this face).
 */

/* PiecewiseLinearX1/2/3 uniform van Leer branch, plm.cpp:103-112 and :148-152 */
static void plm_cell(const double *qm, const double *q0, const double *qp, double cp,
                     double cm, double *qlp, double *qrm) {
  for (int n = 0; n < NWAVE; ++n) {
    double dwl = (q0[n] - qm[n]);
    double dwr = (qp[n] - q0[n]);
    double dw2 = dwl * dwr;
    double dwm = 2.0 * dw2 / (dwl + dwr);
    if (dw2 <= 0.0) dwm = 0.0;
    qlp[n] = q0[n] + cp * dwm;
    qrm[n] = q0[n] - cm * dwm;
  }
}

/* PiecewiseParabolicX1/2/3 uniform-Cartesian CS08 branch, ppm.cpp:113-315, or with
 * fast != 0 PiecewiseParabolicFastX1/2/3 (ppm_fast.cpp: the same interface values, the
 * Mignone limiter, no floors);
 * coefficients c1..c6 = 1/2,1/2,1/2,1/2,1/6,-1/6 (reconstruction.cpp:499-504);
 * floors ppm.cpp:326-331.  q[0..4] = cells i-2..i+2. */
static void ppm_cell(const double *const q[5], double dfloor, double pfloor, int fast,
                     double *qlp, double *qrm) {
  const double C2 = 1.25;
  const double c1 = 0.5, c2 = 0.5, c3 = 0.5, c4 = 0.5, c5 = 1.0 / 6.0, c6 = -1.0 / 6.0;
  for (int n = 0; n < NWAVE; ++n) {
    double q_im2 = q[0][n], q_im1 = q[1][n], qc = q[2][n], q_ip1 = q[3][n], q_ip2 = q[4][n];
    double qa = (qc - q_im1);
    double qb = (q_ip1 - qc);
    double dd_im1 = c1 * qa + c2 * (q_im1 - q_im2);
    double dd = c1 * qb + c2 * qa;
    double dd_ip1 = c1 * (q_ip2 - q_ip1) + c2 * qb;
    double dph = (c3 * q_im1 + c4 * qc) + (c5 * dd_im1 + c6 * dd);
    double dph_ip1 = (c3 * qc + c4 * q_ip1) + (c5 * dd + c6 * dd_ip1);

    double d2qc_im1 = q_im2 + qc - 2.0 * q_im1;
    double d2qc = q_im1 + q_ip1 - 2.0 * qc;
    double d2qc_ip1 = qc + q_ip2 - 2.0 * q_ip1;

    { /* i-1/2 */
      double qa_tmp = dph - q_im1;
      double qb_tmp = qc - dph;
      double a = 3.0 * (q_im1 + qc - 2.0 * dph);
      double b = d2qc_im1, c = d2qc, d = 0.0;
      if (SIGN(a) == SIGN(b) && SIGN(a) == SIGN(c))
        d = SIGN(a) * smin(C2 * fabs(b), smin(C2 * fabs(c), fabs(a)));
      double dph_tmp = 0.5 * (q_im1 + qc) - d / 6.0;
      if (qa_tmp * qb_tmp < 0.0) dph = dph_tmp;
    }
    { /* i+1/2 */
      double qa_tmp = dph_ip1 - qc;
      double qb_tmp = q_ip1 - dph_ip1;
      double a = 3.0 * (qc + q_ip1 - 2.0 * dph_ip1);
      double b = d2qc, c = d2qc_ip1, d = 0.0;
      if (SIGN(a) == SIGN(b) && SIGN(a) == SIGN(c))
        d = SIGN(a) * smin(C2 * fabs(b), smin(C2 * fabs(c), fabs(a)));
      double dphip1_tmp = 0.5 * (qc + q_ip1) - d / 6.0;
      if (qa_tmp * qb_tmp < 0.0) dph_ip1 = dphip1_tmp;
    }
    double qminus = dph, qplus = dph_ip1;
    double dqf_minus = qc - qminus;
    double dqf_plus = qplus - qc;
    if (fast) { /* time/xorder = 3f: Mignone's limiter of the parabola (ppm_fast.cpp:142-165,
                 * ratios 2 on a uniform Cartesian mesh, reconstruction.cpp:490-491) */
      if (dqf_minus * dqf_plus <= 0.0) {
        qminus = qc;
        qplus = qc;
      } else {
        if (fabs(dqf_minus) >= 2.0 * fabs(dqf_plus)) qminus = qc - 2.0 * dqf_plus;
        if (fabs(dqf_plus) >= 2.0 * fabs(dqf_minus)) qplus = qc + 2.0 * dqf_minus;
      }
      qlp[n] = qplus;
      qrm[n] = qminus;
      continue;
    }
    double d2qf = 6.0 * (dph + dph_ip1 - 2.0 * qc);
    { /* CS limiter, ppm.cpp:234-288 */
      double qa_tmp = dqf_minus * dqf_plus;
      double qb_tmp = (q_ip1 - qc) * (qc - q_im1);
      double a = d2qc_im1, b = d2qc, c = d2qc_ip1, d = d2qf, e = 0.0;
      if (SIGN(a) == SIGN(b) && SIGN(a) == SIGN(c) && SIGN(a) == SIGN(d))
        e = SIGN(d) * smin(smin(C2 * fabs(a), C2 * fabs(b)), smin(C2 * fabs(c), fabs(d)));
      a = smax(fabs(q_im1), fabs(q_im2));
      b = smax(smax(fabs(qc), fabs(q_ip1)), fabs(q_ip2));
      double rho = 0.0;
      if (fabs(d) > (1.0e-12) * smax(a, b)) rho = e / d;
      double tmp_m = qc - rho * dqf_minus;
      double tmp_p = qc + rho * dqf_plus;
      double tmp2_m = qc - 2.0 * dqf_plus;
      double tmp2_p = qc + 2.0 * dqf_minus;
      if ((qa_tmp <= 0.0 || qb_tmp <= 0.0)) {
        if (rho <= (1.0 - (1.0e-12))) {
          qminus = tmp_m;
          qplus = tmp_p;
        }
      } else {
        if (fabs(dqf_minus) >= 2.0 * fabs(dqf_plus)) qminus = tmp2_m;
        if (fabs(dqf_plus) >= 2.0 * fabs(dqf_minus)) qplus = tmp2_p;
      }
    }
    qlp[n] = qplus;
    qrm[n] = qminus;
  }
  if (fast) return; /* time/floor_ppm_fast defaults to false (reconstruction.cpp:42) */
  /* ApplyPrimitiveFloors, adiabatic_mhd.cpp:162-172 */
  qlp[IDN] = (qlp[IDN] > dfloor) ? qlp[IDN] : dfloor;
  qlp[IPR] = (qlp[IPR] > pfloor) ? qlp[IPR] : pfloor;
  qrm[IDN] = (qrm[IDN] > dfloor) ? qrm[IDN] : dfloor;
  qrm[IPR] = (qrm[IPR] > pfloor) ? qrm[IPR] : pfloor;
}

/* ------------------------------------------------------------------------------------
 * Hydro::CalculateFluxes, calculate_fluxes.cpp:38-415 (MHD, 3-D, order 1/2/3)
 */

/* wave vector of cell (k,j,i) for sweep direction dir: w in natural order, then the
 * two transverse cell-centred field components (plm.cpp:45-57 for x1, :196-208 for x2,
 * x3 analogous). */
static void load_wave(const orc_mesh *m, const double *w, const double *bcc, int dir, int k,
                      int j, int i, double *q) {
  for (int n = 0; n < NHYDRO; ++n) q[n] = w[CIDX(m, n, k, j, i)];
  q[IBY] = bcc[CIDX(m, (dir + 1) % 3, k, j, i)];
  q[IBZ] = bcc[CIDX(m, (dir + 2) % 3, k, j, i)];
}

/* recon of cell c along dir; returns upper-face (qlp) and lower-face (qrm) states */
static void recon_cell(const orc_mesh *m, int b, const double *w, const double *bcc,
                       int order, int dir, int k, int j, int i, double *qlp, double *qrm) {
  int dk = (dir == 2), dj = (dir == 1), di = (dir == 0);
  if (order == 1) { /* DonorCellX1/2/3, dc.cpp:24-104 */
    load_wave(m, w, bcc, dir, k, j, i, qlp);
    memcpy(qrm, qlp, sizeof(double) * NWAVE);
  } else if (order == 2) {
    double qm[NWAVE], q0[NWAVE], qp[NWAVE];
    load_wave(m, w, bcc, dir, k - dk, j - dj, i - di, qm);
    load_wave(m, w, bcc, dir, k, j, i, q0);
    load_wave(m, w, bcc, dir, k + dk, j + dj, i + di, qp);
    /* (x?f(c+1) - x?v(c))/dx?f(c) and (x?v(c) - x?f(c))/dx?f(c), plm.cpp:148-152 */
    const double *xf, *xv, *dxf;
    int c;
    if (dir == 0) {
      xf = m->x1f + (long)b * (m->nc1 + 1); xv = m->x1v + (long)b * m->nc1;
      dxf = m->dx1f + (long)b * m->nc1; c = i;
    } else if (dir == 1) {
      xf = m->x2f + (long)b * (m->nc2 + 1); xv = m->x2v + (long)b * m->nc2;
      dxf = m->dx2f + (long)b * m->nc2; c = j;
    } else {
      xf = m->x3f + (long)b * (m->nc3 + 1); xv = m->x3v + (long)b * m->nc3;
      dxf = m->dx3f + (long)b * m->nc3; c = k;
    }
    double cp = (xf[c + 1] - xv[c]) / dxf[c];
    double cm = (xv[c] - xf[c]) / dxf[c];
    plm_cell(qm, q0, qp, cp, cm, qlp, qrm);
  } else {
    double qs[5][NWAVE];
    const double *qp[5];
    for (int s = 0; s < 5; ++s) {
      load_wave(m, w, bcc, dir, k + (s - 2) * dk, j + (s - 2) * dj, i + (s - 2) * di, qs[s]);
      qp[s] = qs[s];
    }
    ppm_cell(qp, m->p.dfloor, m->p.pfloor, m->p.ppm_fast, qlp, qrm);
  }
}

/* Hydro::CalculateVelocityDifferences, hydro/calculate_velocity_differences.cpp:20-64
 * (3-D branch): at the face between cells c-1 and c along dir (c = (k, j, i)), dvn is the
 * jump of the normal velocity and dvt the smallest one-sided transverse derivative of the
 * transverse velocities in the two cells.  w: the block's primitives [5][nc3][nc2][nc1]. */
static void vel_diffs(const orc_mesh *m, const double *w, int dir, int k, int j, int i,
                      double *dvn, double *dvt) {
  long vs = m->ncell, sj = m->nc1, sk = (long)m->nc1 * m->nc2;
#define W(n, kk, jj, ii) w[(n) * vs + (kk) * sk + (jj) * sj + (ii)]
  if (dir == 0) {
    *dvn = W(IVX, k, j, i) - W(IVX, k, j, i - 1);
    double dvl = smin(W(IVY, k, j + 1, i - 1) - W(IVY, k, j, i - 1),
                      W(IVY, k, j, i - 1) - W(IVY, k, j - 1, i - 1));
    double dvr = smin(W(IVY, k, j + 1, i) - W(IVY, k, j, i),
                      W(IVY, k, j, i) - W(IVY, k, j - 1, i));
    double dwl = smin(W(IVZ, k + 1, j, i - 1) - W(IVZ, k, j, i - 1),
                      W(IVZ, k, j, i - 1) - W(IVZ, k - 1, j, i - 1));
    double dwr = smin(W(IVZ, k + 1, j, i) - W(IVZ, k, j, i),
                      W(IVZ, k, j, i) - W(IVZ, k - 1, j, i));
    *dvt = smin(smin(dvl, dvr), smin(dwl, dwr));
  } else if (dir == 1) {
    *dvn = W(IVY, k, j, i) - W(IVY, k, j - 1, i);
    double dvl = smin(W(IVZ, k + 1, j - 1, i) - W(IVZ, k, j - 1, i),
                      W(IVZ, k, j - 1, i) - W(IVZ, k - 1, j - 1, i));
    double dvr = smin(W(IVZ, k + 1, j, i) - W(IVZ, k, j, i),
                      W(IVZ, k, j, i) - W(IVZ, k - 1, j, i));
    double dwl = smin(W(IVX, k, j - 1, i + 1) - W(IVX, k, j - 1, i),
                      W(IVX, k, j - 1, i) - W(IVX, k, j - 1, i - 1));
    double dwr = smin(W(IVX, k, j, i + 1) - W(IVX, k, j, i),
                      W(IVX, k, j, i) - W(IVX, k, j, i - 1));
    *dvt = smin(smin(dvl, dvr), smin(dwl, dwr));
  } else {
    *dvn = W(IVZ, k, j, i) - W(IVZ, k - 1, j, i);
    double dvl = smin(W(IVX, k - 1, j, i + 1) - W(IVX, k - 1, j, i),
                      W(IVX, k - 1, j, i) - W(IVX, k - 1, j, i - 1));
    double dvr = smin(W(IVX, k, j, i + 1) - W(IVX, k, j, i),
                      W(IVX, k, j, i) - W(IVX, k, j, i - 1));
    double dwl = smin(W(IVY, k - 1, j + 1, i) - W(IVY, k - 1, j, i),
                      W(IVY, k - 1, j, i) - W(IVY, k - 1, j - 1, i));
    double dwr = smin(W(IVY, k, j + 1, i) - W(IVY, k, j, i),
                      W(IVY, k, j, i) - W(IVY, k, j - 1, i));
    *dvt = smin(smin(dvl, dvr), smin(dwl, dwr));
  }
#undef W
}

/* dvn, dvt: the face's velocity differences (vel_diffs; read by LHLLD only) */
static void riemann(const orc_mesh *m, int dir, const double *wl, const double *wr,
                    double bx, double dvn, double dvt, double *flx7) {
  /* local order: IDN, v_normal, v_t1, v_t2, p, IBY, IBZ; ivx = IVX+dir,
   * ivy = IVX+(dir+1)%3, ivz = IVX+(dir+2)%3 (hlld.cpp:42-43, 59-75) */
  int ivx = IVX + dir, ivy = IVX + (dir + 1) % 3, ivz = IVX + (dir + 2) % 3;
  double wli[NWAVE] = {wl[IDN], wl[ivx], wl[ivy], wl[ivz], wl[IPR], wl[IBY], wl[IBZ]};
  double wri[NWAVE] = {wr[IDN], wr[ivx], wr[ivy], wr[ivz], wr[IPR], wr[IBY], wr[IBZ]};
  if (m->p.relativistic && m->p.rsolver == 2) llf_sr(m->p.gamma, wli, wri, bx, flx7);
  else if (m->p.relativistic && m->p.rsolver == 0) hlld_sr(m->p.gamma, wli, wri, bx, flx7);
  else if (m->p.relativistic) hlle_sr(m->p.gamma, wli, wri, bx, flx7);
  else if (m->p.rsolver == 0) hlld(m->p.gamma, wli, wri, bx, flx7);
  else if (m->p.rsolver == 2) llf(m->p.gamma, wli, wri, bx, flx7);
  else if (m->p.rsolver == 3) roe(m->p.gamma, wli, wri, bx, flx7);
  else if (m->p.rsolver == 4) hlld_core(m->p.gamma, wli, wri, bx, 1, dvn, dvt, flx7);
  else hlle(m->p.gamma, wli, wri, bx, flx7);
}

static void calculate_fluxes(orc_mesh *m, int b, int order, scratch *s) {
  const double *w = m->w + (long)b * NHYDRO * m->ncell;
  const double *bcc = m->bcc + (long)b * 3 * m->ncell;
  const double *b1 = m->b1 + (long)b * m->nf1, *b2 = m->b2 + (long)b * m->nf2,
               *b3 = m->b3 + (long)b * m->nf3;
  const double *dx1f = m->dx1f + (long)b * m->nc1, *dx2f = m->dx2f + (long)b * m->nc2,
               *dx3f = m->dx3f + (long)b * m->nc3;
  double dt = m->dt;
  int is = m->is, ie = m->ie, js = m->js, je = m->je, ks = m->ks, ke = m->ke;
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1), n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1,
       n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  double wl[NWAVE], wr[NWAVE], tmp[NWAVE], f[NWAVE];

  /* x1: k in [ks-1,ke+1], j in [js-1,je+1], faces i in [is,ie+1] (:64-76, :78-102) */
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j)
      for (int i = is; i <= ie + 1; ++i) {
        recon_cell(m, b, w, bcc, order, 0, k, j, i - 1, wl, tmp);
        recon_cell(m, b, w, bcc, order, 0, k, j, i, tmp, wr);
        long fi = F1IDX(m, k, j, i);
        double dvn = 0.0, dvt = 0.0;
        if (m->p.rsolver == 4) vel_diffs(m, w, 0, k, j, i, &dvn, &dvt);
        riemann(m, 0, wl, wr, b1[fi], dvn, dvt, f);
        s->flx1[0 * n1 + fi] = f[0];
        s->flx1[1 * n1 + fi] = f[1];
        s->flx1[2 * n1 + fi] = f[2];
        s->flx1[3 * n1 + fi] = f[3];
        s->flx1[4 * n1 + fi] = f[4];
        s->e3x1[fi] = -f[5];
        s->e2x1[fi] = f[6];
        s->w1f[fi] = weight_for_ct(f[0], wl[IDN], wr[IDN], dx1f[i], dt);
      }
  /* x2: k in [ks-1,ke+1], i in [is-1,ie+1], faces j in [js,je+1] (:169-237) */
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js; j <= je + 1; ++j)
      for (int i = is - 1; i <= ie + 1; ++i) {
        recon_cell(m, b, w, bcc, order, 1, k, j - 1, i, wl, tmp);
        recon_cell(m, b, w, bcc, order, 1, k, j, i, tmp, wr);
        long fi = F2IDX(m, k, j, i);
        double dvn = 0.0, dvt = 0.0;
        if (m->p.rsolver == 4) vel_diffs(m, w, 1, k, j, i, &dvn, &dvt);
        riemann(m, 1, wl, wr, b2[fi], dvn, dvt, f);
        /* flux slots: IDN, ivx=IVY, ivy=IVZ, ivz=IVX, IEN */
        s->flx2[0 * n2 + fi] = f[0];
        s->flx2[2 * n2 + fi] = f[1];
        s->flx2[3 * n2 + fi] = f[2];
        s->flx2[1 * n2 + fi] = f[3];
        s->flx2[4 * n2 + fi] = f[4];
        s->e1x2[fi] = -f[5];
        s->e3x2[fi] = f[6];
        s->w2f[fi] = weight_for_ct(f[0], wl[IDN], wr[IDN], dx2f[j], dt);
      }
  /* x3: j in [js-1,je+1], i in [is-1,ie+1], faces k in [ks,ke+1] (:292-356) */
  for (int k = ks; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j)
      for (int i = is - 1; i <= ie + 1; ++i) {
        recon_cell(m, b, w, bcc, order, 2, k - 1, j, i, wl, tmp);
        recon_cell(m, b, w, bcc, order, 2, k, j, i, tmp, wr);
        long fi = F3IDX(m, k, j, i);
        double dvn = 0.0, dvt = 0.0;
        if (m->p.rsolver == 4) vel_diffs(m, w, 2, k, j, i, &dvn, &dvt);
        riemann(m, 2, wl, wr, b3[fi], dvn, dvt, f);
        /* flux slots: IDN, ivx=IVZ, ivy=IVX, ivz=IVY, IEN */
        s->flx3[0 * n3 + fi] = f[0];
        s->flx3[3 * n3 + fi] = f[1];
        s->flx3[1 * n3 + fi] = f[2];
        s->flx3[2 * n3 + fi] = f[3];
        s->flx3[4 * n3 + fi] = f[4];
        s->e2x3[fi] = -f[5];
        s->e1x3[fi] = f[6];
        s->w3f[fi] = weight_for_ct(f[0], wl[IDN], wr[IDN], dx3f[k], dt);
      }
}

/* ------------------------------------------------------------------------------------
 * Field::ComputeCornerE, calculate_corner_e.cpp:124-236 (3-D, Newtonian and SR branches)
 */
static void corner_e(orc_mesh *m, int b, scratch *s) {
  const double *w = m->w + (long)b * NHYDRO * m->ncell;
  const double *bcc = m->bcc + (long)b * 3 * m->ncell;
  int is = m->is, ie = m->ie, js = m->js, je = m->je, ks = m->ks, ke = m->ke;
  double *cce = s->cce;
  long nc = m->ncell;
  for (int k = ks - 1; k <= ke + 1; ++k)
    for (int j = js - 1; j <= je + 1; ++j)
      for (int i = is - 1; i <= ie + 1; ++i) {
        long c = CIDX(m, 0, k, j, i);
        if (m->p.relativistic) {
          /* SR branch, calculate_corner_e.cpp:161-172 */
          double u1 = w[c + 1 * nc], u2 = w[c + 2 * nc], u3 = w[c + 3 * nc];
          double u0 = sqrt(1.0 + SQR(u1) + SQR(u2) + SQR(u3));
          cce[c] = (u3 * bcc[c + 1 * nc] - u2 * bcc[c + 2 * nc]) / u0;
          cce[c + nc] = (u1 * bcc[c + 2 * nc] - u3 * bcc[c]) / u0;
          cce[c + 2 * nc] = (u2 * bcc[c] - u1 * bcc[c + 1 * nc]) / u0;
        } else {
          cce[c] = w[c + 3 * nc] * bcc[c + 1 * nc] - w[c + 2 * nc] * bcc[c + 2 * nc];
          cce[c + nc] = w[c + 1 * nc] * bcc[c + 2 * nc] - w[c + 3 * nc] * bcc[c];
          cce[c + 2 * nc] = w[c + 2 * nc] * bcc[c] - w[c + 1 * nc] * bcc[c + 1 * nc];
        }
      }
#define CC(n, k, j, i) cce[CIDX(m, n, k, j, i)]
#define W1F(k, j, i) s->w1f[F1IDX(m, k, j, i)]
#define W2F(k, j, i) s->w2f[F2IDX(m, k, j, i)]
#define W3F(k, j, i) s->w3f[F3IDX(m, k, j, i)]
#define E3X1(k, j, i) s->e3x1[F1IDX(m, k, j, i)]
#define E2X1(k, j, i) s->e2x1[F1IDX(m, k, j, i)]
#define E1X2(k, j, i) s->e1x2[F2IDX(m, k, j, i)]
#define E3X2(k, j, i) s->e3x2[F2IDX(m, k, j, i)]
#define E1X3(k, j, i) s->e1x3[F3IDX(m, k, j, i)]
#define E2X3(k, j, i) s->e2x3[F3IDX(m, k, j, i)]
  for (int k = ks; k <= ke + 1; ++k)
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie + 1; ++i) {
        double de1_l3 = (1.0 - W2F(k - 1, j, i)) * (E1X3(k, j, i) - CC(0, k - 1, j, i)) +
                        (W2F(k - 1, j, i)) * (E1X3(k, j - 1, i) - CC(0, k - 1, j - 1, i));
        double de1_r3 = (1.0 - W2F(k, j, i)) * (E1X3(k, j, i) - CC(0, k, j, i)) +
                        (W2F(k, j, i)) * (E1X3(k, j - 1, i) - CC(0, k, j - 1, i));
        double de1_l2 = (1.0 - W3F(k, j - 1, i)) * (E1X2(k, j, i) - CC(0, k, j - 1, i)) +
                        (W3F(k, j - 1, i)) * (E1X2(k - 1, j, i) - CC(0, k - 1, j - 1, i));
        double de1_r2 = (1.0 - W3F(k, j, i)) * (E1X2(k, j, i) - CC(0, k, j, i)) +
                        (W3F(k, j, i)) * (E1X2(k - 1, j, i) - CC(0, k - 1, j, i));
        if (i <= ie)
          m->e1[(long)b * m->ne1 + E1IDX(m, k, j, i)] =
              0.25 * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + E1X2(k - 1, j, i) + E1X2(k, j, i) +
                      E1X3(k, j - 1, i) + E1X3(k, j, i));

        double de2_l3 = (1.0 - W1F(k - 1, j, i)) * (E2X3(k, j, i) - CC(1, k - 1, j, i)) +
                        (W1F(k - 1, j, i)) * (E2X3(k, j, i - 1) - CC(1, k - 1, j, i - 1));
        double de2_r3 = (1.0 - W1F(k, j, i)) * (E2X3(k, j, i) - CC(1, k, j, i)) +
                        (W1F(k, j, i)) * (E2X3(k, j, i - 1) - CC(1, k, j, i - 1));
        double de2_l1 = (1.0 - W3F(k, j, i - 1)) * (E2X1(k, j, i) - CC(1, k, j, i - 1)) +
                        (W3F(k, j, i - 1)) * (E2X1(k - 1, j, i) - CC(1, k - 1, j, i - 1));
        double de2_r1 = (1.0 - W3F(k, j, i)) * (E2X1(k, j, i) - CC(1, k, j, i)) +
                        (W3F(k, j, i)) * (E2X1(k - 1, j, i) - CC(1, k - 1, j, i));
        if (j <= je)
          m->e2[(long)b * m->ne2 + E2IDX(m, k, j, i)] =
              0.25 * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + E2X3(k, j, i - 1) + E2X3(k, j, i) +
                      E2X1(k - 1, j, i) + E2X1(k, j, i));

        double de3_l2 = (1.0 - W1F(k, j - 1, i)) * (E3X2(k, j, i) - CC(2, k, j - 1, i)) +
                        (W1F(k, j - 1, i)) * (E3X2(k, j, i - 1) - CC(2, k, j - 1, i - 1));
        double de3_r2 = (1.0 - W1F(k, j, i)) * (E3X2(k, j, i) - CC(2, k, j, i)) +
                        (W1F(k, j, i)) * (E3X2(k, j, i - 1) - CC(2, k, j, i - 1));
        double de3_l1 = (1.0 - W2F(k, j, i - 1)) * (E3X1(k, j, i) - CC(2, k, j, i - 1)) +
                        (W2F(k, j, i - 1)) * (E3X1(k, j - 1, i) - CC(2, k, j - 1, i - 1));
        double de3_r1 = (1.0 - W2F(k, j, i)) * (E3X1(k, j, i) - CC(2, k, j, i)) +
                        (W2F(k, j, i)) * (E3X1(k, j - 1, i) - CC(2, k, j - 1, i));
        if (k <= ke)
          m->e3[(long)b * m->ne3 + E3IDX(m, k, j, i)] =
              0.25 * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + E3X2(k, j, i - 1) + E3X2(k, j, i) +
                      E3X1(k, j - 1, i) + E3X1(k, j, i));
      }
#undef CC
#undef W1F
#undef W2F
#undef W3F
#undef E3X1
#undef E2X1
#undef E1X2
#undef E3X2
#undef E1X3
#undef E2X3
}

/* ------------------------------------------------------------------------------------
 * Same-level EMF correction on block faces, FaceCenteredBoundaryVariable
 * (flux_correction_fc.cpp:51-260 pack, :689-940 add, :1355-1530 average).  Every edge on
 * a block face receives the pre-averaging values that the blocks sharing it computed,
 * added to its own in the order of the neighbour list (bvals_base.cpp:326-720: faces
 * x1-, x1+, x2-, x2+, x3-, x3+, then x1x2, x1x3, x2x3 edges), and is then scaled by 1/2
 * (edges inside a face) or 1/4 (edges shared by four blocks).  Periodic uniform mesh:
 * the neighbour in direction o holds the same edge at index - o*nx.
 */
static int nbr_block(const orc_mesh *m, int b, int o1, int o2, int o3) {
  int n[3] = {m->p.nbx1, m->p.nbx2, m->p.nbx3};
  int l[3] = {b % n[0], (b / n[0]) % n[1], b / (n[0] * n[1])};
  int o[3] = {o1, o2, o3};
  for (int a = 0; a < 3; ++a) {
    int t = l[a] + o[a];
    if (t < 0 || t >= n[a]) {  /* across a mesh face: periodic wrap, else no neighbour */
      if (m->p.bc[2 * a + (t < 0 ? 0 : 1)] != 0) return -1;
      t = (t + n[a]) % n[a];
    }
    l[a] = t;
  }
  return (l[2] * n[1] + l[1]) * n[0] + l[0];
}

/* is there a block (or a periodic image) across offset (o1, o2, o3) of block b? */
static int has_nbr(const orc_mesh *m, int b, int o1, int o2, int o3) {
  if (m->ml_nblev)
    return m->ml_nblev[(long)b * 27 + (o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)] != -1;
  return nbr_block(m, b, o1, o2, o3) >= 0;
}

/* corrected value of edge component c (0,1,2 = e1,e2,e3) at (k,j,i) of block b */
static double emf_corrected(const orc_mesh *m, int b, int c, int k, int j, int i) {
  const double *E = (c == 0) ? m->e1 : (c == 1) ? m->e2 : m->e3;
  long ne = (c == 0) ? m->ne1 : (c == 1) ? m->ne2 : m->ne3;
#define EV(bb, kk, jj, ii) \
  E[(long)(bb) * ne + ((c == 0) ? E1IDX(m, kk, jj, ii) : (c == 1) ? E2IDX(m, kk, jj, ii) \
                                                                    : E3IDX(m, kk, jj, ii))]
  int o[3] = {0, 0, 0};  /* position of the edge on the block faces, per axis */
  if (c != 0) o[0] = (i == m->is) ? -1 : (i == m->ie + 1) ? 1 : 0;
  if (c != 1) o[1] = (j == m->js) ? -1 : (j == m->je + 1) ? 1 : 0;
  if (c != 2) o[2] = (k == m->ks) ? -1 : (k == m->ke + 1) ? 1 : 0;
  int nx[3] = {m->p.nx1, m->p.nx2, m->p.nx3};
  int on = (o[0] != 0) + (o[1] != 0) + (o[2] != 0);
  double own = EV(b, k, j, i);
  if (on == 0) return own;
  /* the two transverse axes of this component, in neighbour-list order */
  int a0 = (c == 0) ? 1 : 0, a1 = (c == 2) ? 1 : 2;
  double sum = own;
  int axes[2] = {a0, a1};
  int count = 1; /* blocks of the same level sharing the edge (CountFineEdges) */
  for (int t = 0; t < 2; ++t) { /* face neighbours */
    int ax = axes[t];
    if (o[ax] == 0) continue;
    int d[3] = {0, 0, 0};
    d[ax] = o[ax];
    int nb = nbr_block(m, b, d[0], d[1], d[2]);
    if (nb < 0) continue; /* a physical boundary: nothing received */
    sum += EV(nb, k - d[2] * nx[2], j - d[1] * nx[1], i - d[0] * nx[0]);
    ++count;
  }
  if (on == 2) { /* edge neighbour; flux_correction_fc.cpp:1477-1481 divides by the count */
    int nb = nbr_block(m, b, o[0], o[1], o[2]);
    if (nb >= 0) {
      sum += EV(nb, k - o[2] * nx[2], j - o[1] * nx[1], i - o[0] * nx[0]);
      ++count;
    }
    if (count == 1) return own;
    return sum * (1.0 / (double)count);
  }
  /* face interior (flux_correction_fc.cpp:1362-1380): halved only if the face has a
   * neighbour */
  return count == 2 ? sum * 0.5 : own;
#undef EV
}

/* own edge EMFs with the block-face edges replaced by their corrected values */
static void corrected_edges(const orc_mesh *m, int b, scratch *s) {
  memcpy(s->e1, m->e1 + (long)b * m->ne1, sizeof(double) * m->ne1);
  memcpy(s->e2, m->e2 + (long)b * m->ne2, sizeof(double) * m->ne2);
  memcpy(s->e3, m->e3 + (long)b * m->ne3, sizeof(double) * m->ne3);
  int is = m->is, ie = m->ie, js = m->js, je = m->je, ks = m->ks, ke = m->ke;
  for (int k = ks; k <= ke + 1; ++k)
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie; ++i)
        if (j == js || j == je + 1 || k == ks || k == ke + 1)
          s->e1[E1IDX(m, k, j, i)] = emf_corrected(m, b, 0, k, j, i);
  for (int k = ks; k <= ke + 1; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie + 1; ++i)
        if (i == is || i == ie + 1 || k == ks || k == ke + 1)
          s->e2[E2IDX(m, k, j, i)] = emf_corrected(m, b, 1, k, j, i);
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie + 1; ++i)
        if (i == is || i == ie + 1 || j == js || j == je + 1)
          s->e3[E3IDX(m, k, j, i)] = emf_corrected(m, b, 2, k, j, i);
}

/* ------------------------------------------------------------------------------------
 * Hydro::AddFluxDivergence, add_flux_divergence.cpp:39-96 (Cartesian areas and volumes,
 * coordinates.cpp:448-548)
 */
static void add_flux_divergence(orc_mesh *m, int b, double wght, double *u, scratch *s) {
  const double *dx1f = m->dx1f + (long)b * m->nc1, *dx2f = m->dx2f + (long)b * m->nc2,
               *dx3f = m->dx3f + (long)b * m->nc3;
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1), n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1,
       n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  for (int k = m->ks; k <= m->ke; ++k)
    for (int j = m->js; j <= m->je; ++j)
      for (int i = m->is; i <= m->ie; ++i) {
        double x1area = dx2f[j] * dx3f[k];
        double x2area = dx1f[i] * dx3f[k];
        double x3area = dx1f[i] * dx2f[j];
        double vol = dx1f[i] * dx2f[j] * dx3f[k];
        for (int n = 0; n < NHYDRO; ++n) {
          double dflx = (x1area * s->flx1[n * n1 + F1IDX(m, k, j, i + 1)] -
                         x1area * s->flx1[n * n1 + F1IDX(m, k, j, i)]);
          dflx += (x2area * s->flx2[n * n2 + F2IDX(m, k, j + 1, i)] -
                   x2area * s->flx2[n * n2 + F2IDX(m, k, j, i)]);
          dflx += (x3area * s->flx3[n * n3 + F3IDX(m, k + 1, j, i)] -
                   x3area * s->flx3[n * n3 + F3IDX(m, k, j, i)]);
          u[CIDX(m, n, k, j, i)] -= wght * dflx / vol;
        }
      }
}

/* Field::CT, ct.cpp:31-116 (Cartesian edge lengths and areas) */
static void ct_update(orc_mesh *m, int b, double wght, double *b1, double *b2, double *b3,
                      scratch *s) {
  const double *dx1f = m->dx1f + (long)b * m->nc1, *dx2f = m->dx2f + (long)b * m->nc2,
               *dx3f = m->dx3f + (long)b * m->nc3;
  int is = m->is, ie = m->ie, js = m->js, je = m->je, ks = m->ks, ke = m->ke;
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie + 1; ++i) {
        double area = dx2f[j] * dx3f[k];
        double len = dx3f[k], len_p1 = dx3f[k];
        double *bf = &b1[F1IDX(m, k, j, i)];
        *bf -= (wght / area) * (len_p1 * s->e3[E3IDX(m, k, j + 1, i)] -
                                len * s->e3[E3IDX(m, k, j, i)]);
        len = dx2f[j]; len_p1 = dx2f[j];
        *bf += (wght / area) * (len_p1 * s->e2[E2IDX(m, k + 1, j, i)] -
                                len * s->e2[E2IDX(m, k, j, i)]);
      }
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie; ++i) {
        double area = dx1f[i] * dx3f[k];
        double len = dx3f[k], len_ip1 = dx3f[k];
        double *bf = &b2[F2IDX(m, k, j, i)];
        *bf += (wght / area) * (len_ip1 * s->e3[E3IDX(m, k, j, i + 1)] -
                                len * s->e3[E3IDX(m, k, j, i)]);
        len = dx1f[i];
        double len_p1 = dx1f[i];
        *bf -= (wght / area) * (len_p1 * s->e1[E1IDX(m, k + 1, j, i)] -
                                len * s->e1[E1IDX(m, k, j, i)]);
      }
  for (int k = ks; k <= ke + 1; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        double area = dx1f[i] * dx2f[j];
        double len = dx2f[j], len_ip1 = dx2f[j];
        double *bf = &b3[F3IDX(m, k, j, i)];
        *bf -= (wght / area) * (len_ip1 * s->e2[E2IDX(m, k, j, i + 1)] -
                                len * s->e2[E2IDX(m, k, j, i)]);
        len = dx1f[i];
        double len_p1 = dx1f[i];
        *bf += (wght / area) * (len_p1 * s->e1[E1IDX(m, k, j + 1, i)] -
                                len * s->e1[E1IDX(m, k, j, i)]);
      }
}

/* ------------------------------------------------------------------------------------
 * Field::CalculateCellCenteredField (field.cpp:112-180, uniform branch) and
 * EquationOfState::ConservedToPrimitive (adiabatic_mhd.cpp:41-90) over [kl,ku]x...
 */
static void cell_centered_field(orc_mesh *m, int b, int il, int iu, int jl, int ju, int kl,
                                int ku) {
  const double *b1 = m->b1 + (long)b * m->nf1, *b2 = m->b2 + (long)b * m->nf2,
               *b3 = m->b3 + (long)b * m->nf3;
  double *bcc = m->bcc + (long)b * 3 * m->ncell;
  for (int k = kl; k <= ku; ++k)
    for (int j = jl; j <= ju; ++j)
      for (int i = il; i <= iu; ++i) {
        double lw = 0.5, rw = 0.5;
        bcc[CIDX(m, 0, k, j, i)] = lw * b1[F1IDX(m, k, j, i)] + rw * b1[F1IDX(m, k, j, i + 1)];
        bcc[CIDX(m, 1, k, j, i)] = lw * b2[F2IDX(m, k, j, i)] + rw * b2[F2IDX(m, k, j + 1, i)];
        bcc[CIDX(m, 2, k, j, i)] = lw * b3[F3IDX(m, k, j, i)] + rw * b3[F3IDX(m, k + 1, j, i)];
      }
}

static long sr_c2p_block(orc_mesh *m, int b, double *u, double *prim, int il, int iu,
                         int jl, int ju, int kl, int ku);

static long con2prim_range(orc_mesh *m, int b, double *u, double *prim, int il, int iu,
                           int jl, int ju, int kl, int ku);

static long con2prim(orc_mesh *m, int b, double *u, double *prim) {
  /* the interior plus the ghost layers that have a neighbour (time_integrator.cpp:
   * 2206-2212, mesh.cpp:1820-1831); ghosts on physical boundaries come from the boundary
   * functions instead */
  int ng = m->p.ng;
  int il = m->is - (has_nbr(m, b, -1, 0, 0) ? ng : 0);
  int iu = m->ie + (has_nbr(m, b, 1, 0, 0) ? ng : 0);
  int jl = m->js - (has_nbr(m, b, 0, -1, 0) ? ng : 0);
  int ju = m->je + (has_nbr(m, b, 0, 1, 0) ? ng : 0);
  int kl = m->ks - (has_nbr(m, b, 0, 0, -1) ? ng : 0);
  int ku = m->ke + (has_nbr(m, b, 0, 0, 1) ? ng : 0);
  return con2prim_range(m, b, u, prim, il, iu, jl, ju, kl, ku);
}

/* EquationOfState::ConservedToPrimitive over [il,iu]x[jl,ju]x[kl,ku] of block b, with the
 * cell-centred field of the same range first */
static long con2prim_range(orc_mesh *m, int b, double *u, double *prim, int il, int iu,
                           int jl, int ju, int kl, int ku) {
  cell_centered_field(m, b, il, iu, jl, ju, kl, ku);
  if (m->p.relativistic) return sr_c2p_block(m, b, u, prim, il, iu, jl, ju, kl, ku);
  const double *bcc = m->bcc + (long)b * 3 * m->ncell;
  double gm1 = m->p.gamma - 1.0;
  double dfl = m->p.dfloor, pfl = m->p.pfloor;
  long nc = m->ncell;
  for (int k = kl; k <= ku; ++k)
    for (int j = jl; j <= ju; ++j)
      for (int i = il; i <= iu; ++i) {
        long c = CIDX(m, 0, k, j, i);
        double *u_d = &u[c], *u_e = &u[c + 4 * nc];
        double u_m1 = u[c + nc], u_m2 = u[c + 2 * nc], u_m3 = u[c + 3 * nc];
        *u_d = (*u_d > dfl) ? *u_d : dfl;
        prim[c] = *u_d;
        double di = 1.0 / *u_d;
        prim[c + nc] = u_m1 * di;
        prim[c + 2 * nc] = u_m2 * di;
        prim[c + 3 * nc] = u_m3 * di;
        double bcc1 = bcc[c], bcc2 = bcc[c + nc], bcc3 = bcc[c + 2 * nc];
        double pb = 0.5 * (SQR(bcc1) + SQR(bcc2) + SQR(bcc3));
        double e_k = 0.5 * di * (SQR(u_m1) + SQR(u_m2) + SQR(u_m3));
        double w_p = gm1 * (*u_e - e_k - pb);
        *u_e = (w_p > pfl) ? *u_e : ((pfl / gm1) + e_k + pb);
        prim[c + 4 * nc] = (w_p > pfl) ? w_p : pfl;
      }
  return 0;
}

/* ------------------------------------------------------------------------------------
 * SR-MHD conserved->primitive, eos/adiabatic_mhd_sr.cpp:72-272, with the Newman & Hamlin
 * (2014) fixed-point solve ConservedToPrimitiveNormal (:404-522).
 */
#define ORC_PI 3.1415926535897932 /* defs.hpp.in:140 */

/* ConservedToPrimitiveNormal, adiabatic_mhd_sr.cpp:404-522.  prim[5] receives
 * (rho, u1, u2, u3, pgas) in IDN, IVX..IVZ, IPR slots.  *iters = loop index at exit. */
static int sr_normal(double gamma_adi, double dd, double ee, double mm_sq, double mm1,
                     double mm2, double mm3, double bb_sq, double bb1, double bb2,
                     double bb3, double tt, double pgas_old, double *prim,
                     double *p_gamma_lor, double *p_pmag, int *iters) {
  const int max_iterations = 15;
  const double tol = 1.0e-12;
  const double pgas_uniform_min = 1.0e-12;
  const double a_min = 1.0e-12;
  const double v_sq_max = 1.0 - 1.0e-12;
  const double rr_max = 1.0 - 1.0e-12;
  double d = 0.5 * (mm_sq * bb_sq - SQR(tt));
  d = smax(d, 0.0);
  double pgas_min = cbrt(27.0 / 4.0 * d) - ee - 0.5 * bb_sq;
  pgas_min = smax(pgas_min, pgas_uniform_min);
  double pgas[3];
  pgas[0] = smax(pgas_old, pgas_min);
  int n;
  for (n = 0; n < max_iterations; ++n) {
    double a = 0.0;
    if (n % 3 != 2) {
      a = ee + pgas[n % 3] + 0.5 * bb_sq;
      a = smax(a, a_min);
    }
    if (n % 3 != 2) {
      double phi = acos(1.0 / a * sqrt(27.0 * d / (4.0 * a)));
      double eee = a / 3.0 - 2.0 / 3.0 * a * cos(2.0 / 3.0 * (phi + ORC_PI));
      double ll = eee - bb_sq;
      double v_sq = (mm_sq * SQR(ll) + SQR(tt) * (bb_sq + 2.0 * ll)) / SQR(ll * (bb_sq + ll));
      v_sq = smin(smax(v_sq, 0.0), v_sq_max);
      double gamma_sq = 1.0 / (1.0 - v_sq);
      double gamma = sqrt(gamma_sq);
      double wgas = ll / gamma_sq;
      double rho = dd / gamma;
      pgas[(n + 1) % 3] = (gamma_adi - 1.0) / gamma_adi * (wgas - rho);
      pgas[(n + 1) % 3] = smax(pgas[(n + 1) % 3], pgas_min);
    }
    if (n % 3 != 2) {
      if (pgas[(n + 1) % 3] > pgas_min && fabs(pgas[(n + 1) % 3] - pgas[n % 3]) < tol) break;
    }
    if (n % 3 == 2) {
      double rr = (pgas[2] - pgas[1]) / (pgas[1] - pgas[0]);
      if (!isfinite(rr) || fabs(rr) > rr_max) continue;
      pgas[0] = pgas[1] + (pgas[2] - pgas[1]) / (1.0 - rr);
      pgas[0] = smax(pgas[0], pgas_min);
      if (pgas[0] > pgas_min && fabs(pgas[0] - pgas[2]) < tol) break;
    }
  }
  *iters = n;
  if (n == max_iterations) return 0;
  prim[IPR] = pgas[(n + 1) % 3];
  if (!isfinite(prim[IPR])) return 0;
  double a = ee + prim[IPR] + 0.5 * bb_sq;
  a = smax(a, a_min);
  double phi = acos(1.0 / a * sqrt(27.0 * d / (4.0 * a)));
  double eee = a / 3.0 - 2.0 / 3.0 * a * cos(2.0 / 3.0 * (phi + ORC_PI));
  double ll = eee - bb_sq;
  double v_sq = (mm_sq * SQR(ll) + SQR(tt) * (bb_sq + 2.0 * ll)) / SQR(ll * (bb_sq + ll));
  v_sq = smin(smax(v_sq, 0.0), v_sq_max);
  double gamma_sq = 1.0 / (1.0 - v_sq);
  double gamma = sqrt(gamma_sq);
  prim[IDN] = dd / gamma;
  if (!isfinite(prim[IDN])) return 0;
  double ss = tt / ll;
  double v1 = (mm1 + ss * bb1) / (ll + bb_sq);
  double v2 = (mm2 + ss * bb2) / (ll + bb_sq);
  double v3 = (mm3 + ss * bb3) / (ll + bb_sq);
  prim[IVX] = gamma * v1;
  prim[IVY] = gamma * v2;
  prim[IVZ] = gamma * v3;
  if (!isfinite(prim[IVX]) || !isfinite(prim[IVY]) || !isfinite(prim[IVZ])) return 0;
  *p_gamma_lor = gamma;
  *p_pmag = 0.5 * (bb_sq / gamma_sq + SQR(ss));
  return 1;
}

/* one cell of EquationOfState::ConservedToPrimitive (SR), adiabatic_mhd_sr.cpp:87-268.
 * cons[5] (natural slots) may be rewritten; prim[5] holds the fallback/guess on entry and
 * the result on exit.  Returns 1 if the cell used the fallback. */
static int sr_c2p_cell(double gamma_adi, double dfloor, double pfloor, double sigma_max,
                       double beta_min, double gamma_max, double *cons, double bc1,
                       double bc2, double bc3, double *prim, int *iters) {
  const double mm_sq_ee_sq_max = 1.0 - 1.0e-12;
  double dd = cons[IDN], ee = cons[IPR];
  double mm_sq = SQR(cons[IVX]) + SQR(cons[IVY]) + SQR(cons[IVZ]);
  double mm1 = cons[IVX], mm2 = cons[IVY], mm3 = cons[IVZ];
  double bb_sq = SQR(bc1) + SQR(bc2) + SQR(bc3);
  double tt = cons[IVX] * bc1 + cons[IVY] * bc2 + cons[IVZ] * bc3;
  int fixed = 0;
  double density_floor_local = dfloor, pressure_floor_local = pfloor;
  double dd_min = density_floor_local;
  if (dd < dd_min) { dd = dd_min; fixed = 1; }
  double ee_min = density_floor_local + pressure_floor_local / (gamma_adi - 1.0) + 0.5 * bb_sq;
  if (ee < ee_min) { ee = ee_min; fixed = 1; }
  double mm_sq_max = mm_sq_ee_sq_max * SQR(ee);
  if (mm_sq > mm_sq_max) {
    double factor = sqrt(mm_sq_max / mm_sq);
    mm_sq = mm_sq_max;
    mm1 *= factor; mm2 *= factor; mm3 *= factor;
    tt *= factor;
    fixed = 1;
  }
  double rho_old = smax(prim[IDN], density_floor_local);
  double pgas_old = smax(prim[IPR], pressure_floor_local);
  double u1_old = prim[IVX], u2_old = prim[IVY], u3_old = prim[IVZ];
  double gamma = 0.0, pmag = 0.0;
  int success = sr_normal(gamma_adi, dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bc1, bc2, bc3, tt,
                          pgas_old, prim, &gamma, &pmag, iters);
  if (!success) {
    prim[IDN] = rho_old; prim[IPR] = pgas_old;
    prim[IVX] = u1_old; prim[IVY] = u2_old; prim[IVZ] = u3_old;
    fixed = 1;
  }
  if (sigma_max > 0.0) density_floor_local = smax(density_floor_local, 2.0 * pmag / sigma_max);
  if (beta_min > 0.0) pressure_floor_local = smax(pressure_floor_local, beta_min * pmag);
  double rho_add = smax(density_floor_local - prim[IDN], 0.0);
  double pgas_add = smax(pressure_floor_local - prim[IPR], 0.0);
  if (success && (rho_add > 0.0 || pgas_add > 0.0)) {
    double wgas_add = rho_add + gamma_adi / (gamma_adi - 1.0) * pgas_add;
    dd += rho_add * gamma;
    ee += wgas_add * SQR(gamma) + pgas_add;
    int it2;
    success = sr_normal(gamma_adi, dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bc1, bc2, bc3, tt,
                        pgas_old, prim, &gamma, &pmag, &it2);
    if (!success) {
      prim[IDN] = rho_old; prim[IPR] = pgas_old;
      prim[IVX] = u1_old; prim[IVY] = u2_old; prim[IVZ] = u3_old;
    }
    fixed = 1;
  }
  double *u1 = &prim[IVX], *u2 = &prim[IVY], *u3 = &prim[IVZ];
  if (!success) gamma = sqrt(1.0 + SQR(*u1) + SQR(*u2) + SQR(*u3));
  int velocity_ceiling = 0;
  if (gamma > gamma_max) {
    double factor = sqrt((SQR(gamma_max) - 1.0) / (SQR(gamma) - 1.0));
    *u1 *= factor; *u2 *= factor; *u3 *= factor;
    fixed = 1;
    velocity_ceiling = 1;
  }
  if (velocity_ceiling) {
    double b0 = *u1 * bc1 + *u2 * bc2 + *u3 * bc3;
    pmag = 0.5 * (bb_sq / SQR(gamma) + SQR(b0 / gamma));
  }
  density_floor_local = dfloor;
  if (sigma_max > 0.0) density_floor_local = smax(density_floor_local, 2.0 * pmag / sigma_max);
  pressure_floor_local = pfloor;
  if (beta_min > 0.0) pressure_floor_local = smax(pressure_floor_local, beta_min * pmag);
  double *rho = &prim[IDN], *pgas = &prim[IPR];
  if (*rho < density_floor_local) { *rho = density_floor_local; fixed = 1; }
  if (*pgas < pressure_floor_local) { *pgas = pressure_floor_local; fixed = 1; }
  if (!success) {
    *rho = density_floor_local;
    *pgas = pressure_floor_local;
    *u1 = *u2 = *u3 = 0.0;
  }
  if (fixed) {
    gamma = sqrt(1.0 + SQR(*u1) + SQR(*u2) + SQR(*u3));
    double b0 = bc1 * *u1 + bc2 * *u2 + bc3 * *u3;
    double b1 = (bc1 + b0 * *u1) / gamma;
    double b2 = (bc2 + b0 * *u2) / gamma;
    double b3 = (bc3 + b0 * *u3) / gamma;
    double b_sq = -SQR(b0) + SQR(b1) + SQR(b2) + SQR(b3);
    double wgas = *rho + gamma_adi / (gamma_adi - 1.0) * *pgas;
    double wtot = wgas + b_sq;
    pmag = 0.5 * b_sq;
    cons[IDN] = *rho * gamma;
    cons[IPR] = wtot * SQR(gamma) - SQR(b0) - (*pgas + pmag);
    cons[IVX] = wtot * gamma * *u1 - b0 * b1;
    cons[IVY] = wtot * gamma * *u2 - b0 * b2;
    cons[IVZ] = wtot * gamma * *u3 - b0 * b3;
  }
  return !success;
}

static long sr_c2p_block(orc_mesh *m, int b, double *u, double *prim, int il, int iu,
                         int jl, int ju, int kl, int ku) {
  const double *bcc = m->bcc + (long)b * 3 * m->ncell;
  long nc = m->ncell, fails = 0;
  for (int k = kl; k <= ku; ++k)
    for (int j = jl; j <= ju; ++j)
      for (int i = il; i <= iu; ++i) {
        long c = CIDX(m, 0, k, j, i);
        double cons[5], pr[5];
        for (int n = 0; n < 5; ++n) { cons[n] = u[c + n * nc]; pr[n] = prim[c + n * nc]; }
        int it;
        fails += sr_c2p_cell(m->p.gamma, m->p.dfloor, m->p.pfloor, m->p.sigma_max,
                             m->p.beta_min, m->p.gamma_max, cons, bcc[c], bcc[c + nc],
                             bcc[c + 2 * nc], pr, &it);
        for (int n = 0; n < 5; ++n) { u[c + n * nc] = cons[n]; prim[c + n * nc] = pr[n]; }
      }
  return fails;
}

void orc_sr_c2p_cells(long n, double gamma, double pgas_floor, const double *cons,
                      const double *bcc, const double *pgas_guess, double *prim,
                      int *iterations) {
  (void)pgas_floor;
#pragma omp parallel for schedule(static)
  for (long c = 0; c < n; ++c) {
    const double *q = cons + 5 * c, *bb = bcc + 3 * c;
    double mm_sq = SQR(q[IVX]) + SQR(q[IVY]) + SQR(q[IVZ]);
    double bb_sq = SQR(bb[0]) + SQR(bb[1]) + SQR(bb[2]);
    double tt = q[IVX] * bb[0] + q[IVY] * bb[1] + q[IVZ] * bb[2];
    double pr[5] = {0, 0, 0, 0, 0}, g, pm;
    int it;
    int ok = sr_normal(gamma, q[IDN], q[IPR], mm_sq, q[IVX], q[IVY], q[IVZ], bb_sq, bb[0],
                       bb[1], bb[2], tt, pgas_guess[c], pr, &g, &pm, &it);
    for (int v = 0; v < 5; ++v) prim[5 * c + v] = pr[v];
    iterations[c] = ok ? it : -1;
  }
}

/* SR prim -> cons, adiabatic_mhd_sr.cpp:284-332 (used by tests to build states) */
static void sr_p2c(double gamma_adi, const double *w, double bb1, double bb2, double bb3,
                   double *u) {
  double gamma_adi_red = gamma_adi / (gamma_adi - 1.0);
  double rho = w[IDN], pgas = w[IPR], u1 = w[IVX], u2 = w[IVY], u3 = w[IVZ];
  double u0 = sqrt(1.0 + SQR(u1) + SQR(u2) + SQR(u3));
  double b0 = bb1 * u1 + bb2 * u2 + bb3 * u3;
  double b1 = (bb1 + b0 * u1) / u0;
  double b2 = (bb2 + b0 * u2) / u0;
  double b3 = (bb3 + b0 * u3) / u0;
  double b_sq = -SQR(b0) + SQR(b1) + SQR(b2) + SQR(b3);
  double wtot_u02 = (rho + gamma_adi_red * pgas + b_sq) * u0 * u0;
  u[IDN] = rho * u0;
  u[IPR] = wtot_u02 - b0 * b0 - (pgas + 0.5 * b_sq);
  u[IVX] = wtot_u02 * u1 / u0 - b0 * b1;
  u[IVY] = wtot_u02 * u2 / u0 - b0 * b2;
  u[IVZ] = wtot_u02 * u3 / u0 - b0 * b3;
}

void orc_sr_prim_to_cons(long n, double gamma, const double *w, const double *bcc,
                         double *u) {
  for (long c = 0; c < n; ++c) sr_p2c(gamma, w + 5 * c, bcc[3 * c], bcc[3 * c + 1],
                                      bcc[3 * c + 2], u + 5 * c);
}

/* ------------------------------------------------------------------------------------
 * Hydro::NewBlockTimeStep, new_blockdt.cpp:45-230 (MHD branch :80-103)
 */
static double new_block_dt(orc_mesh *m, int b) {
  const double *w = m->w + (long)b * NHYDRO * m->ncell;
  const double *bcc = m->bcc + (long)b * 3 * m->ncell;
  const double *b1 = m->b1 + (long)b * m->nf1, *b2 = m->b2 + (long)b * m->nf2,
               *b3 = m->b3 + (long)b * m->nf3;
  const double *dx1f = m->dx1f + (long)b * m->nc1, *dx2f = m->dx2f + (long)b * m->nc2,
               *dx3f = m->dx3f + (long)b * m->nc3;
  long nc = m->ncell;
  double min_dt = DBL_MAX;
  const double cspeed = 0.0;
  for (int k = m->ks; k <= m->ke; ++k)
    for (int j = m->js; j <= m->je; ++j)
      for (int i = m->is; i <= m->ie; ++i) {
        double dt1 = dx1f[i], dt2 = dx2f[j], dt3 = dx3f[k];
        if (!m->p.relativistic) {
          long c = CIDX(m, 0, k, j, i);
          double wi[NWAVE];
          wi[IDN] = w[c]; wi[IVX] = w[c + nc]; wi[IVY] = w[c + 2 * nc];
          wi[IVZ] = w[c + 3 * nc]; wi[IPR] = w[c + 4 * nc];
          double bc1 = bcc[c], bc2 = bcc[c + nc], bc3 = bcc[c + 2 * nc];
          double bx = bc1 + fabs(b1[F1IDX(m, k, j, i)] - bc1);
          wi[IBY] = bc2; wi[IBZ] = bc3;
          double cf = fast_ms(m->p.gamma, wi, bx);
          double speed = smax(cspeed, (fabs(wi[IVX]) + cf));
          dt1 /= (speed);
          wi[IBY] = bc3; wi[IBZ] = bc1;
          bx = bc2 + fabs(b2[F2IDX(m, k, j, i)] - bc2);
          cf = fast_ms(m->p.gamma, wi, bx);
          speed = smax(cspeed, (fabs(wi[IVY]) + cf));
          dt2 /= (speed);
          wi[IBY] = bc1; wi[IBZ] = bc2;
          bx = bc3 + fabs(b3[F3IDX(m, k, j, i)] - bc3);
          cf = fast_ms(m->p.gamma, wi, bx);
          speed = smax(cspeed, (fabs(wi[IVZ]) + cf));
          dt3 /= (speed);
        }
        min_dt = smin(min_dt, dt1);
        min_dt = smin(min_dt, dt2);
        min_dt = smin(min_dt, dt3);
      }
  return min_dt * m->p.cfl_number;
}

/* Mesh::NewTimeStep, mesh.cpp:1236-1281 */
static void new_time_step(orc_mesh *m, const double *block_dt) {
  double dt = 2.0 * m->dt;
  for (int b = 0; b < m->nb; ++b) dt = smin(dt, block_dt[b]);
  if (m->time < m->p.tlim && (m->p.tlim - m->time) < dt) dt = m->p.tlim - m->time;
  m->dt = dt;
}

/* ------------------------------------------------------------------------------------
 * Same-level periodic ghost exchange: the value every ghost receives from its neighbour
 * (bvals_cc.cpp:287-430; face fields bvals_fc.cpp:344-397 and the matching set routine).
 * For face fields the block's own faces in the normal direction are [is, ie+1]; faces
 * outside that range come from the neighbour, as in LoadBoundaryBufferSameLevel.
 */
/* returns 1 when idx lies outside the block's own range and was mapped to the
 * neighbour (which is the block itself when the mesh has one block along the axis) */
static int locate(int own_lo, int own_hi, int n, int nb, int lx, int idx, int *nlx,
                  int *nidx, int bc_lo, int bc_hi) {
  if (idx < own_lo) {
    if (lx == 0 && bc_lo != 0) return -1;  /* physical boundary: no neighbour */
    *nlx = (lx - 1 + nb) % nb; *nidx = idx + n; return 1;
  }
  if (idx > own_hi) {
    if (lx == nb - 1 && bc_hi != 0) return -1;
    *nlx = (lx + 1) % nb; *nidx = idx - n; return 1;
  }
  *nlx = lx; *nidx = idx;
  return 0;
}

/* combine per-axis locate() results: -1 if any axis has no neighbour, else 1 if moved */
static int loc_or(int a, int b) { return (a < 0 || b < 0) ? -1 : (a | b); }

static void exchange(orc_mesh *m, double *cc, int nvar, double *f1, double *f2, double *f3) {
  int nbx1 = m->p.nbx1, nbx2 = m->p.nbx2, nbx3 = m->p.nbx3;
  int nx1 = m->p.nx1, nx2 = m->p.nx2, nx3 = m->p.nx3;
  const int *bc = m->p.bc;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < m->nb; ++b) {
    int lx1 = b % nbx1, lx2 = (b / nbx1) % nbx2, lx3 = b / (nbx1 * nbx2);
    for (int k = 0; k < m->nc3; ++k)
      for (int j = 0; j < m->nc2; ++j)
        for (int i = 0; i < m->nc1 + 1; ++i) {
          int a1, a2, a3, si, sj, sk;
          int mv = locate(m->ks, m->ke, nx3, nbx3, lx3, k, &a3, &sk, bc[4], bc[5]);
          mv = loc_or(mv, locate(m->js, m->je, nx2, nbx2, lx2, j, &a2, &sj, bc[2], bc[3]));
          int sb;
          if (cc && i < m->nc1) {
            int r = loc_or(mv, locate(m->is, m->ie, nx1, nbx1, lx1, i, &a1, &si, bc[0],
                                      bc[1]));
            if (r > 0) {
              sb = (a3 * nbx2 + a2) * nbx1 + a1;
              for (int n = 0; n < nvar; ++n)
                cc[(long)b * nvar * m->ncell + CIDX(m, n, k, j, i)] =
                    cc[(long)sb * nvar * m->ncell + CIDX(m, n, sk, sj, si)];
            }
          }
          if (f1) {
            int r = loc_or(mv, locate(m->is, m->ie + 1, nx1, nbx1, lx1, i, &a1, &si, bc[0],
                                      bc[1]));
            if (r > 0) {
              sb = (a3 * nbx2 + a2) * nbx1 + a1;
              f1[(long)b * m->nf1 + F1IDX(m, k, j, i)] =
                  f1[(long)sb * m->nf1 + F1IDX(m, sk, sj, si)];
            }
          }
        }
    if (f2)
      for (int k = 0; k < m->nc3; ++k)
        for (int j = 0; j < m->nc2 + 1; ++j)
          for (int i = 0; i < m->nc1; ++i) {
            int a1, a2, a3, si, sj, sk;
            int mv = locate(m->ks, m->ke, nx3, nbx3, lx3, k, &a3, &sk, bc[4], bc[5]);
            mv = loc_or(mv, locate(m->js, m->je + 1, nx2, nbx2, lx2, j, &a2, &sj, bc[2],
                                   bc[3]));
            mv = loc_or(mv, locate(m->is, m->ie, nx1, nbx1, lx1, i, &a1, &si, bc[0], bc[1]));
            if (mv > 0) {
              int sb = (a3 * nbx2 + a2) * nbx1 + a1;
              f2[(long)b * m->nf2 + F2IDX(m, k, j, i)] =
                  f2[(long)sb * m->nf2 + F2IDX(m, sk, sj, si)];
            }
          }
    if (f3)
      for (int k = 0; k < m->nc3 + 1; ++k)
        for (int j = 0; j < m->nc2; ++j)
          for (int i = 0; i < m->nc1; ++i) {
            int a1, a2, a3, si, sj, sk;
            int mv = locate(m->ks, m->ke + 1, nx3, nbx3, lx3, k, &a3, &sk, bc[4], bc[5]);
            mv = loc_or(mv, locate(m->js, m->je, nx2, nbx2, lx2, j, &a2, &sj, bc[2], bc[3]));
            mv = loc_or(mv, locate(m->is, m->ie, nx1, nbx1, lx1, i, &a1, &si, bc[0], bc[1]));
            if (mv > 0) {
              int sb = (a3 * nbx2 + a2) * nbx1 + a1;
              f3[(long)b * m->nf3 + F3IDX(m, k, j, i)] =
                  f3[(long)sb * m->nf3 + F3IDX(m, sk, sj, si)];
            }
          }
  }
}

/* ------------------------------------------------------------------------------------
 * mesh life cycle
 */
orc_mesh *orc_create(const orc_params *p, const double *x1f, const double *dx1f,
                     const double *x2f, const double *dx2f, const double *x3f,
                     const double *dx3f) {
  orc_mesh *m = calloc(1, sizeof(orc_mesh));
  m->p = *p;
  m->nb = p->nbx1 * p->nbx2 * p->nbx3;
  m->nc1 = p->nx1 + 2 * p->ng; m->nc2 = p->nx2 + 2 * p->ng; m->nc3 = p->nx3 + 2 * p->ng;
  m->is = p->ng; m->ie = p->ng + p->nx1 - 1;
  m->js = p->ng; m->je = p->ng + p->nx2 - 1;
  m->ks = p->ng; m->ke = p->ng + p->nx3 - 1;
  m->ncell = (long)m->nc1 * m->nc2 * m->nc3;
  m->nf1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1);
  m->nf2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1;
  m->nf3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  m->ne1 = (long)(m->nc3 + 1) * (m->nc2 + 1) * m->nc1;
  m->ne2 = (long)(m->nc3 + 1) * m->nc2 * (m->nc1 + 1);
  m->ne3 = (long)m->nc3 * (m->nc2 + 1) * (m->nc1 + 1);
  long nb = m->nb;
  m->e1 = calloc(nb * m->ne1, sizeof(double));
  m->e2 = calloc(nb * m->ne2, sizeof(double));
  m->e3 = calloc(nb * m->ne3, sizeof(double));
  m->u = calloc(nb * NHYDRO * m->ncell, sizeof(double));
  m->u1 = calloc(nb * NHYDRO * m->ncell, sizeof(double));
  m->w = calloc(nb * NHYDRO * m->ncell, sizeof(double));
  m->w1 = calloc(nb * NHYDRO * m->ncell, sizeof(double));
  m->bcc = calloc(nb * 3 * m->ncell, sizeof(double));
  m->b1 = calloc(nb * m->nf1, sizeof(double));
  m->b2 = calloc(nb * m->nf2, sizeof(double));
  m->b3 = calloc(nb * m->nf3, sizeof(double));
  m->bb1 = calloc(nb * m->nf1, sizeof(double));
  m->bb2 = calloc(nb * m->nf2, sizeof(double));
  m->bb3 = calloc(nb * m->nf3, sizeof(double));
  m->x1f = malloc(sizeof(double) * nb * (m->nc1 + 1));
  m->x2f = malloc(sizeof(double) * nb * (m->nc2 + 1));
  m->x3f = malloc(sizeof(double) * nb * (m->nc3 + 1));
  m->dx1f = malloc(sizeof(double) * nb * m->nc1);
  m->dx2f = malloc(sizeof(double) * nb * m->nc2);
  m->dx3f = malloc(sizeof(double) * nb * m->nc3);
  m->x1v = malloc(sizeof(double) * nb * m->nc1);
  m->x2v = malloc(sizeof(double) * nb * m->nc2);
  m->x3v = malloc(sizeof(double) * nb * m->nc3);
  memcpy(m->x1f, x1f, sizeof(double) * nb * (m->nc1 + 1));
  memcpy(m->x2f, x2f, sizeof(double) * nb * (m->nc2 + 1));
  memcpy(m->x3f, x3f, sizeof(double) * nb * (m->nc3 + 1));
  memcpy(m->dx1f, dx1f, sizeof(double) * nb * m->nc1);
  memcpy(m->dx2f, dx2f, sizeof(double) * nb * m->nc2);
  memcpy(m->dx3f, dx3f, sizeof(double) * nb * m->nc3);
  /* x?v = 0.5*(x?f(i+1) + x?f(i)), cartesian.cpp:28-32 */
  for (long b = 0; b < nb; ++b) {
    for (int i = 0; i < m->nc1; ++i)
      m->x1v[b * m->nc1 + i] = 0.5 * (m->x1f[b * (m->nc1 + 1) + i + 1] +
                                      m->x1f[b * (m->nc1 + 1) + i]);
    for (int j = 0; j < m->nc2; ++j)
      m->x2v[b * m->nc2 + j] = 0.5 * (m->x2f[b * (m->nc2 + 1) + j + 1] +
                                      m->x2f[b * (m->nc2 + 1) + j]);
    for (int k = 0; k < m->nc3; ++k)
      m->x3v[b * m->nc3 + k] = 0.5 * (m->x3f[b * (m->nc3 + 1) + k + 1] +
                                      m->x3f[b * (m->nc3 + 1) + k]);
  }
  m->dt = DBL_MAX;  /* mesh.cpp:100 */
  m->time = 0.0;
  return m;
}

void orc_destroy(orc_mesh *m) {
  if (!m) return;
  ml_free(m->ml, m->nb);
  free(m->u); free(m->u1); free(m->w); free(m->w1); free(m->bcc); free(m->b1);
  free(m->b2); free(m->b3); free(m->bb1); free(m->bb2); free(m->bb3); free(m->x1f);
  free(m->x2f); free(m->x3f); free(m->dx1f); free(m->dx2f); free(m->dx3f);
  free(m->x1v); free(m->x2v); free(m->x3v); free(m->e1); free(m->e2); free(m->e3);
  free(m);
}

int orc_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

void orc_set_state(orc_mesh *m, const double *u, const double *b1, const double *b2,
                   const double *b3) {
  memcpy(m->u, u, sizeof(double) * m->nb * NHYDRO * m->ncell);
  memcpy(m->b1, b1, sizeof(double) * m->nb * m->nf1);
  memcpy(m->b2, b2, sizeof(double) * m->nb * m->nf2);
  memcpy(m->b3, b3, sizeof(double) * m->nb * m->nf3);
}

void orc_set_prim(orc_mesh *m, const double *w) {
  memcpy(m->w, w, sizeof(double) * m->nb * NHYDRO * m->ncell);
  memcpy(m->w1, w, sizeof(double) * m->nb * NHYDRO * m->ncell);
}

void orc_get_state(const orc_mesh *m, double *u, double *b1, double *b2, double *b3) {
  if (u) memcpy(u, m->u, sizeof(double) * m->nb * NHYDRO * m->ncell);
  if (b1) memcpy(b1, m->b1, sizeof(double) * m->nb * m->nf1);
  if (b2) memcpy(b2, m->b2, sizeof(double) * m->nb * m->nf2);
  if (b3) memcpy(b3, m->b3, sizeof(double) * m->nb * m->nf3);
}

void orc_get_prim(const orc_mesh *m, double *w, double *bcc) {
  if (w) memcpy(w, m->w, sizeof(double) * m->nb * NHYDRO * m->ncell);
  if (bcc) memcpy(bcc, m->bcc, sizeof(double) * m->nb * 3 * m->ncell);
}

double orc_get_dt(const orc_mesh *m) { return m->dt; }
double orc_get_time(const orc_mesh *m) { return m->time; }
void orc_set_dt(orc_mesh *m, double dt) { m->dt = dt; }
long orc_c2p_failures(const orc_mesh *m) { return m->c2p_fail; }

/* ------------------------------------------------------------------------------------
 * BoundaryValues::ApplyPhysicalBoundaries (bvals/bvals.cpp:453-680) on the primitives
 * and the face field of block b: for each mesh face of the block that is a physical
 * boundary, in the order inner/outer x1, x2, x3, the outflow or reflecting function of
 * the hydro primitives (bvals/cc/outflow_cc.cpp, bvals/cc/hydro/reflect_hydro.cpp) and of
 * the face field (bvals/fc/outflow_fc.cpp, bvals/fc/reflect_fc.cpp), then the
 * cell-centred field of the ghost cells it filled (bvals.cpp:516-520).  The conserved
 * state of those ghost cells (bvals.cpp:521-522) is not formed: nothing on the path
 * reads it.
 */
/* EquationOfState::PrimitiveToConserved, Newtonian MHD (adiabatic_mhd.cpp:99-133), over
 * a cell range of block b (from w and the cell-centred field) */
static void p2c_range(orc_mesh *m, int b, const double *w, int i0, int i1, int j0, int j1,
                      int k0, int k1) {
  double igm1 = 1.0 / (m->p.gamma - 1.0);
  double *ub = m->u + (long)b * NHYDRO * m->ncell;
  const double *wb = w + (long)b * NHYDRO * m->ncell;
  const double *bc = m->bcc + (long)b * 3 * m->ncell;
  long nc = m->ncell;
  for (int k = k0; k <= k1; ++k)
    for (int j = j0; j <= j1; ++j)
      for (int i = i0; i <= i1; ++i) {
        long q = CIDX(m, 0, k, j, i);
        double w_d = wb[q], w_vx = wb[q + nc], w_vy = wb[q + 2 * nc], w_vz = wb[q + 3 * nc],
               w_p = wb[q + 4 * nc];
        double bcc1 = bc[q], bcc2 = bc[q + nc], bcc3 = bc[q + 2 * nc];
        ub[q] = w_d;
        ub[q + nc] = w_vx * w_d;
        ub[q + 2 * nc] = w_vy * w_d;
        ub[q + 3 * nc] = w_vz * w_d;
        ub[q + 4 * nc] = w_p * igm1 + 0.5 * (w_d * (SQR(w_vx) + SQR(w_vy) + SQR(w_vz)) +
                                             (SQR(bcc1) + SQR(bcc2) + SQR(bcc3)));
      }
}

static void apply_bcs(orc_mesh *m, int b, double *w) {
  int ng = m->p.ng;
  int lo[3] = {m->is, m->js, m->ks}, hi[3] = {m->ie, m->je, m->ke};
  int has[6];  /* neighbour (block or periodic) across each block face */
  for (int f = 0; f < 6; ++f) {
    int o[3] = {0, 0, 0};
    o[f / 2] = (f & 1) ? 1 : -1;
    has[f] = has_nbr(m, b, o[0], o[1], o[2]);
  }
  double *wb = w + (long)b * NHYDRO * m->ncell;
  double *fb[3] = {m->b1 + (long)b * m->nf1, m->b2 + (long)b * m->nf2,
                   m->b3 + (long)b * m->nf3};
  long nc = m->ncell;
  for (int a = 0; a < 3; ++a) {
    /* transverse ranges: x1 uses the extended j/k ranges only where those faces are not
     * physical; x2 the full i range; x3 the full i and j ranges (bvals.cpp:457-470,596) */
    int rl[3], rh[3];
    for (int d = 0; d < 3; ++d) { rl[d] = lo[d]; rh[d] = hi[d]; }
    if (a == 0) {
      if (has[2]) rl[1] -= ng;
      if (has[3]) rh[1] += ng;
      if (has[4]) rl[2] -= ng;
      if (has[5]) rh[2] += ng;
    } else if (a == 1) {
      rl[0] -= ng; rh[0] += ng;
      if (has[4]) rl[2] -= ng;
      if (has[5]) rh[2] += ng;
    } else {
      rl[0] -= ng; rh[0] += ng;
      rl[1] -= ng; rh[1] += ng;
    }
    for (int side = 0; side < 2; ++side) {
      int f = 2 * a + side;
      if (has[f]) continue;
      int kind = m->p.bc[f];  /* 1 outflow, 2 reflecting */
      /* primitives */
      for (int g = 1; g <= ng; ++g) {
        int dst = side ? hi[a] + g : lo[a] - g;
        int src = (kind == 1) ? (side ? hi[a] : lo[a]) : (side ? hi[a] - g + 1 : lo[a] + g - 1);
        int r0[3], r1[3];
        for (int d = 0; d < 3; ++d) { r0[d] = rl[d]; r1[d] = rh[d]; }
        r0[a] = r1[a] = dst;
        for (int n = 0; n < NHYDRO; ++n) {
          double sg = (kind == 2 && n == IVX + a) ? -1.0 : 1.0;
          for (int k = r0[2]; k <= r1[2]; ++k)
            for (int j = r0[1]; j <= r1[1]; ++j)
              for (int i = r0[0]; i <= r1[0]; ++i) {
                int s3[3] = {i, j, k};
                s3[a] = src;
                double v = wb[CIDX(m, n, s3[2], s3[1], s3[0])];
                wb[CIDX(m, n, k, j, i)] = (sg < 0.0) ? -v : v;
              }
        }
      }
      /* face field */
      for (int d = 0; d < 3; ++d) {
        double *F = fb[d];
        for (int g = 1; g <= ng; ++g) {
          int dst, src;
          double sg = 1.0;
          if (d == a) { /* the normal component */
            dst = side ? hi[a] + 1 + g : lo[a] - g;
            src = (kind == 1) ? (side ? hi[a] + 1 : lo[a]) : (side ? hi[a] + 1 - g : lo[a] + g);
            if (kind == 2) sg = -1.0;
          } else {
            dst = side ? hi[a] + g : lo[a] - g;
            src = (kind == 1) ? (side ? hi[a] : lo[a]) : (side ? hi[a] - g + 1 : lo[a] + g - 1);
          }
          int r0[3], r1[3];
          for (int e = 0; e < 3; ++e) { r0[e] = rl[e]; r1[e] = rh[e]; }
          r1[d] += (d != a) ? 1 : 0;  /* the face count along its own direction */
          r0[a] = r1[a] = dst;
          for (int k = r0[2]; k <= r1[2]; ++k)
            for (int j = r0[1]; j <= r1[1]; ++j)
              for (int i = r0[0]; i <= r1[0]; ++i) {
                int s3[3] = {i, j, k};
                s3[a] = src;
                long di = (d == 0) ? F1IDX(m, k, j, i) : (d == 1) ? F2IDX(m, k, j, i)
                                                                   : F3IDX(m, k, j, i);
                long si = (d == 0) ? F1IDX(m, s3[2], s3[1], s3[0])
                        : (d == 1) ? F2IDX(m, s3[2], s3[1], s3[0])
                                   : F3IDX(m, s3[2], s3[1], s3[0]);
                double v = F[si];
                F[di] = (sg < 0.0) ? -v : v;
              }
        }
      }
      /* cell-centred field of the filled ghost cells */
      int c0[3], c1[3];
      for (int d = 0; d < 3; ++d) { c0[d] = rl[d]; c1[d] = rh[d]; }
      c0[a] = side ? hi[a] + 1 : lo[a] - ng;
      c1[a] = side ? hi[a] + ng : lo[a] - 1;
      cell_centered_field(m, b, c0[0], c1[0], c0[1], c1[1], c0[2], c1[2]);
      /* the conserved state of those ghost cells (bvals.cpp:514-515); the relativistic
       * path reads no ghost U and does not form it */
      if (!m->p.relativistic) p2c_range(m, b, w, c0[0], c1[0], c0[1], c1[1], c0[2], c1[2]);
    }
  }
  (void)nc;
}

static int any_physical(const orc_mesh *m) {
  for (int f = 0; f < 6; ++f)
    if (m->p.bc[f] != 0) return 1;
  return 0;
}

static void all_bcs(orc_mesh *m, double *w) {
  if (!any_physical(m)) return;
#pragma omp parallel for schedule(static)
  for (int b = 0; b < m->nb; ++b) apply_bcs(m, b, w);
}

static void all_con2prim(orc_mesh *m, double *wout) {
  long fails = 0;
#pragma omp parallel for schedule(static) reduction(+ : fails)
  for (int b = 0; b < m->nb; ++b)
    fails += con2prim(m, b, m->u + (long)b * NHYDRO * m->ncell,
                      wout + (long)b * NHYDRO * m->ncell);
  m->c2p_fail = fails;
}

static void all_new_dt(orc_mesh *m) {
  double *bdt = malloc(sizeof(double) * m->nb);
#pragma omp parallel for schedule(static)
  for (int b = 0; b < m->nb; ++b) bdt[b] = new_block_dt(m, b);
  new_time_step(m, bdt);
  free(bdt);
}

void orc_initialize(orc_mesh *m) {
  if (m->ml) { ml_initialize(m); return; }
  /* Mesh::Initialize: boundaries (mesh.cpp:1698-1725), W(U) into w over the whole block
   * (mesh.cpp:1833), NewBlockTimeStep + NewTimeStep (mesh.cpp:1959-1964) */
  exchange(m, m->u, NHYDRO, m->b1, m->b2, m->b3);
  all_con2prim(m, m->w);
  all_bcs(m, m->w);  /* mesh.cpp:1886 */
  all_new_dt(m);
}

#define SWAP(a, b) do { double *t_ = (a); (a) = (b); (b) = t_; } while (0)

static stage_w stage_weights(const orc_mesh *m, int stage) {
  stage_w w;
  w.g1 = 0.0; w.g2 = 1.0; w.swap = 1;
  w.order = m->p.xorder;
  if (m->integ == ORC_RK1) {           /* one stage */
    w.beta = 1.0; w.delta = 1.0;
  } else if (m->integ == ORC_RK2) {    /* :338-465: Heun / SSPRK(2,2) */
    if (stage == 1) { w.beta = 1.0; w.delta = 1.0; }
    else { w.beta = 0.5; w.delta = 0.0; w.g1 = 0.5; w.g2 = 0.5; w.swap = 0; }
  } else {                             /* vl2, :111-236 */
    w.beta = (stage == 1) ? 0.5 : 1.0;
    w.delta = (stage == 1) ? 1.0 : 0.0;
    if (stage == 1) w.order = 1;
  }
  return w;
}

/* WeightedAve(u1, u, ..., {1, delta, 0, 0, 0}) then, unless the registers swap,
 * WeightedAve(u, u1, ..., {g1, g2, 0, 0, 0}) (weighted_ave.cpp:35-230) over the interior
 * of one block; returns the register IntegrateHydro then updates (the pointer swap itself
 * happens after all blocks, so with a swap that register is u1). */
static double *hydro_registers(orc_mesh *m, const stage_w *sw, double *u, double *u1) {
  if (sw->delta != 0.0)
    for (int n = 0; n < NHYDRO; ++n)
      for (int k = m->ks; k <= m->ke; ++k)
        for (int j = m->js; j <= m->je; ++j)
          for (int i = m->is; i <= m->ie; ++i)
            u1[CIDX(m, n, k, j, i)] += sw->delta * u[CIDX(m, n, k, j, i)];
  if (sw->swap) return u1;
  for (int n = 0; n < NHYDRO; ++n)
    for (int k = m->ks; k <= m->ke; ++k)
      for (int j = m->js; j <= m->je; ++j)
        for (int i = m->is; i <= m->ie; ++i)
          u[CIDX(m, n, k, j, i)] = sw->g1 * u[CIDX(m, n, k, j, i)] +
                                   sw->g2 * u1[CIDX(m, n, k, j, i)];
  return u;
}

/* the same for the face field of one block (weighted_ave.cpp:360-560: x1 faces
 * [is, ie+1], x2 faces [js, je+1], x3 faces [ks, ke+1]); f = b1 registers, g = b */
static void field_registers(orc_mesh *m, const stage_w *sw, double *const f[3],
                            double *const g[3]) {
  int iu[3] = {1, 0, 0}, ju[3] = {0, 1, 0}, ku[3] = {0, 0, 1};
  for (int d = 0; d < 3; ++d)
    for (int k = m->ks; k <= m->ke + ku[d]; ++k)
      for (int j = m->js; j <= m->je + ju[d]; ++j)
        for (int i = m->is; i <= m->ie + iu[d]; ++i) {
          const long o = d == 0 ? F1IDX(m, k, j, i) : d == 1 ? F2IDX(m, k, j, i)
                                                             : F3IDX(m, k, j, i);
          if (sw->delta != 0.0) f[d][o] += sw->delta * g[d][o];
          if (!sw->swap) g[d][o] = sw->g1 * g[d][o] + sw->g2 * f[d][o];
        }
}

/* one stage of TimeIntegratorTaskList for MHD (time_integrator.cpp:1606-2318):
 * StartupTaskList zeroing, CalculateHydroFlux (DC on the first vl2 stage),
 * CalculateEMF, EMF averaging, IntegrateHydro/IntegrateField with the register
 * averages, ghost exchange, Primitives (W(U) into w1 then swap), NewBlockTimeStep on the
 * last stage. */
void orc_stage(orc_mesh *m, int stage) {
  if (m->ml) { ml_stage(m, stage); return; }
  const stage_w sw = stage_weights(m, stage);
  long nb = m->nb;
  if (stage == 1) { /* StartupTaskList, :1606-1625 */
    memset(m->u1, 0, sizeof(double) * nb * NHYDRO * m->ncell);
    memset(m->bb1, 0, sizeof(double) * nb * m->nf1);
    memset(m->bb2, 0, sizeof(double) * nb * m->nf2);
    memset(m->bb3, 0, sizeof(double) * nb * m->nf3);
  }
#pragma omp parallel
  {
    scratch s;
    scratch_alloc(m, &s);
    /* phase A: fluxes, corner EMFs, hydro register average + flux divergence */
#pragma omp for schedule(dynamic, 1)
    for (int b = 0; b < m->nb; ++b) {
      calculate_fluxes(m, b, sw.order, &s);
      corner_e(m, b, &s);
      double *u = m->u + (long)b * NHYDRO * m->ncell;
      double *u1 = m->u1 + (long)b * NHYDRO * m->ncell;
      add_flux_divergence(m, b, sw.beta * m->dt, hydro_registers(m, &sw, u, u1), &s);
    }
    /* phase B: EMF correction (needs every block's edges), field registers + CT */
#pragma omp for schedule(dynamic, 1)
    for (int b = 0; b < m->nb; ++b) {
      double *const f[3] = {m->bb1 + b * m->nf1, m->bb2 + b * m->nf2, m->bb3 + b * m->nf3};
      double *const g[3] = {m->b1 + b * m->nf1, m->b2 + b * m->nf2, m->b3 + b * m->nf3};
      field_registers(m, &sw, f, g);
      corrected_edges(m, b, &s);
      double *const *t = sw.swap ? f : g;
      ct_update(m, b, sw.beta * m->dt, t[0], t[1], t[2], &s);
    }
    scratch_free(&s);
  }
  if (sw.swap) {
    SWAP(m->u, m->u1);
    SWAP(m->b1, m->bb1);
    SWAP(m->b2, m->bb2);
    SWAP(m->b3, m->bb3);
  }
  exchange(m, m->u, NHYDRO, m->b1, m->b2, m->b3);
  all_con2prim(m, m->w1);  /* ConservedToPrimitive(u, w, b, w1, ...) (:2221-2223) */
  SWAP(m->w, m->w1);       /* :2269 */
  all_bcs(m, m->w);        /* PhysicalBoundary task, :2278-2299 */
}

/* the stages of one cycle and time += dt (main.cpp:535), without the new time step */
void orc_advance(orc_mesh *m) {
  orc_stage(m, 1);
  if (m->integ != ORC_RK1) orc_stage(m, 2);
  m->time += m->dt;
}

/* NewBlockTimeStep of every block (last stage) + Mesh::NewTimeStep */
void orc_new_dt(orc_mesh *m) { all_new_dt(m); }

void orc_set_time(orc_mesh *m, double t) { m->time = t; }

void orc_cycle(orc_mesh *m) {
  orc_advance(m);
  all_new_dt(m);
}

/* ------------------------------------------------------------------------------------
 * Per-operator restatements on block b of the oracle's mesh (checkers of the library's
 * per-operator entry points): each runs one member function of the reference on the
 * mesh's own arrays (w, bcc, b, u) and copies its outputs.  Test infrastructure only.
 */

/* Hydro::CalculateFluxes (calculate_fluxes.cpp:38-415) with dt for the CT weights:
 * flx? [5][face] and emf[9] = e3_x1f, e2_x1f, wght.x1f, e1_x2f, e3_x2f, wght.x2f, e1_x3f,
 * e2_x3f, wght.x3f */
void orc_op_fluxes(orc_mesh *m, int b, int order, double dt, double *flx1, double *flx2,
                   double *flx3, double *const emf[9]) {
  scratch s;
  scratch_alloc(m, &s);
  double dt_keep = m->dt;
  m->dt = dt;
  calculate_fluxes(m, b, order, &s);
  m->dt = dt_keep;
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1), n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1,
       n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  memcpy(flx1, s.flx1, sizeof(double) * NHYDRO * n1);
  memcpy(flx2, s.flx2, sizeof(double) * NHYDRO * n2);
  memcpy(flx3, s.flx3, sizeof(double) * NHYDRO * n3);
  const double *src[9] = {s.e3x1, s.e2x1, s.w1f, s.e1x2, s.e3x2, s.w2f, s.e1x3, s.e2x3, s.w3f};
  const long len[9] = {n1, n1, n1, n2, n2, n2, n3, n3, n3};
  for (int q = 0; q < 9; ++q) memcpy(emf[q], src[q], sizeof(double) * len[q]);
  scratch_free(&s);
}

/* Field::ComputeCornerE (calculate_corner_e.cpp:28-236) from the face EMFs emf[9] (as
 * orc_op_fluxes gives them) and the mesh's w, bcc: the edge EMFs before any averaging */
void orc_op_corner_e(orc_mesh *m, int b, const double *const emf[9], double *e1, double *e2,
                     double *e3) {
  scratch s;
  scratch_alloc(m, &s);
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1), n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1,
       n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  double *dst[9] = {s.e3x1, s.e2x1, s.w1f, s.e1x2, s.e3x2, s.w2f, s.e1x3, s.e2x3, s.w3f};
  const long len[9] = {n1, n1, n1, n2, n2, n2, n3, n3, n3};
  for (int q = 0; q < 9; ++q) memcpy(dst[q], emf[q], sizeof(double) * len[q]);
  /* corner_e writes the mesh's own edge arrays of block b: start them from e1..e3 */
  double *me1 = m->e1 + (long)b * m->ne1, *me2 = m->e2 + (long)b * m->ne2,
         *me3 = m->e3 + (long)b * m->ne3;
  memcpy(me1, e1, sizeof(double) * m->ne1);
  memcpy(me2, e2, sizeof(double) * m->ne2);
  memcpy(me3, e3, sizeof(double) * m->ne3);
  corner_e(m, b, &s);
  memcpy(e1, me1, sizeof(double) * m->ne1);
  memcpy(e2, me2, sizeof(double) * m->ne2);
  memcpy(e3, me3, sizeof(double) * m->ne3);
  scratch_free(&s);
}

/* Hydro::AddFluxDivergence (add_flux_divergence.cpp:39-96) on u (one block's array) */
void orc_op_add_flux_divergence(orc_mesh *m, int b, double wght, const double *flx1,
                                const double *flx2, const double *flx3, double *u) {
  scratch s;
  scratch_alloc(m, &s);
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1), n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1,
       n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  memcpy(s.flx1, flx1, sizeof(double) * NHYDRO * n1);
  memcpy(s.flx2, flx2, sizeof(double) * NHYDRO * n2);
  memcpy(s.flx3, flx3, sizeof(double) * NHYDRO * n3);
  add_flux_divergence(m, b, wght, u, &s);
  scratch_free(&s);
}

/* Field::CT (ct.cpp:31-116) with the given edge EMFs on b1..b3 (one block's arrays) */
void orc_op_ct(orc_mesh *m, int b, double wght, const double *e1, const double *e2,
               const double *e3, double *b1, double *b2, double *b3) {
  scratch s;
  scratch_alloc(m, &s);
  memcpy(s.e1, e1, sizeof(double) * (m->nc3 + 1) * (m->nc2 + 1) * m->nc1);
  memcpy(s.e2, e2, sizeof(double) * (m->nc3 + 1) * m->nc2 * (m->nc1 + 1));
  memcpy(s.e3, e3, sizeof(double) * m->nc3 * (m->nc2 + 1) * (m->nc1 + 1));
  ct_update(m, b, wght, b1, b2, b3, &s);
  scratch_free(&s);
}

/* EquationOfState::ConservedToPrimitive over a range, on the mesh's own u, w, bcc and b of
 * block b (prim = the mesh's w); returns the relativistic failures */
long orc_op_con2prim(orc_mesh *m, int b, int il, int iu, int jl, int ju, int kl, int ku) {
  return con2prim_range(m, b, m->u + (long)b * NHYDRO * m->ncell,
                        m->w + (long)b * NHYDRO * m->ncell, il, iu, jl, ju, kl, ku);
}

/* Hydro::NewBlockTimeStep (new_blockdt.cpp:45-230) of block b: cfl times the minimum */
double orc_op_new_block_dt(orc_mesh *m, int b) { return new_block_dt(m, b); }

void orc_riemann_face(int rsolver, int relativistic, double gamma, const double *wli,
                      const double *wri, double bx, double dvn, double dvt, double *flx7) {
  if (relativistic && rsolver == 2) llf_sr(gamma, wli, wri, bx, flx7);
  else if (relativistic && rsolver == 0) hlld_sr(gamma, wli, wri, bx, flx7);
  else if (relativistic) hlle_sr(gamma, wli, wri, bx, flx7);
  else if (rsolver == 0) hlld(gamma, wli, wri, bx, flx7);
  else if (rsolver == 2) llf(gamma, wli, wri, bx, flx7);
  else if (rsolver == 3) roe(gamma, wli, wri, bx, flx7);
  else if (rsolver == 4) hlld_core(gamma, wli, wri, bx, 1, dvn, dvt, flx7);
  else hlle(gamma, wli, wri, bx, flx7);
}

#include "athena_oracle_ml.c"
