/* Multi-level (SMR/AMR) part of the CPU oracle — TEST INFRASTRUCTURE, not the product.
 *
 * Included at the end of athena_oracle.c (it uses that file's static kernels).  A mesh
 * whose MeshBlocks sit on several refinement levels is advanced exactly as the
 * reference's TimeIntegratorTaskList does for `refinement = static/adaptive`
 * (time_integrator.cpp:904-1208): fluxes, hydro flux correction from finer neighbours
 * (bvals/cc/flux_correction_cc.cpp), the flux divergence, the corner EMFs, the EMF
 * correction across levels (bvals/fc/flux_correction_fc.cpp), CT, the ghost exchange of
 * U and B with restriction to coarser and coarse-buffer filling from coarser neighbours
 * (bvals/cc/bvals_cc.cpp, bvals/fc/bvals_fc.cpp), ProlongateBoundaries
 * (bvals/bvals_refine.cpp with mesh/mesh_refinement.cpp), W(U) over the ranges the
 * neighbour levels give, and the physical boundaries.
 *
 * The host builds the block list and the neighbour lists (athena_gb300/meshtree.py,
 * the reference's MeshBlockTree and SearchAndSetNeighbors) and passes them in with the
 * coarse-buffer coordinates.  Every region below states the reference function whose
 * index ranges it reproduces; the send and receive sides of one transfer give boxes of
 * the same shape, and a transfer copies box to box in (n, k, j, i) order, which is the
 * order the reference packs and unpacks its buffers.
 */

enum { ML_FACE = 0, ML_EDGE = 1, ML_CORNER = 2 };
enum { ML_NF = 10, ML_MAXNB = 56 };

typedef struct {
  int gid, level, ox1, ox2, ox3, type, fi1, fi2, fid, eid;
} ml_nbr;

typedef struct orc_ml {
  ml_nbr *nbr;      /* [nb][ML_MAXNB] */
  int *nnbr;        /* [nb] */
  int *nblev;       /* [nb][27], (ox3+1)*9 + (ox2+1)*3 + (ox1+1) */
  long long *loc;   /* [nb][4]: level, lx1, lx2, lx3 */
  int *edge_flag;   /* [nb][12] */
  int *nedge_fine;  /* [nb][12] */
  int ncc1, ncc2, ncc3, cis, cie, cjs, cje, cks, cke, cng;
  long nccell, ncf1, ncf2, ncf3;
  double *ccons, *cprim, *cbcc, *cb1, *cb2, *cb3;   /* coarse buffers, per block */
  double *cdx1f, *cdx2f, *cdx3f, *cx1v, *cx2v, *cx3v; /* coarse coordinates, per block */
  scratch *sb;      /* per-block scratch of one stage (fluxes, face EMFs, weights) */
} orc_ml;

#define NBL(ml, b, o1, o2, o3) ((ml)->nblev[(long)(b) * 27 + ((o3) + 1) * 9 + ((o2) + 1) * 3 + ((o1) + 1)])
#define CCI(ml, n, k, j, i) ((((long)(n) * (ml)->ncc3 + (k)) * (ml)->ncc2 + (j)) * (ml)->ncc1 + (i))
#define CF1(ml, k, j, i) ((((long)(k)) * (ml)->ncc2 + (j)) * ((ml)->ncc1 + 1) + (i))
#define CF2(ml, k, j, i) ((((long)(k)) * ((ml)->ncc2 + 1) + (j)) * (ml)->ncc1 + (i))
#define CF3(ml, k, j, i) ((((long)(k)) * (ml)->ncc2 + (j)) * (ml)->ncc1 + (i))

/* ---- array views and boxes ---------------------------------------------------------- */
typedef struct { double *p; int n1, n2, n3; } view3;   /* [n3][n2][n1], n1 fastest */
typedef struct { int s[3], e[3]; } box3;                /* inclusive, index 0 = i */

static inline double *V(view3 v, int k, int j, int i) {
  return v.p + ((long)k * v.n2 + j) * v.n1 + i;
}

static view3 fine_cc(const orc_mesh *m, double *base, int b, int nvar, int n) {
  view3 v = {base + ((long)b * nvar + n) * m->ncell, m->nc1, m->nc2, m->nc3};
  return v;
}
static view3 fine_fc(const orc_mesh *m, int d, double *base, int b) {
  view3 v;
  if (d == 0) { v.p = base + (long)b * m->nf1; v.n1 = m->nc1 + 1; v.n2 = m->nc2; v.n3 = m->nc3; }
  else if (d == 1) { v.p = base + (long)b * m->nf2; v.n1 = m->nc1; v.n2 = m->nc2 + 1; v.n3 = m->nc3; }
  else { v.p = base + (long)b * m->nf3; v.n1 = m->nc1; v.n2 = m->nc2; v.n3 = m->nc3 + 1; }
  return v;
}
static view3 coarse_cc(const orc_ml *ml, double *base, int b, int nvar, int n) {
  view3 v = {base + ((long)b * nvar + n) * ml->nccell, ml->ncc1, ml->ncc2, ml->ncc3};
  return v;
}
static view3 coarse_fc(const orc_ml *ml, int d, double *base, int b) {
  view3 v;
  if (d == 0) { v.p = base + (long)b * ml->ncf1; v.n1 = ml->ncc1 + 1; v.n2 = ml->ncc2; v.n3 = ml->ncc3; }
  else if (d == 1) { v.p = base + (long)b * ml->ncf2; v.n1 = ml->ncc1; v.n2 = ml->ncc2 + 1; v.n3 = ml->ncc3; }
  else { v.p = base + (long)b * ml->ncf3; v.n1 = ml->ncc1; v.n2 = ml->ncc2; v.n3 = ml->ncc3 + 1; }
  return v;
}

/* copy box s of src into box d of dst element by element in (k, j, i) order */
static void copy_box(view3 dst, box3 d, view3 src, box3 s) {
  for (int a = 0; a < 3; ++a)
    if (d.e[a] - d.s[a] != s.e[a] - s.s[a]) {
      fprintf(stderr, "oracle: mismatched transfer boxes\n");
      abort();
    }
  for (int k = 0; k <= d.e[2] - d.s[2]; ++k)
    for (int j = 0; j <= d.e[1] - d.s[1]; ++j)
      for (int i = 0; i <= d.e[0] - d.s[0]; ++i)
        *V(dst, d.s[2] + k, d.s[1] + j, d.s[0] + i) = *V(src, s.s[2] + k, s.s[1] + j, s.s[0] + i);
}

static inline int ml_level(const orc_mesh *m, int b) { return (int)m->ml->loc[(long)b * 4]; }
static inline long long ml_lx(const orc_mesh *m, int b, int d) {
  return m->ml->loc[(long)b * 4 + 1 + d];
}
static inline const ml_nbr *ml_nb(const orc_mesh *m, int b, int n) {
  return &m->ml->nbr[(long)b * ML_MAXNB + n];
}

/* the entry of block s's neighbour list that points at block r in direction -o */
static const ml_nbr *ml_back(const orc_mesh *m, int s, int r, const ml_nbr *fwd) {
  for (int n = 0; n < m->ml->nnbr[s]; ++n) {
    const ml_nbr *q = ml_nb(m, s, n);
    if (q->gid == r && q->ox1 == -fwd->ox1 && q->ox2 == -fwd->ox2 && q->ox3 == -fwd->ox3)
      return q;
  }
  fprintf(stderr, "oracle: inconsistent neighbour lists (%d -> %d)\n", s, r);
  abort();
  return NULL;
}

/* ---- restriction (mesh_refinement.cpp:116-189, 272-463; Cartesian areas and volumes,
 * coordinates.cpp:448-547) --------------------------------------------------------- */
static void restrict_cc(const orc_mesh *m, int b, view3 fine, view3 coarse, box3 c) {
  const orc_ml *ml = m->ml;
  const double *dx1 = m->dx1f + (long)b * m->nc1, *dx2 = m->dx2f + (long)b * m->nc2,
               *dx3 = m->dx3f + (long)b * m->nc3;
  for (int ck = c.s[2]; ck <= c.e[2]; ++ck) {
    int k = (ck - ml->cks) * 2 + m->ks;
    for (int cj = c.s[1]; cj <= c.e[1]; ++cj) {
      int j = (cj - ml->cjs) * 2 + m->js;
      for (int ci = c.s[0]; ci <= c.e[0]; ++ci) {
        int i = (ci - ml->cis) * 2 + m->is;
        /* CellVolume(k,j,...)(i) = dx1f(i)*dx2f(j)*dx3f(k) */
        double v000 = dx1[i] * dx2[j] * dx3[k], v001 = dx1[i + 1] * dx2[j] * dx3[k];
        double v010 = dx1[i] * dx2[j + 1] * dx3[k], v011 = dx1[i + 1] * dx2[j + 1] * dx3[k];
        double v100 = dx1[i] * dx2[j] * dx3[k + 1], v101 = dx1[i + 1] * dx2[j] * dx3[k + 1];
        double v110 = dx1[i] * dx2[j + 1] * dx3[k + 1],
               v111 = dx1[i + 1] * dx2[j + 1] * dx3[k + 1];
        double tvol = ((v000 + v010) + (v001 + v011)) + ((v100 + v110) + (v101 + v111));
        *V(coarse, ck, cj, ci) =
            (((*V(fine, k, j, i) * v000 + *V(fine, k, j + 1, i) * v010) +
              (*V(fine, k, j, i + 1) * v001 + *V(fine, k, j + 1, i + 1) * v011)) +
             ((*V(fine, k + 1, j, i) * v100 + *V(fine, k + 1, j + 1, i) * v110) +
              (*V(fine, k + 1, j, i + 1) * v101 + *V(fine, k + 1, j + 1, i + 1) * v111))) /
            tvol;
      }
    }
  }
}

/* x1 faces: area-weighted mean of the four fine faces in the coarse face */
static void restrict_f1(const orc_mesh *m, int b, view3 fine, view3 coarse, box3 c) {
  const orc_ml *ml = m->ml;
  const double *dx2 = m->dx2f + (long)b * m->nc2, *dx3 = m->dx3f + (long)b * m->nc3;
  for (int ck = c.s[2]; ck <= c.e[2]; ++ck) {
    int k = (ck - ml->cks) * 2 + m->ks;
    for (int cj = c.s[1]; cj <= c.e[1]; ++cj) {
      int j = (cj - ml->cjs) * 2 + m->js;
      double a00 = dx2[j] * dx3[k], a01 = dx2[j + 1] * dx3[k];
      double a10 = dx2[j] * dx3[k + 1], a11 = dx2[j + 1] * dx3[k + 1];
      for (int ci = c.s[0]; ci <= c.e[0]; ++ci) {
        int i = (ci - ml->cis) * 2 + m->is;
        double tarea = a00 + a01 + a10 + a11;
        *V(coarse, ck, cj, ci) =
            (*V(fine, k, j, i) * a00 + *V(fine, k, j + 1, i) * a01 +
             *V(fine, k + 1, j, i) * a10 + *V(fine, k + 1, j + 1, i) * a11) / tarea;
      }
    }
  }
}

static void restrict_f2(const orc_mesh *m, int b, view3 fine, view3 coarse, box3 c) {
  const orc_ml *ml = m->ml;
  const double *dx1 = m->dx1f + (long)b * m->nc1, *dx3 = m->dx3f + (long)b * m->nc3;
  for (int ck = c.s[2]; ck <= c.e[2]; ++ck) {
    int k = (ck - ml->cks) * 2 + m->ks;
    for (int cj = c.s[1]; cj <= c.e[1]; ++cj) {
      int j = (cj - ml->cjs) * 2 + m->js;
      for (int ci = c.s[0]; ci <= c.e[0]; ++ci) {
        int i = (ci - ml->cis) * 2 + m->is;
        double s0i = dx1[i] * dx3[k], s0p = dx1[i + 1] * dx3[k];
        double s1i = dx1[i] * dx3[k + 1], s1p = dx1[i + 1] * dx3[k + 1];
        double tarea = s0i + s0p + s1i + s1p;
        *V(coarse, ck, cj, ci) =
            (*V(fine, k, j, i) * s0i + *V(fine, k, j, i + 1) * s0p +
             *V(fine, k + 1, j, i) * s1i + *V(fine, k + 1, j, i + 1) * s1p) / tarea;
      }
    }
  }
}

static void restrict_f3(const orc_mesh *m, int b, view3 fine, view3 coarse, box3 c) {
  const orc_ml *ml = m->ml;
  const double *dx1 = m->dx1f + (long)b * m->nc1, *dx2 = m->dx2f + (long)b * m->nc2;
  for (int ck = c.s[2]; ck <= c.e[2]; ++ck) {
    int k = (ck - ml->cks) * 2 + m->ks;
    for (int cj = c.s[1]; cj <= c.e[1]; ++cj) {
      int j = (cj - ml->cjs) * 2 + m->js;
      for (int ci = c.s[0]; ci <= c.e[0]; ++ci) {
        int i = (ci - ml->cis) * 2 + m->is;
        double s0i = dx1[i] * dx2[j], s0p = dx1[i + 1] * dx2[j];
        double s1i = dx1[i] * dx2[j + 1], s1p = dx1[i + 1] * dx2[j + 1];
        double tarea = s0i + s0p + s1i + s1p;
        *V(coarse, ck, cj, ci) =
            (*V(fine, k, j, i) * s0i + *V(fine, k, j, i + 1) * s0p +
             *V(fine, k, j + 1, i) * s1i + *V(fine, k, j + 1, i + 1) * s1p) / tarea;
      }
    }
  }
}

static void restrict_fc(const orc_mesh *m, int b, int d, view3 fine, view3 coarse, box3 c) {
  if (d == 0) restrict_f1(m, b, fine, coarse, c);
  else if (d == 1) restrict_f2(m, b, fine, coarse, c);
  else restrict_f3(m, b, fine, coarse, c);
}

/* ---- transfer regions ------------------------------------------------------------------
 * Conventions: o[3] = the neighbour offset as seen by the block whose region is computed
 * (ox1, ox2, ox3 of that block's NeighborBlock entry); fi1/fi2 that entry's fine-block
 * offsets.  lo/hi = the block's own interior range, per axis. */
typedef struct {
  int lo[3], hi[3];      /* fine interior: is..ie, js..je, ks..ke */
  int clo[3], chi[3];    /* coarse interior: cis..cie, ... */
  int n[3];              /* nx1, nx2, nx3 */
  int ng, cng;
} ml_ix;

static ml_ix ml_index(const orc_mesh *m) {
  ml_ix x;
  x.lo[0] = m->is; x.hi[0] = m->ie; x.lo[1] = m->js; x.hi[1] = m->je;
  x.lo[2] = m->ks; x.hi[2] = m->ke;
  x.clo[0] = m->ml->cis; x.chi[0] = m->ml->cie; x.clo[1] = m->ml->cjs;
  x.chi[1] = m->ml->cje; x.clo[2] = m->ml->cks; x.chi[2] = m->ml->cke;
  x.n[0] = m->p.nx1; x.n[1] = m->p.nx2; x.n[2] = m->p.nx3;
  x.ng = m->p.ng; x.cng = m->ml->cng;
  return x;
}

static void nb_off(const ml_nbr *q, int o[3]) { o[0] = q->ox1; o[1] = q->ox2; o[2] = q->ox3; }

/* which fine-block offset selects the half of axis a (a has offset 0): axis 0 always
 * fi1; axis 1 fi1 when ox1 != 0, else fi2; axis 2 fi1 when ox1 and ox2 are both
 * nonzero, else fi2 (bvals_cc.cpp:369-394, 502-531) */
static int half_sel(const ml_nbr *q, int a) {
  if (a == 0) return q->fi1;
  if (a == 1) return q->ox1 != 0 ? q->fi1 : q->fi2;
  return (q->ox1 != 0 && q->ox2 != 0) ? q->fi1 : q->fi2;
}

/* CellCenteredBoundaryVariable::LoadBoundaryBufferSameLevel (bvals_cc.cpp:260-276) */
static box3 cc_send_same(const ml_ix *x, const ml_nbr *q) {
  box3 r; int o[3]; nb_off(q, o);
  for (int a = 0; a < 3; ++a) {
    r.s[a] = (o[a] > 0) ? x->hi[a] - x->ng + 1 : x->lo[a];
    r.e[a] = (o[a] < 0) ? x->lo[a] + x->ng - 1 : x->hi[a];
  }
  return r;
}
/* SetBoundarySameLevel (bvals_cc.cpp:403-417) */
static box3 cc_recv_same(const ml_ix *x, const ml_nbr *q) {
  box3 r; int o[3]; nb_off(q, o);
  for (int a = 0; a < 3; ++a) {
    if (o[a] == 0) { r.s[a] = x->lo[a]; r.e[a] = x->hi[a]; }
    else if (o[a] > 0) { r.s[a] = x->hi[a] + 1; r.e[a] = x->hi[a] + x->ng; }
    else { r.s[a] = x->lo[a] - x->ng; r.e[a] = x->lo[a] - 1; }
  }
  return r;
}
/* LoadBoundaryBufferToCoarser (bvals_cc.cpp:284-303), coarse indices */
static box3 cc_send_coarser(const ml_ix *x, const ml_nbr *q) {
  box3 r; int o[3]; nb_off(q, o);
  int cn = x->ng - 1;
  for (int a = 0; a < 3; ++a) {
    r.s[a] = (o[a] > 0) ? x->chi[a] - cn : x->clo[a];
    r.e[a] = (o[a] < 0) ? x->clo[a] + cn : x->chi[a];
  }
  return r;
}
/* SetBoundaryFromFiner (bvals_cc.cpp:491-540) */
static box3 cc_recv_finer(const ml_ix *x, const ml_nbr *q) {
  box3 r; int o[3]; nb_off(q, o);
  for (int a = 0; a < 3; ++a) {
    if (o[a] == 0) {
      r.s[a] = x->lo[a]; r.e[a] = x->hi[a];
      if (half_sel(q, a) == 1) r.s[a] += x->n[a] / 2; else r.e[a] -= x->n[a] / 2;
    } else if (o[a] > 0) { r.s[a] = x->hi[a] + 1; r.e[a] = x->hi[a] + x->ng; }
    else { r.s[a] = x->lo[a] - x->ng; r.e[a] = x->lo[a] - 1; }
  }
  return r;
}
/* LoadBoundaryBufferToFiner (bvals_cc.cpp:311-351), fine indices of the coarse sender */
static box3 cc_send_finer(const ml_ix *x, const ml_nbr *q) {
  box3 r; int o[3]; nb_off(q, o);
  int cn = x->cng - 1;
  for (int a = 0; a < 3; ++a) {
    r.s[a] = (o[a] > 0) ? x->hi[a] - cn : x->lo[a];
    r.e[a] = (o[a] < 0) ? x->lo[a] + cn : x->hi[a];
    if (o[a] == 0) {
      if (half_sel(q, a) == 1) r.s[a] += x->n[a] / 2 - x->cng;
      else r.e[a] -= x->n[a] / 2 - x->cng;
    }
  }
  return r;
}
/* SetBoundaryFromCoarser (bvals_cc.cpp:423-468), coarse indices of the fine receiver;
 * par[a] = the receiver's lx parity along a */
static box3 cc_recv_coarser(const ml_ix *x, const ml_nbr *q, const int par[3]) {
  box3 r; int o[3]; nb_off(q, o);
  for (int a = 0; a < 3; ++a) {
    if (o[a] == 0) {
      r.s[a] = x->clo[a]; r.e[a] = x->chi[a];
      if (par[a] == 0) r.e[a] += x->cng; else r.s[a] -= x->cng;
    } else if (o[a] > 0) { r.s[a] = x->chi[a] + 1; r.e[a] = x->chi[a] + x->cng; }
    else { r.s[a] = x->clo[a] - x->cng; r.e[a] = x->clo[a] - 1; }
  }
  return r;
}

/* Face fields.  For component d the axis a == d runs over faces (own range lo..hi+1).
 * The reference computes the three components one after another, carrying the ranges
 * of the axes it does not recompute (bvals_fc.cpp:344-970); every case below is written
 * out per axis. */

/* LoadBoundaryBufferSameLevel (bvals_fc.cpp:344-398), multilevel mesh */
static box3 fc_send_same(const ml_ix *x, const ml_nbr *q, int d) {
  box3 r; int o[3]; nb_off(q, o);
  int ng = x->ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) { r.s[a] = x->lo[a]; r.e[a] = x->hi[a] + 1; }
      else if (o[a] > 0) { r.s[a] = x->hi[a] - ng + 1; r.e[a] = x->hi[a]; }
      else { r.s[a] = x->lo[a] + 1; r.e[a] = x->lo[a] + ng; }
      if (q->type != ML_FACE) {  /* the overlapping face of edges and corners */
        if (o[a] > 0) r.e[a]++;
        else if (o[a] < 0) r.s[a]--;
      }
    } else {
      if (o[a] == 0) { r.s[a] = x->lo[a]; r.e[a] = x->hi[a]; }
      else if (o[a] > 0) { r.s[a] = x->hi[a] - ng + 1; r.e[a] = x->hi[a]; }
      else { r.s[a] = x->lo[a]; r.e[a] = x->lo[a] + ng - 1; }
    }
  }
  return r;
}
/* SetBoundarySameLevel (bvals_fc.cpp:583-684), multilevel mesh */
static box3 fc_recv_same(const ml_ix *x, const ml_nbr *q, int d) {
  box3 r; int o[3]; nb_off(q, o);
  int ng = x->ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) { r.s[a] = x->lo[a]; r.e[a] = x->hi[a] + 1; }
      else if (o[a] > 0) { r.s[a] = x->hi[a] + 2; r.e[a] = x->hi[a] + ng + 1; }
      else { r.s[a] = x->lo[a] - ng; r.e[a] = x->lo[a] - 1; }
      if (q->type != ML_FACE) {
        if (o[a] > 0) r.s[a]--;
        else if (o[a] < 0) r.e[a]++;
      }
    } else {
      if (o[a] == 0) { r.s[a] = x->lo[a]; r.e[a] = x->hi[a]; }
      else if (o[a] > 0) { r.s[a] = x->hi[a] + 1; r.e[a] = x->hi[a] + ng; }
      else { r.s[a] = x->lo[a] - ng; r.e[a] = x->lo[a] - 1; }
    }
  }
  return r;
}
/* LoadBoundaryBufferToCoarser (bvals_fc.cpp:403-471), coarse indices; the ghost width
 * here is NGHOST */
static box3 fc_send_coarser(const ml_ix *x, const ml_nbr *q, int d) {
  box3 r; int o[3]; nb_off(q, o);
  int cg = x->ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) { r.s[a] = x->clo[a]; r.e[a] = x->chi[a] + 1; }
      else if (o[a] > 0) { r.s[a] = x->chi[a] - cg + 1; r.e[a] = x->chi[a]; }
      else { r.s[a] = x->clo[a] + 1; r.e[a] = x->clo[a] + cg; }
      if (q->type != ML_FACE) {
        if (o[a] > 0) r.e[a]++;
        else if (o[a] < 0) r.s[a]--;
      }
    } else {
      if (o[a] == 0) { r.s[a] = x->clo[a]; r.e[a] = x->chi[a]; }
      else if (o[a] > 0) { r.s[a] = x->chi[a] - cg + 1; r.e[a] = x->chi[a]; }
      else { r.s[a] = x->clo[a]; r.e[a] = x->clo[a] + cg - 1; }
    }
  }
  return r;
}
/* SetBoundaryFromFiner (bvals_fc.cpp:813-973) */
static box3 fc_recv_finer(const ml_ix *x, const ml_nbr *q, int d) {
  box3 r; int o[3]; nb_off(q, o);
  int ng = x->ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) {
        r.s[a] = x->lo[a]; r.e[a] = x->hi[a] + 1;
        if (half_sel(q, a) == 1) r.s[a] += x->n[a] / 2; else r.e[a] -= x->n[a] / 2;
      } else if (o[a] > 0) { r.s[a] = x->hi[a] + 2; r.e[a] = x->hi[a] + ng + 1; }
      else { r.s[a] = x->lo[a] - ng; r.e[a] = x->lo[a] - 1; }
      if (q->type != ML_FACE) {
        if (o[a] > 0) r.s[a]--;
        else if (o[a] < 0) r.e[a]++;
      }
    } else {
      if (o[a] == 0) {
        r.s[a] = x->lo[a]; r.e[a] = x->hi[a];
        if (half_sel(q, a) == 1) r.s[a] += x->n[a] / 2; else r.e[a] -= x->n[a] / 2;
      } else if (o[a] > 0) { r.s[a] = x->hi[a] + 1; r.e[a] = x->hi[a] + ng; }
      else { r.s[a] = x->lo[a] - ng; r.e[a] = x->lo[a] - 1; }
    }
  }
  return r;
}
/* LoadBoundaryBufferToFiner (bvals_fc.cpp:476-578), fine indices of the coarse sender */
static box3 fc_send_finer(const ml_ix *x, const ml_nbr *q, int d) {
  box3 r; int o[3]; nb_off(q, o);
  int cg = x->cng, cn = x->cng - 1;
  for (int a = 0; a < 3; ++a) {
    int h = x->n[a] / 2 - cg;
    if (a == d) {
      if (o[a] == 0) {
        r.s[a] = x->lo[a]; r.e[a] = x->hi[a] + 1;
        if (half_sel(q, a) == 1) r.s[a] += h; else r.e[a] -= h;
      } else if (o[a] > 0) { r.s[a] = x->hi[a] + 1 - cg; r.e[a] = x->hi[a] + 1; }
      else { r.s[a] = x->lo[a]; r.e[a] = x->lo[a] + cg; }
    } else {
      if (o[a] == 0) {
        r.s[a] = x->lo[a]; r.e[a] = x->hi[a];
        if (half_sel(q, a) == 1) r.s[a] += h; else r.e[a] -= h;
      } else if (o[a] > 0) { r.s[a] = x->hi[a] - cn; r.e[a] = x->hi[a]; }
      else { r.s[a] = x->lo[a]; r.e[a] = x->lo[a] + cn; }
    }
  }
  return r;
}
/* SetBoundaryFromCoarser (bvals_fc.cpp:690-808), coarse indices of the fine receiver */
static box3 fc_recv_coarser(const ml_ix *x, const ml_nbr *q, int d, const int par[3]) {
  box3 r; int o[3]; nb_off(q, o);
  int cg = x->cng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) {
        r.s[a] = x->clo[a]; r.e[a] = x->chi[a] + 1;
        if (par[a] == 0) r.e[a] += cg; else r.s[a] -= cg;
      } else if (o[a] > 0) { r.s[a] = x->chi[a] + 1; r.e[a] = x->chi[a] + 1 + cg; }
      else { r.s[a] = x->clo[a] - cg; r.e[a] = x->clo[a]; }
    } else {
      if (o[a] == 0) {
        r.s[a] = x->clo[a]; r.e[a] = x->chi[a];
        if (par[a] == 0) r.e[a] += cg; else r.s[a] -= cg;
      } else if (o[a] > 0) { r.s[a] = x->chi[a] + 1; r.e[a] = x->chi[a] + cg; }
      else { r.s[a] = x->clo[a] - cg; r.e[a] = x->clo[a] - 1; }
    }
  }
  return r;
}

/* ---- ghost exchange across levels ------------------------------------------------------
 * SendBoundaryBuffers / ReceiveAndSetBoundariesWithWait for U (cell-centred, nvar
 * variables of `cc`) and the face field: first every block's restriction for its coarser
 * neighbours into its own coarse buffers (the side effect of LoadBoundaryBufferToCoarser,
 * whose values are the ones sent), then per receiving block, in neighbour-list order,
 * the copies into its ghost zones (same level, finer senders) or its coarse buffers
 * (coarser senders).  The senders read only their own cells and faces, so the order
 * across blocks does not matter; within one block the list order decides the faces that
 * edges and corners overwrite. */
static void ml_exchange(orc_mesh *m, double *cc, int nvar, double *ccoarse, double *f1,
                        double *f2, double *f3) {
  orc_ml *ml = m->ml;
  ml_ix x = ml_index(m);
  double *fb[3] = {f1, f2, f3};
  double *cfb[3] = {ml->cb1, ml->cb2, ml->cb3};
#pragma omp parallel for schedule(dynamic, 1)
  for (int s = 0; s < m->nb; ++s) {
    int lev = ml_level(m, s);
    for (int n = 0; n < ml->nnbr[s]; ++n) {
      const ml_nbr *q = ml_nb(m, s, n);
      if (q->level >= lev) continue;
      if (cc) {
        box3 c = cc_send_coarser(&x, q);
        for (int v = 0; v < nvar; ++v)
          restrict_cc(m, s, fine_cc(m, cc, s, nvar, v), coarse_cc(ml, ccoarse, s, nvar, v), c);
      }
      if (f1)
        for (int d = 0; d < 3; ++d)
          restrict_fc(m, s, d, fine_fc(m, d, fb[d], s), coarse_fc(ml, d, cfb[d], s),
                      fc_send_coarser(&x, q, d));
    }
  }
  /* the values sent to coarser blocks, as packed at send time: a block's own receives
   * from its coarser neighbours below may overwrite parts of its coarse buffers */
  double *scc = NULL, *sfb[3] = {NULL, NULL, NULL};
  if (cc) {
    scc = malloc(sizeof(double) * m->nb * nvar * ml->nccell);
    memcpy(scc, ccoarse, sizeof(double) * m->nb * nvar * ml->nccell);
  }
  if (f1) {
    long nf[3] = {ml->ncf1, ml->ncf2, ml->ncf3};
    for (int d = 0; d < 3; ++d) {
      sfb[d] = malloc(sizeof(double) * m->nb * nf[d]);
      memcpy(sfb[d], cfb[d], sizeof(double) * m->nb * nf[d]);
    }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int r = 0; r < m->nb; ++r) {
    int lev = ml_level(m, r);
    int par[3] = {(int)(ml_lx(m, r, 0) & 1), (int)(ml_lx(m, r, 1) & 1),
                  (int)(ml_lx(m, r, 2) & 1)};
    for (int n = 0; n < ml->nnbr[r]; ++n) {
      const ml_nbr *q = ml_nb(m, r, n);
      int s = q->gid;
      const ml_nbr *qs = ml_back(m, s, r, q);
      if (q->level == lev) {
        if (cc) {
          box3 d = cc_recv_same(&x, q), o = cc_send_same(&x, qs);
          for (int v = 0; v < nvar; ++v)
            copy_box(fine_cc(m, cc, r, nvar, v), d, fine_cc(m, cc, s, nvar, v), o);
        }
        if (f1)
          for (int dd = 0; dd < 3; ++dd)
            copy_box(fine_fc(m, dd, fb[dd], r), fc_recv_same(&x, q, dd),
                     fine_fc(m, dd, fb[dd], s), fc_send_same(&x, qs, dd));
      } else if (q->level < lev) {  /* coarser sender: into my coarse buffers */
        if (cc) {
          box3 d = cc_recv_coarser(&x, q, par), o = cc_send_finer(&x, qs);
          for (int v = 0; v < nvar; ++v)
            copy_box(coarse_cc(ml, ccoarse, r, nvar, v), d, fine_cc(m, cc, s, nvar, v), o);
        }
        if (f1)
          for (int dd = 0; dd < 3; ++dd)
            copy_box(coarse_fc(ml, dd, cfb[dd], r), fc_recv_coarser(&x, q, dd, par),
                     fine_fc(m, dd, fb[dd], s), fc_send_finer(&x, qs, dd));
      } else {  /* finer sender: its restricted values into my ghost zones */
        if (cc) {
          box3 d = cc_recv_finer(&x, q), o = cc_send_coarser(&x, qs);
          for (int v = 0; v < nvar; ++v)
            copy_box(fine_cc(m, cc, r, nvar, v), d, coarse_cc(ml, scc, s, nvar, v), o);
        }
        if (f1)
          for (int dd = 0; dd < 3; ++dd)
            copy_box(fine_fc(m, dd, fb[dd], r), fc_recv_finer(&x, q, dd),
                     coarse_fc(ml, dd, sfb[dd], s), fc_send_coarser(&x, qs, dd));
      }
    }
  }
  free(scc);
  free(sfb[0]); free(sfb[1]); free(sfb[2]);
}

/* ---- hydro flux correction (flux_correction_cc.cpp:54-140, 237-286) ----------------------
 * The coarse block's fluxes on a face shared with four finer blocks are replaced by the
 * area-weighted restriction of the finer blocks' fluxes. */
static void ml_flux_correction(orc_mesh *m) {
  orc_ml *ml = m->ml;
  long n1 = (long)m->nc3 * m->nc2 * (m->nc1 + 1), n2 = (long)m->nc3 * (m->nc2 + 1) * m->nc1,
       n3 = (long)(m->nc3 + 1) * m->nc2 * m->nc1;
  int nx1 = m->p.nx1, nx2 = m->p.nx2, nx3 = m->p.nx3;
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < m->nb; ++b) {
    int lev = ml_level(m, b);
    for (int n = 0; n < ml->nnbr[b]; ++n) {
      const ml_nbr *q = ml_nb(m, b, n);
      if (q->type != ML_FACE) break;
      if (q->level != lev + 1) continue;
      int f = q->gid;
      const scratch *sf = &ml->sb[f];
      scratch *sc = &ml->sb[b];
      const double *dx1 = m->dx1f + (long)f * m->nc1, *dx2 = m->dx2f + (long)f * m->nc2,
                   *dx3 = m->dx3f + (long)f * m->nc3;
      if (q->fid == 0 || q->fid == 1) {
        int ic = (q->fid == 0) ? m->is : m->ie + 1;
        int iff = (q->fid == 0) ? m->ie + 1 : m->is;  /* the finer block's face */
        int jl = m->js, ju = m->je, kl = m->ks, ku = m->ke;
        if (q->fi1 == 0) ju -= nx2 / 2; else jl += nx2 / 2;
        if (q->fi2 == 0) ku -= nx3 / 2; else kl += nx3 / 2;
        for (int v = 0; v < NHYDRO; ++v)
          for (int k = kl; k <= ku; ++k)
            for (int j = jl; j <= ju; ++j) {
              int kf = m->ks + 2 * (k - kl), jf = m->js + 2 * (j - jl);
              double amm = dx2[jf] * dx3[kf], amp = dx2[jf + 1] * dx3[kf];
              double apm = dx2[jf] * dx3[kf + 1], app = dx2[jf + 1] * dx3[kf + 1];
              double tarea = amm + amp + apm + app;
              const double *F = sf->flx1 + v * n1;
              sc->flx1[v * n1 + F1IDX(m, k, j, ic)] =
                  (F[F1IDX(m, kf, jf, iff)] * amm + F[F1IDX(m, kf, jf + 1, iff)] * amp +
                   F[F1IDX(m, kf + 1, jf, iff)] * apm + F[F1IDX(m, kf + 1, jf + 1, iff)] * app) /
                  tarea;
            }
      } else if (q->fid == 2 || q->fid == 3) {
        int jc = (q->fid == 2) ? m->js : m->je + 1;
        int jff = (q->fid == 2) ? m->je + 1 : m->js;
        int il = m->is, iu = m->ie, kl = m->ks, ku = m->ke;
        if (q->fi1 == 0) iu -= nx1 / 2; else il += nx1 / 2;
        if (q->fi2 == 0) ku -= nx3 / 2; else kl += nx3 / 2;
        for (int v = 0; v < NHYDRO; ++v)
          for (int k = kl; k <= ku; ++k)
            for (int i = il; i <= iu; ++i) {
              int kf = m->ks + 2 * (k - kl), iff = m->is + 2 * (i - il);
              double s0i = dx1[iff] * dx3[kf], s0p = dx1[iff + 1] * dx3[kf];
              double s1i = dx1[iff] * dx3[kf + 1], s1p = dx1[iff + 1] * dx3[kf + 1];
              double tarea = s0i + s0p + s1i + s1p;
              const double *F = sf->flx2 + v * n2;
              sc->flx2[v * n2 + F2IDX(m, k, jc, i)] =
                  (F[F2IDX(m, kf, jff, iff)] * s0i + F[F2IDX(m, kf, jff, iff + 1)] * s0p +
                   F[F2IDX(m, kf + 1, jff, iff)] * s1i + F[F2IDX(m, kf + 1, jff, iff + 1)] * s1p) /
                  tarea;
            }
      } else {
        int kc = (q->fid == 4) ? m->ks : m->ke + 1;
        int kff = (q->fid == 4) ? m->ke + 1 : m->ks;
        int il = m->is, iu = m->ie, jl = m->js, ju = m->je;
        if (q->fi1 == 0) iu -= nx1 / 2; else il += nx1 / 2;
        if (q->fi2 == 0) ju -= nx2 / 2; else jl += nx2 / 2;
        for (int v = 0; v < NHYDRO; ++v)
          for (int j = jl; j <= ju; ++j)
            for (int i = il; i <= iu; ++i) {
              int jf = m->js + 2 * (j - jl), iff = m->is + 2 * (i - il);
              double s0i = dx1[iff] * dx2[jf], s0p = dx1[iff + 1] * dx2[jf];
              double s1i = dx1[iff] * dx2[jf + 1], s1p = dx1[iff + 1] * dx2[jf + 1];
              double tarea = s0i + s0p + s1i + s1p;
              const double *F = sf->flx3 + v * n3;
              sc->flx3[v * n3 + F3IDX(m, kc, j, i)] =
                  (F[F3IDX(m, kff, jf, iff)] * s0i + F[F3IDX(m, kff, jf, iff + 1)] * s0p +
                   F[F3IDX(m, kff, jf + 1, iff)] * s1i + F[F3IDX(m, kff, jf + 1, iff + 1)] * s1p) /
                  tarea;
            }
      }
    }
  }
}

/* ---- EMF correction across levels (flux_correction_fc.cpp) ------------------------------
 * FaceCenteredBoundaryVariable::CountFineEdges (bvals_fc.cpp:1129-1196): per block edge,
 * whether it touches no finer block (edge_flag) and how many blocks of the finest level
 * around it share it (nedge_fine). */
static void ml_count_fine_edges(orc_mesh *m, int b) {
  orc_ml *ml = m->ml;
  int lev = ml_level(m, b), eid = 0;
  /* x1x2 edges (ox2 outer, ox1 inner), x1x3 (ox3, ox1), x2x3 (ox3, ox2) */
  for (int t = 0; t < 3; ++t) {
    int a = (t == 2) ? 1 : 0, c = (t == 0) ? 1 : 2;  /* inner axis a, outer axis c */
    for (int oc = -1; oc <= 1; oc += 2)
      for (int oa = -1; oa <= 1; oa += 2) {
        int nas = (oa - 1 > -1) ? oa - 1 : -1, nae = (oa + 1 < 1) ? oa + 1 : 1;
        int ncs = (oc - 1 > -1) ? oc - 1 : -1, nce = (oc + 1 < 1) ? oc + 1 : 1;
        int nf = 0, fl = lev;
        for (int nc = ncs; nc <= nce; ++nc)
          for (int na = nas; na <= nae; ++na) {
            int o[3] = {0, 0, 0};
            o[a] = na; o[c] = nc;
            int l = NBL(ml, b, o[0], o[1], o[2]);
            if (l > fl) { fl++; nf = 0; }
            if (l == fl) nf++;
          }
        ml->edge_flag[b * 12 + eid] = (fl == lev);
        ml->nedge_fine[b * 12 + eid] = nf;
        eid++;
      }
  }
}

/* position of the block-face plane or edge line of face fid / edge eid */
static int face_pos(const orc_mesh *m, int fid) {
  int lo[3] = {m->is, m->js, m->ks}, hi[3] = {m->ie, m->je, m->ke};
  return (fid & 1) ? hi[fid >> 1] + 1 : lo[fid >> 1];
}
static void edge_pos(const orc_mesh *m, int eid, int *p1, int *p2) {
  /* eid 0-3: (i, j) of an e3 line; 4-7: (i, k) of e2; 8-11: (j, k) of e1 */
  int a = (eid < 8) ? 0 : 1, c = (eid < 4) ? 1 : 2;
  int lo[3] = {m->is, m->js, m->ks}, hi[3] = {m->ie, m->je, m->ke};
  *p1 = (eid & 1) ? hi[a] + 1 : lo[a];
  *p2 = (eid & 2) ? hi[c] + 1 : lo[c];
}

#define EA(E, kk, jj, ii, c) (E)[(c) == 0 ? E1IDX(m, kk, jj, ii) : (c) == 1 ? E2IDX(m, kk, jj, ii) : E3IDX(m, kk, jj, ii)]

/* the corrected edges of block b, from every block's own pre-correction edges
 * (m->e1..e3): same-level sums (SetFluxBoundarySameLevel), clearing of edges shared
 * with finer blocks (ClearCoarseFluxBoundary), sums of the finer blocks' restricted
 * edges (SetFluxBoundaryFromFiner) and the division by the number of contributions
 * (AverageFluxBoundary); flux_correction_fc.cpp:689-1545 */
static void ml_emf_correct_block(orc_mesh *m, int b, double *e1, double *e2, double *e3) {
  orc_ml *ml = m->ml;
  int lev = ml_level(m, b);
  int is = m->is, ie = m->ie, js = m->js, je = m->je, ks = m->ks, ke = m->ke;
  int nx1 = m->p.nx1, nx2 = m->p.nx2, nx3 = m->p.nx3;
  double *E[3] = {e1, e2, e3};
  memcpy(e1, m->e1 + (long)b * m->ne1, sizeof(double) * m->ne1);
  memcpy(e2, m->e2 + (long)b * m->ne2, sizeof(double) * m->ne2);
  memcpy(e3, m->e3 + (long)b * m->ne3, sizeof(double) * m->ne3);
  /* same level */
  for (int n = 0; n < ml->nnbr[b]; ++n) {
    const ml_nbr *q = ml_nb(m, b, n);
    if (q->type != ML_FACE && q->type != ML_EDGE) break;
    if (q->level != lev) continue;
    if (q->type == ML_EDGE && !ml->edge_flag[b * 12 + q->eid]) continue;
    int s = q->gid;
    const ml_nbr *qs = ml_back(m, s, b, q);
    const double *S[3] = {m->e1 + (long)s * m->ne1, m->e2 + (long)s * m->ne2,
                          m->e3 + (long)s * m->ne3};
    if (q->type == ML_FACE) {
      int p = face_pos(m, q->fid), ps = face_pos(m, qs->fid), ax = q->fid >> 1;
      if (ax == 0) {
        for (int k = ks; k <= ke + 1; ++k)
          for (int j = js; j <= je; ++j) EA(E[1], k, j, p, 1) += EA(S[1], k, j, ps, 1);
        for (int k = ks; k <= ke; ++k)
          for (int j = js; j <= je + 1; ++j) EA(E[2], k, j, p, 2) += EA(S[2], k, j, ps, 2);
      } else if (ax == 1) {
        for (int k = ks; k <= ke + 1; ++k)
          for (int i = is; i <= ie; ++i) EA(E[0], k, p, i, 0) += EA(S[0], k, ps, i, 0);
        for (int k = ks; k <= ke; ++k)
          for (int i = is; i <= ie + 1; ++i) EA(E[2], k, p, i, 2) += EA(S[2], k, ps, i, 2);
      } else {
        for (int j = js; j <= je + 1; ++j)
          for (int i = is; i <= ie; ++i) EA(E[0], p, j, i, 0) += EA(S[0], ps, j, i, 0);
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie + 1; ++i) EA(E[1], p, j, i, 1) += EA(S[1], ps, j, i, 1);
      }
    } else {
      int p1, p2, s1, s2;
      edge_pos(m, q->eid, &p1, &p2);
      edge_pos(m, qs->eid, &s1, &s2);
      if (q->eid < 4) {
        for (int k = ks; k <= ke; ++k) EA(E[2], k, p2, p1, 2) += EA(S[2], k, s2, s1, 2);
      } else if (q->eid < 8) {
        for (int j = js; j <= je; ++j) EA(E[1], p2, j, p1, 1) += EA(S[1], s2, j, s1, 1);
      } else {
        for (int i = is; i <= ie; ++i) EA(E[0], p2, p1, i, 0) += EA(S[0], s2, s1, i, 0);
      }
    }
  }
  /* ClearCoarseFluxBoundary (flux_correction_fc.cpp:1214-1352) */
  for (int f = 0; f < 6; ++f) {
    int o[3] = {0, 0, 0};
    o[f >> 1] = (f & 1) ? 1 : -1;
    if (NBL(ml, b, o[0], o[1], o[2]) <= lev) continue;
    int p = face_pos(m, f);
    if (f < 2) {
      for (int k = ks + 1; k <= ke; ++k)
        for (int j = js; j <= je; ++j) EA(E[1], k, j, p, 1) = 0.0;
      for (int k = ks; k <= ke; ++k)
        for (int j = js + 1; j <= je; ++j) EA(E[2], k, j, p, 2) = 0.0;
    } else if (f < 4) {
      for (int k = ks + 1; k <= ke; ++k)
        for (int i = is; i <= ie; ++i) EA(E[0], k, p, i, 0) = 0.0;
      for (int k = ks; k <= ke; ++k)
        for (int i = is + 1; i <= ie; ++i) EA(E[2], k, p, i, 2) = 0.0;
    } else {
      for (int j = js + 1; j <= je; ++j)
        for (int i = is; i <= ie; ++i) EA(E[0], p, j, i, 0) = 0.0;
      for (int j = js; j <= je; ++j)
        for (int i = is + 1; i <= ie; ++i) EA(E[1], p, j, i, 1) = 0.0;
    }
  }
  for (int eid = 0; eid < 12; ++eid) {
    if (ml->edge_flag[b * 12 + eid]) continue;
    int p1, p2;
    edge_pos(m, eid, &p1, &p2);
    if (eid < 4) for (int k = ks; k <= ke; ++k) EA(E[2], k, p2, p1, 2) = 0.0;
    else if (eid < 8) for (int j = js; j <= je; ++j) EA(E[1], p2, j, p1, 1) = 0.0;
    else for (int i = is; i <= ie; ++i) EA(E[0], p2, p1, i, 0) = 0.0;
  }
  /* from finer blocks: the sender restricts its edges (LoadFluxBoundaryBufferToCoarser,
   * flux_correction_fc.cpp:315-570), the receiver adds them to its half of the face or
   * edge */
  for (int n = 0; n < ml->nnbr[b]; ++n) {
    const ml_nbr *q = ml_nb(m, b, n);
    if (q->type != ML_FACE && q->type != ML_EDGE) break;
    if (q->level != lev + 1) continue;
    int s = q->gid;
    const ml_nbr *qs = ml_back(m, s, b, q);
    const double *S[3] = {m->e1 + (long)s * m->ne1, m->e2 + (long)s * m->ne2,
                          m->e3 + (long)s * m->ne3};
    const double *dx1 = m->dx1f + (long)s * m->nc1, *dx2 = m->dx2f + (long)s * m->nc2,
                 *dx3 = m->dx3f + (long)s * m->nc3;
    if (q->type == ML_FACE) {
      int p = face_pos(m, q->fid), ps = face_pos(m, qs->fid), ax = q->fid >> 1;
      if (ax == 0) {
        int jl = js, ju = je, kl = ks, ku = ke;
        if (q->fi1 == 0) ju = js + nx2 / 2 - 1; else jl = js + nx2 / 2;
        if (q->fi2 == 0) ku = ks + nx3 / 2 - 1; else kl = ks + nx3 / 2;
        for (int k = kl; k <= ku + 1; ++k)
          for (int j = jl; j <= ju; ++j) {
            int kf = ks + 2 * (k - kl), jf = js + 2 * (j - jl);
            double el1 = dx2[jf], el2 = dx2[jf + 1];
            EA(E[1], k, j, p, 1) += (EA(S[1], kf, jf, ps, 1) * el1 +
                                     EA(S[1], kf, jf + 1, ps, 1) * el2) / (el1 + el2);
          }
        for (int k = kl; k <= ku; ++k)
          for (int j = jl; j <= ju + 1; ++j) {
            int kf = ks + 2 * (k - kl), jf = js + 2 * (j - jl);
            double el1 = dx3[kf], el2 = dx3[kf + 1];
            EA(E[2], k, j, p, 2) += (EA(S[2], kf, jf, ps, 2) * el1 +
                                     EA(S[2], kf + 1, jf, ps, 2) * el2) / (el1 + el2);
          }
      } else if (ax == 1) {
        int il = is, iu = ie, kl = ks, ku = ke;
        if (q->fi1 == 0) iu = is + nx1 / 2 - 1; else il = is + nx1 / 2;
        if (q->fi2 == 0) ku = ks + nx3 / 2 - 1; else kl = ks + nx3 / 2;
        for (int k = kl; k <= ku + 1; ++k)
          for (int i = il; i <= iu; ++i) {
            int kf = ks + 2 * (k - kl), iff = is + 2 * (i - il);
            double l1 = dx1[iff], l2 = dx1[iff + 1];
            EA(E[0], k, p, i, 0) += (EA(S[0], kf, ps, iff, 0) * l1 +
                                     EA(S[0], kf, ps, iff + 1, 0) * l2) / (l1 + l2);
          }
        for (int k = kl; k <= ku; ++k)
          for (int i = il; i <= iu + 1; ++i) {
            int kf = ks + 2 * (k - kl), iff = is + 2 * (i - il);
            double l1 = dx3[kf], l2 = dx3[kf + 1];
            EA(E[2], k, p, i, 2) += (EA(S[2], kf, ps, iff, 2) * l1 +
                                     EA(S[2], kf + 1, ps, iff, 2) * l2) / (l1 + l2);
          }
      } else {
        int il = is, iu = ie, jl = js, ju = je;
        if (q->fi1 == 0) iu = is + nx1 / 2 - 1; else il = is + nx1 / 2;
        if (q->fi2 == 0) ju = js + nx2 / 2 - 1; else jl = js + nx2 / 2;
        for (int j = jl; j <= ju + 1; ++j)
          for (int i = il; i <= iu; ++i) {
            int jf = js + 2 * (j - jl), iff = is + 2 * (i - il);
            double l1 = dx1[iff], l2 = dx1[iff + 1];
            EA(E[0], p, j, i, 0) += (EA(S[0], ps, jf, iff, 0) * l1 +
                                     EA(S[0], ps, jf, iff + 1, 0) * l2) / (l1 + l2);
          }
        for (int j = jl; j <= ju; ++j)
          for (int i = il; i <= iu + 1; ++i) {
            int jf = js + 2 * (j - jl), iff = is + 2 * (i - il);
            double l1 = dx2[jf], l2 = dx2[jf + 1];
            EA(E[1], p, j, i, 1) += (EA(S[1], ps, jf, iff, 1) * l1 +
                                     EA(S[1], ps, jf + 1, iff, 1) * l2) / (l1 + l2);
          }
      }
    } else {
      int p1, p2, s1, s2;
      edge_pos(m, q->eid, &p1, &p2);
      edge_pos(m, qs->eid, &s1, &s2);
      if (q->eid < 4) {
        int kl = ks, ku = ke;
        if (q->fi1 == 0) ku = ks + nx3 / 2 - 1; else kl = ks + nx3 / 2;
        for (int k = kl; k <= ku; ++k) {
          int kf = ks + 2 * (k - kl);
          double l1 = dx3[kf], l2 = dx3[kf + 1];
          EA(E[2], k, p2, p1, 2) += (EA(S[2], kf, s2, s1, 2) * l1 +
                                     EA(S[2], kf + 1, s2, s1, 2) * l2) / (l1 + l2);
        }
      } else if (q->eid < 8) {
        int jl = js, ju = je;
        if (q->fi1 == 0) ju = js + nx2 / 2 - 1; else jl = js + nx2 / 2;
        for (int j = jl; j <= ju; ++j) {
          int jf = js + 2 * (j - jl);
          double l1 = dx2[jf], l2 = dx2[jf + 1];
          EA(E[1], p2, j, p1, 1) += (EA(S[1], s2, jf, s1, 1) * l1 +
                                     EA(S[1], s2, jf + 1, s1, 1) * l2) / (l1 + l2);
        }
      } else {
        int il = is, iu = ie;
        if (q->fi1 == 0) iu = is + nx1 / 2 - 1; else il = is + nx1 / 2;
        for (int i = il; i <= iu; ++i) {
          int iff = is + 2 * (i - il);
          double l1 = dx1[iff], l2 = dx1[iff + 1];
          EA(E[0], p2, p1, i, 0) += (EA(S[0], s2, s1, iff, 0) * l1 +
                                     EA(S[0], s2, s1, iff + 1, 0) * l2) / (l1 + l2);
        }
      }
    }
  }
  /* AverageFluxBoundary (flux_correction_fc.cpp:1355-1545) */
  for (int f = 0; f < 6; ++f) {
    int o[3] = {0, 0, 0};
    o[f >> 1] = (f & 1) ? 1 : -1;
    int nl = NBL(ml, b, o[0], o[1], o[2]);
    if (nl < 0) continue;   /* a physical mesh face */
    int p = face_pos(m, f);
    if (nl == lev) {
      if (f < 2) {
        for (int k = ks + 1; k <= ke; ++k)
          for (int j = js; j <= je; ++j) EA(E[1], k, j, p, 1) *= 0.5;
        for (int k = ks; k <= ke; ++k)
          for (int j = js + 1; j <= je; ++j) EA(E[2], k, j, p, 2) *= 0.5;
      } else if (f < 4) {
        for (int k = ks + 1; k <= ke; ++k)
          for (int i = is; i <= ie; ++i) EA(E[0], k, p, i, 0) *= 0.5;
        for (int k = ks; k <= ke; ++k)
          for (int i = is + 1; i <= ie; ++i) EA(E[2], k, p, i, 2) *= 0.5;
      } else {
        for (int j = js + 1; j <= je; ++j)
          for (int i = is; i <= ie; ++i) EA(E[0], p, j, i, 0) *= 0.5;
        for (int j = js; j <= je; ++j)
          for (int i = is + 1; i <= ie; ++i) EA(E[1], p, j, i, 1) *= 0.5;
      }
    } else if (nl > lev) {
      if (f < 2) {
        int k = ks + nx3 / 2;
        for (int j = js; j <= je; ++j) EA(E[1], k, j, p, 1) *= 0.5;
        int j = js + nx2 / 2;
        for (int kk = ks; kk <= ke; ++kk) EA(E[2], kk, j, p, 2) *= 0.5;
      } else if (f < 4) {
        int k = ks + nx3 / 2;
        for (int i = is; i <= ie; ++i) EA(E[0], k, p, i, 0) *= 0.5;
        int i = is + nx1 / 2;
        for (int kk = ks; kk <= ke; ++kk) EA(E[2], kk, p, i, 2) *= 0.5;
      } else {
        int j = js + nx2 / 2;
        for (int i = is; i <= ie; ++i) EA(E[0], p, j, i, 0) *= 0.5;
        int i = is + nx1 / 2;
        for (int jj = js; jj <= je; ++jj) EA(E[1], p, jj, i, 1) *= 0.5;
      }
    }
  }
  for (int eid = 0; eid < 12; ++eid) {
    int nf = ml->nedge_fine[b * 12 + eid];
    if (nf == 1) continue;
    double div = 1.0 / (double)nf;
    int p1, p2;
    edge_pos(m, eid, &p1, &p2);
    if (eid < 4) for (int k = ks; k <= ke; ++k) EA(E[2], k, p2, p1, 2) *= div;
    else if (eid < 8) for (int j = js; j <= je; ++j) EA(E[1], p2, j, p1, 1) *= div;
    else for (int i = is; i <= ie; ++i) EA(E[0], p2, p1, i, 0) *= div;
  }
}

/* ---- prolongation of the ghost zones next to coarser blocks --------------------------- */

/* physical boundary function of face f (0..5, kind 1 outflow / 2 reflecting) on the
 * primitive array p[5] and the face field fb[3], over the transverse ranges t (index =
 * axis) with ng ghost layers beyond the own range [lo, hi] of the normal axis
 * (outflow_cc.cpp, reflect_hydro.cpp, outflow_fc.cpp, reflect_fc.cpp) */
static void bc_face_views(view3 p[NHYDRO], view3 fb[3], int f, int kind, int lo, int hi,
                          const int ts[3], const int te[3], int ng) {
  int a = f >> 1, side = f & 1;
  int c[3];
  for (int g = 1; g <= ng; ++g) {
    int dst = side ? hi + g : lo - g;
    int src = (kind == 1) ? (side ? hi : lo) : (side ? hi - g + 1 : lo + g - 1);
    for (int n = 0; n < NHYDRO; ++n) {
      int flip = (kind == 2 && n == IVX + a);
      int r0[3], r1[3];
      for (int d = 0; d < 3; ++d) { r0[d] = ts[d]; r1[d] = te[d]; }
      r0[a] = r1[a] = dst;
      for (c[2] = r0[2]; c[2] <= r1[2]; ++c[2])
        for (c[1] = r0[1]; c[1] <= r1[1]; ++c[1])
          for (c[0] = r0[0]; c[0] <= r1[0]; ++c[0]) {
            int s3[3] = {c[0], c[1], c[2]};
            s3[a] = src;
            double v = *V(p[n], s3[2], s3[1], s3[0]);
            *V(p[n], c[2], c[1], c[0]) = flip ? -v : v;
          }
    }
    for (int d = 0; d < 3; ++d) {
      int fdst, fsrc, flip = 0;
      if (d == a) {
        fdst = side ? hi + 1 + g : lo - g;
        fsrc = (kind == 1) ? (side ? hi + 1 : lo) : (side ? hi + 1 - g : lo + g);
        flip = (kind == 2);
      } else {
        fdst = dst;
        fsrc = src;
      }
      int r0[3], r1[3];
      for (int e = 0; e < 3; ++e) { r0[e] = ts[e]; r1[e] = te[e]; }
      if (d != a) r1[d] += 1;
      r0[a] = r1[a] = fdst;
      for (c[2] = r0[2]; c[2] <= r1[2]; ++c[2])
        for (c[1] = r0[1]; c[1] <= r1[1]; ++c[1])
          for (c[0] = r0[0]; c[0] <= r1[0]; ++c[0]) {
            int s3[3] = {c[0], c[1], c[2]};
            s3[a] = fsrc;
            double v = *V(fb[d], s3[2], s3[1], s3[0]);
            *V(fb[d], c[2], c[1], c[0]) = flip ? -v : v;
          }
    }
  }
}

/* W(U) of adiabatic MHD (adiabatic_mhd.cpp:41-90) with the cell-centred field
 * (field.cpp:112-180) on the coarse buffers of block b over box c */
static void ml_c2p_coarse(orc_mesh *m, int b, box3 c) {
  orc_ml *ml = m->ml;
  double gm1 = m->p.gamma - 1.0, dfl = m->p.dfloor, pfl = m->p.pfloor;
  double *u = ml->ccons + (long)b * NHYDRO * ml->nccell;
  double *w = ml->cprim + (long)b * NHYDRO * ml->nccell;
  double *bc = ml->cbcc + (long)b * 3 * ml->nccell;
  const double *b1 = ml->cb1 + (long)b * ml->ncf1, *b2 = ml->cb2 + (long)b * ml->ncf2,
               *b3 = ml->cb3 + (long)b * ml->ncf3;
  long nc = ml->nccell;
  for (int k = c.s[2]; k <= c.e[2]; ++k)
    for (int j = c.s[1]; j <= c.e[1]; ++j)
      for (int i = c.s[0]; i <= c.e[0]; ++i) {
        long q = CCI(ml, 0, k, j, i);
        double lw = 0.5, rw = 0.5;
        bc[q] = lw * b1[CF1(ml, k, j, i)] + rw * b1[CF1(ml, k, j, i + 1)];
        bc[q + nc] = lw * b2[CF2(ml, k, j, i)] + rw * b2[CF2(ml, k, j + 1, i)];
        bc[q + 2 * nc] = lw * b3[CF3(ml, k, j, i)] + rw * b3[CF3(ml, k + 1, j, i)];
      }
  for (int k = c.s[2]; k <= c.e[2]; ++k)
    for (int j = c.s[1]; j <= c.e[1]; ++j)
      for (int i = c.s[0]; i <= c.e[0]; ++i) {
        long q = CCI(ml, 0, k, j, i);
        double *u_d = &u[q], *u_e = &u[q + 4 * nc];
        double u_m1 = u[q + nc], u_m2 = u[q + 2 * nc], u_m3 = u[q + 3 * nc];
        *u_d = (*u_d > dfl) ? *u_d : dfl;
        w[q] = *u_d;
        double di = 1.0 / *u_d;
        w[q + nc] = u_m1 * di;
        w[q + 2 * nc] = u_m2 * di;
        w[q + 3 * nc] = u_m3 * di;
        double bcc1 = bc[q], bcc2 = bc[q + nc], bcc3 = bc[q + 2 * nc];
        double pb = 0.5 * (SQR(bcc1) + SQR(bcc2) + SQR(bcc3));
        double e_k = 0.5 * di * (SQR(u_m1) + SQR(u_m2) + SQR(u_m3));
        double w_p = gm1 * (*u_e - e_k - pb);
        *u_e = (w_p > pfl) ? *u_e : ((pfl / gm1) + e_k + pb);
        w[q + 4 * nc] = (w_p > pfl) ? w_p : pfl;
      }
}

/* minmod gradient of the prolongation (mesh_refinement.cpp:525-536) */
static inline double mm_grad(double cm, double c0, double cp, double dxm, double dxp) {
  double gm = (c0 - cm) / dxm, gp = (cp - c0) / dxp;
  return 0.5 * (SIGN(gm) + SIGN(gp)) * smin(fabs(gm), fabs(gp));
}

/* ProlongateCellCenteredValues (mesh_refinement.cpp:464-540), 3-D */
static void prolong_cc(const orc_mesh *m, int b, view3 coarse, view3 fine, box3 c) {
  const orc_ml *ml = m->ml;
  const double *cx1 = ml->cx1v + (long)b * ml->ncc1, *cx2 = ml->cx2v + (long)b * ml->ncc2,
               *cx3 = ml->cx3v + (long)b * ml->ncc3;
  const double *fx1 = m->x1v + (long)b * m->nc1, *fx2 = m->x2v + (long)b * m->nc2,
               *fx3 = m->x3v + (long)b * m->nc3;
  for (int k = c.s[2]; k <= c.e[2]; ++k) {
    int fk = (k - ml->cks) * 2 + m->ks;
    double x3c = cx3[k], dx3m = x3c - cx3[k - 1], dx3p = cx3[k + 1] - x3c;
    double dx3fm = x3c - fx3[fk], dx3fp = fx3[fk + 1] - x3c;
    for (int j = c.s[1]; j <= c.e[1]; ++j) {
      int fj = (j - ml->cjs) * 2 + m->js;
      double x2c = cx2[j], dx2m = x2c - cx2[j - 1], dx2p = cx2[j + 1] - x2c;
      double dx2fm = x2c - fx2[fj], dx2fp = fx2[fj + 1] - x2c;
      for (int i = c.s[0]; i <= c.e[0]; ++i) {
        int fi = (i - ml->cis) * 2 + m->is;
        double x1c = cx1[i], dx1m = x1c - cx1[i - 1], dx1p = cx1[i + 1] - x1c;
        double dx1fm = x1c - fx1[fi], dx1fp = fx1[fi + 1] - x1c;
        double cc = *V(coarse, k, j, i);
        double g1 = mm_grad(*V(coarse, k, j, i - 1), cc, *V(coarse, k, j, i + 1), dx1m, dx1p);
        double g2 = mm_grad(*V(coarse, k, j - 1, i), cc, *V(coarse, k, j + 1, i), dx2m, dx2p);
        double g3 = mm_grad(*V(coarse, k - 1, j, i), cc, *V(coarse, k + 1, j, i), dx3m, dx3p);
        *V(fine, fk, fj, fi) = cc - (g1 * dx1fm + g2 * dx2fm + g3 * dx3fm);
        *V(fine, fk, fj, fi + 1) = cc + (g1 * dx1fp - g2 * dx2fm - g3 * dx3fm);
        *V(fine, fk, fj + 1, fi) = cc - (g1 * dx1fm - g2 * dx2fp + g3 * dx3fm);
        *V(fine, fk, fj + 1, fi + 1) = cc + (g1 * dx1fp + g2 * dx2fp - g3 * dx3fm);
        *V(fine, fk + 1, fj, fi) = cc - (g1 * dx1fm + g2 * dx2fm - g3 * dx3fp);
        *V(fine, fk + 1, fj, fi + 1) = cc + (g1 * dx1fp - g2 * dx2fm + g3 * dx3fp);
        *V(fine, fk + 1, fj + 1, fi) = cc - (g1 * dx1fm - g2 * dx2fp - g3 * dx3fp);
        *V(fine, fk + 1, fj + 1, fi + 1) = cc + (g1 * dx1fp + g2 * dx2fp + g3 * dx3fp);
      }
    }
  }
}

/* ProlongateSharedFieldX1/X2/X3, Cartesian branches (mesh_refinement.cpp:829-870,
 * 974-1012, 1118-1156): the fine faces lying in a coarse face, from the coarse face value
 * and its minmod slopes along the face (x?s? = x?v in Cartesian coordinates,
 * cartesian.cpp) */
static void prolong_shared(const orc_mesh *m, int b, int d, view3 coarse, view3 fine,
                           box3 c) {
  const orc_ml *ml = m->ml;
  const double *cx[3] = {ml->cx1v + (long)b * ml->ncc1, ml->cx2v + (long)b * ml->ncc2,
                         ml->cx3v + (long)b * ml->ncc3};
  const double *fx[3] = {m->x1v + (long)b * m->nc1, m->x2v + (long)b * m->nc2,
                         m->x3v + (long)b * m->nc3};
  int clo[3] = {ml->cis, ml->cjs, ml->cks}, flo[3] = {m->is, m->js, m->ks};
  int ta = (d == 0) ? 1 : 0, tb = (d == 2) ? 1 : 2;   /* the two in-face axes */
  int cidx[3];
  for (cidx[2] = c.s[2]; cidx[2] <= c.e[2]; ++cidx[2])
    for (cidx[1] = c.s[1]; cidx[1] <= c.e[1]; ++cidx[1])
      for (cidx[0] = c.s[0]; cidx[0] <= c.e[0]; ++cidx[0]) {
        int f[3];
        for (int a = 0; a < 3; ++a) f[a] = (cidx[a] - clo[a]) * 2 + flo[a];
        double cc = *V(coarse, cidx[2], cidx[1], cidx[0]);
        double g[3], am[3], ap[3];
        for (int t = 0; t < 2; ++t) {
          int a = t ? tb : ta;
          int mi[3] = {cidx[0], cidx[1], cidx[2]}, pi[3] = {cidx[0], cidx[1], cidx[2]};
          mi[a]--; pi[a]++;
          double xc = cx[a][cidx[a]];
          g[a] = mm_grad(*V(coarse, mi[2], mi[1], mi[0]), cc, *V(coarse, pi[2], pi[1], pi[0]),
                         xc - cx[a][cidx[a] - 1], cx[a][cidx[a] + 1] - xc);
          am[a] = xc - fx[a][f[a]];      /* (x_c - fx_m) */
          ap[a] = fx[a][f[a] + 1] - xc;  /* (fx_p - x_c) */
        }
        /* fine faces (ta offset, tb offset): -,- ; +,- ; -,+ ; +,+ with the reference's
         * term order (first in-face axis, then second) */
        for (int ob = 0; ob < 2; ++ob)
          for (int oa = 0; oa < 2; ++oa) {
            int ff[3] = {f[0], f[1], f[2]};
            ff[ta] += oa; ff[tb] += ob;
            double ta_t = oa ? g[ta] * ap[ta] : g[ta] * am[ta];
            double tb_t = ob ? g[tb] * ap[tb] : g[tb] * am[tb];
            double v = cc;
            v = oa ? v + ta_t : v - ta_t;
            v = ob ? v + tb_t : v - tb_t;
            *V(fine, ff[2], ff[1], ff[0]) = v;
          }
      }
}

/* ProlongateInternalField (mesh_refinement.cpp:1223-1300), 3-D: the fine faces inside a
 * coarse cell from the shared faces around it, divergence-free (Toth & Roe 2002) */
static void prolong_internal(const orc_mesh *m, int b, view3 x1f, view3 x2f, view3 x3f,
                             box3 c) {
  const orc_ml *ml = m->ml;
  const double *dx1 = m->dx1f + (long)b * m->nc1, *dx2 = m->dx2f + (long)b * m->nc2,
               *dx3 = m->dx3f + (long)b * m->nc3;
  for (int k = c.s[2]; k <= c.e[2]; ++k) {
    int fk = (k - ml->cks) * 2 + m->ks;
    for (int j = c.s[1]; j <= c.e[1]; ++j) {
      int fj = (j - ml->cjs) * 2 + m->js;
      for (int i = c.s[0]; i <= c.e[0]; ++i) {
        int fi = (i - ml->cis) * 2 + m->is;
#define A1(kk, jj) (dx2[fj + (jj)] * dx3[fk + (kk)])          /* Face1Area(fk+kk, fj+jj) */
#define A2(kk, ii) (dx1[(ii)] * dx3[fk + (kk)])               /* Face2Area(fk+kk, .)(ii) */
#define A3(jj, ii) (dx1[(ii)] * dx2[fj + (jj)])               /* Face3Area(., fj+jj)(ii) */
        double Uxx = 0.0, Vyy = 0.0, Wzz = 0.0, Uxyz = 0.0, Vxyz = 0.0, Wxyz = 0.0;
        for (int jj = 0; jj < 2; ++jj) {
          double sj = (double)(2 * jj - 1);
          int fjj = fj + jj, fjp = fj + 2 * jj;
          for (int ii = 0; ii < 2; ++ii) {
            double si = (double)(2 * ii - 1);
            int fii = fi + ii, fip = fi + 2 * ii;
            double x2lo = *V(x2f, fk, fjp, fii) * A2(0, fii);
            double x2hi = *V(x2f, fk + 1, fjp, fii) * A2(1, fii);
            double x3lo = *V(x3f, fk, fjj, fii) * A3(jj, fii);
            double x3hi = *V(x3f, fk + 2, fjj, fii) * A3(jj, fii);
            double x1lo = *V(x1f, fk, fjj, fip) * A1(0, jj);
            double x1hi = *V(x1f, fk + 1, fjj, fip) * A1(1, jj);
            Uxx += si * (sj * (x2lo + x2hi) + (x3hi - x3lo));
            Vyy += sj * ((x3hi - x3lo) + si * (x1lo + x1hi));
            Wzz += si * (x1hi - x1lo) + sj * (x2hi - x2lo);
            Uxyz += (si * sj) * (x1hi - x1lo);
            Vxyz += (si * sj) * (x2hi - x2lo);
            Wxyz += (si * sj) * (x3hi - x3lo);
          }
        }
        double Sdx1 = SQR(dx1[fi] + dx1[fi + 1]);
        double Sdx2 = SQR(dx2[fj] + dx2[fj + 1]);
        double Sdx3 = SQR(dx3[fk] + dx3[fk + 1]);
        Uxx *= 0.125; Vyy *= 0.125; Wzz *= 0.125;
        Uxyz *= 0.125 / (Sdx2 + Sdx3);
        Vxyz *= 0.125 / (Sdx1 + Sdx3);
        Wxyz *= 0.125 / (Sdx1 + Sdx2);
        for (int kk = 0; kk < 2; ++kk)
          for (int jj = 0; jj < 2; ++jj) {
            double a = A1(kk, jj);
            double v = 0.5 * (*V(x1f, fk + kk, fj + jj, fi) * a +
                              *V(x1f, fk + kk, fj + jj, fi + 2) * a) + Uxx;
            v = kk ? v + Sdx3 * Vxyz : v - Sdx3 * Vxyz;
            v = jj ? v + Sdx2 * Wxyz : v - Sdx2 * Wxyz;
            *V(x1f, fk + kk, fj + jj, fi + 1) = v / a;
          }
        for (int kk = 0; kk < 2; ++kk)
          for (int ii = 0; ii < 2; ++ii) {
            double v = 0.5 * (*V(x2f, fk + kk, fj, fi + ii) * A2(kk, fi + ii) +
                              *V(x2f, fk + kk, fj + 2, fi + ii) * A2(kk, fi + ii)) + Vyy;
            v = kk ? v + Sdx3 * Uxyz : v - Sdx3 * Uxyz;
            v = ii ? v + Sdx1 * Wxyz : v - Sdx1 * Wxyz;
            *V(x2f, fk + kk, fj + 1, fi + ii) = v / A2(kk, fi + ii);
          }
        for (int jj = 0; jj < 2; ++jj)
          for (int ii = 0; ii < 2; ++ii) {
            double v = 0.5 * (*V(x3f, fk + 2, fj + jj, fi + ii) * A3(jj, fi + ii) +
                              *V(x3f, fk, fj + jj, fi + ii) * A3(jj, fi + ii)) + Wzz;
            v = jj ? v + Sdx2 * Uxyz : v - Sdx2 * Uxyz;
            v = ii ? v + Sdx1 * Vxyz : v - Sdx1 * Vxyz;
            *V(x3f, fk + 1, fj + jj, fi + ii) = v / A3(jj, fi + ii);
          }
#undef A1
#undef A2
#undef A3
      }
    }
  }
}

/* RestrictGhostCellsOnSameLevel (bvals_refine.cpp:262-352): the ghost cells and faces
 * that same-level neighbours filled, restricted into the coarse buffers around the
 * prolongation region of neighbour q; (ni, nj, nk) = the neighbour direction */
static void ml_restrict_ghost_same(orc_mesh *m, int b, const ml_nbr *q, int ni, int nj,
                                   int nk) {
  orc_ml *ml = m->ml;
  int lev = ml_level(m, b);
  int clo[3] = {ml->cis, ml->cjs, ml->cks}, chi[3] = {ml->cie, ml->cje, ml->cke};
  int o[3] = {q->ox1, q->ox2, q->ox3}, nn[3] = {ni, nj, nk};
  box3 r;
  for (int a = 0; a < 3; ++a) {
    if (nn[a] == 0) {
      r.s[a] = clo[a]; r.e[a] = chi[a];
      if (o[a] == 1) r.s[a] = chi[a];
      else if (o[a] == -1) r.e[a] = clo[a];
    } else if (nn[a] == 1) {
      r.s[a] = r.e[a] = chi[a] + 1;
    } else {
      r.s[a] = r.e[a] = clo[a] - 1;
    }
  }
  for (int v = 0; v < NHYDRO; ++v)
    restrict_cc(m, b, fine_cc(m, m->u, b, NHYDRO, v), coarse_cc(ml, ml->ccons, b, NHYDRO, v), r);
  double *fb[3] = {m->b1, m->b2, m->b3}, *cfb[3] = {ml->cb1, ml->cb2, ml->cb3};
  for (int d = 0; d < 3; ++d) {
    box3 rf = r;
    int rs = r.s[d], re = r.e[d] + 1;
    int om[3] = {ni, nj, nk}, op[3] = {ni, nj, nk};
    om[d] -= 1; op[d] += 1;
    if (rs == clo[d] && NBL(ml, b, om[0], om[1], om[2]) < lev) rs++;
    if (re == chi[d] + 1 && NBL(ml, b, op[0], op[1], op[2]) < lev) re--;
    rf.s[d] = rs; rf.e[d] = re;
    restrict_fc(m, b, d, fine_fc(m, d, fb[d], b), coarse_fc(ml, d, cfb[d], b), rf);
  }
}

/* BoundaryValues::ProlongateBoundaries (bvals_refine.cpp:97-256) for block b: for every
 * coarser neighbour in list order, restrict the same-level ghost-ghost zone, form the
 * coarse primitives (W(U) on the coarse buffer) and apply the physical boundaries on the
 * coarse level, prolongate the primitives into w and the face field, then the
 * cell-centred field and U(W) of the filled fine ghost cells (ProlongateGhostCells,
 * :512-637) */
static void ml_prolongate_block(orc_mesh *m, int b, double *w) {
  orc_ml *ml = m->ml;
  int lev = ml_level(m, b);
  int clo[3] = {ml->cis, ml->cjs, ml->cks}, chi[3] = {ml->cie, ml->cje, ml->cke};
  int flo[3] = {m->is, m->js, m->ks};
  int cn = ml->cng - 1;
  for (int n = 0; n < ml->nnbr[b]; ++n) {
    const ml_nbr *q = ml_nb(m, b, n);
    if (q->level >= lev) continue;
    int o[3] = {q->ox1, q->ox2, q->ox3};
    int ns[3], ne[3];
    for (int a = 0; a < 3; ++a) {
      ns[a] = (o[a] - 1 > -1) ? o[a] - 1 : -1;
      ne[a] = (o[a] + 1 < 1) ? o[a] + 1 : 1;
    }
    for (int nk = ns[2]; nk <= ne[2]; ++nk)
      for (int nj = ns[1]; nj <= ne[1]; ++nj)
        for (int ni = ns[0]; ni <= ne[0]; ++ni) {
          int ntype = abs(ni) + abs(nj) + abs(nk);
          if (ntype == 0 || NBL(ml, b, ni, nj, nk) != lev) continue;
          ml_restrict_ghost_same(m, b, q, ni, nj, nk);
        }
    box3 c;
    for (int a = 0; a < 3; ++a) {
      if (o[a] == 0) {
        c.s[a] = clo[a]; c.e[a] = chi[a];
        if ((ml_lx(m, b, a) & 1LL) == 0LL) c.e[a] += cn; else c.s[a] -= cn;
      } else if (o[a] > 0) { c.s[a] = chi[a] + 1; c.e[a] = chi[a] + cn; }
      else { c.s[a] = clo[a] - cn; c.e[a] = clo[a] - 1; }
    }
    /* ApplyPhysicalBoundariesOnCoarseLevel (bvals_refine.cpp:366-505) */
    box3 cx = c;
    for (int a = 0; a < 3; ++a) {
      int om[3] = {0, 0, 0}, op[3] = {0, 0, 0};
      om[a] = -1; op[a] = 1;
      int fm = 1, fp = 1;
      if (o[a] == 0) {
        fm = NBL(ml, b, om[0], om[1], om[2]) != -1;
        fp = NBL(ml, b, op[0], op[1], op[2]) != -1;
      }
      cx.s[a] -= fm; cx.e[a] += fp;
    }
    ml_c2p_coarse(m, b, cx);
    view3 pv[NHYDRO], fv[3];
    for (int v = 0; v < NHYDRO; ++v) pv[v] = coarse_cc(ml, ml->cprim, b, NHYDRO, v);
    fv[0] = coarse_fc(ml, 0, ml->cb1, b);
    fv[1] = coarse_fc(ml, 1, ml->cb2, b);
    fv[2] = coarse_fc(ml, 2, ml->cb3, b);
    for (int a = 0; a < 3; ++a) {
      if (o[a] != 0) continue;
      for (int side = 0; side < 2; ++side) {
        int od[3] = {0, 0, 0};
        od[a] = side ? 1 : -1;
        if (NBL(ml, b, od[0], od[1], od[2]) != -1) continue;  /* not a physical face */
        int ts[3], te[3];
        for (int d = 0; d < 3; ++d) { ts[d] = c.s[d]; te[d] = c.e[d]; }
        ts[a] = clo[a]; te[a] = chi[a];
        bc_face_views(pv, fv, 2 * a + side, m->p.bc[2 * a + side], clo[a], chi[a], ts, te,
                      m->p.ng);
      }
    }
    /* ProlongateGhostCells */
    for (int v = 0; v < NHYDRO; ++v)
      prolong_cc(m, b, coarse_cc(ml, ml->cprim, b, NHYDRO, v), fine_cc(m, w, b, NHYDRO, v), c);
    double *fb[3] = {m->b1, m->b2, m->b3}, *cfb[3] = {ml->cb1, ml->cb2, ml->cb3};
    for (int d = 0; d < 3; ++d) {
      box3 cf = c;
      int lo = c.s[d], hi = c.e[d] + 1;
      int om[3] = {o[0], o[1], o[2]}, op[3] = {o[0], o[1], o[2]};
      om[d] -= 1; op[d] += 1;
      if (o[d] >= 0 && NBL(ml, b, om[0], om[1], om[2]) >= lev) lo++;
      if (o[d] <= 0 && NBL(ml, b, op[0], op[1], op[2]) >= lev) hi--;
      cf.s[d] = lo; cf.e[d] = hi;
      prolong_shared(m, b, d, coarse_fc(ml, d, cfb[d], b), fine_fc(m, d, fb[d], b), cf);
    }
    prolong_internal(m, b, fine_fc(m, 0, m->b1, b), fine_fc(m, 1, m->b2, b),
                     fine_fc(m, 2, m->b3, b), c);
    int fs[3], fe[3];
    for (int a = 0; a < 3; ++a) {
      fs[a] = (c.s[a] - clo[a]) * 2 + flo[a];
      fe[a] = (c.e[a] - clo[a]) * 2 + flo[a] + 1;
    }
    cell_centered_field(m, b, fs[0], fe[0], fs[1], fe[1], fs[2], fe[2]);
    /* PrimitiveToConserved, adiabatic_mhd.cpp:99-133 */
    double igm1 = 1.0 / (m->p.gamma - 1.0);
    double *ub = m->u + (long)b * NHYDRO * m->ncell;
    const double *wb = w + (long)b * NHYDRO * m->ncell;
    const double *bc = m->bcc + (long)b * 3 * m->ncell;
    long nc = m->ncell;
    for (int k = fs[2]; k <= fe[2]; ++k)
      for (int j = fs[1]; j <= fe[1]; ++j)
        for (int i = fs[0]; i <= fe[0]; ++i) {
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
}

/* ---- the multi-level stage and initialization ------------------------------------------ */

/* one stage on a multi-level mesh, the register averages of stage_weights */
static void ml_stage(orc_mesh *m, int stage) {
  const stage_w sw = stage_weights(m, stage);
  orc_ml *ml = m->ml;
  long nb = m->nb;
  if (stage == 1) {  /* StartupTaskList zeroes the registers */
    memset(m->u1, 0, sizeof(double) * nb * NHYDRO * m->ncell);
    memset(m->bb1, 0, sizeof(double) * nb * m->nf1);
    memset(m->bb2, 0, sizeof(double) * nb * m->nf2);
    memset(m->bb3, 0, sizeof(double) * nb * m->nf3);
  }
  const int order = sw.order;
  /* CalculateHydroFlux, CalculateEMF (corner EMFs into m->e1..e3) */
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < m->nb; ++b) {
    calculate_fluxes(m, b, order, &ml->sb[b]);
    corner_e(m, b, &ml->sb[b]);
  }
  /* SEND/RECV_HYDFLX: fluxes on faces shared with finer blocks */
  ml_flux_correction(m);
  /* IntegrateHydro (weighted_ave.cpp, add_flux_divergence.cpp) */
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < m->nb; ++b) {
    double *u = m->u + (long)b * NHYDRO * m->ncell;
    double *u1 = m->u1 + (long)b * NHYDRO * m->ncell;
    add_flux_divergence(m, b, sw.beta * m->dt, hydro_registers(m, &sw, u, u1), &ml->sb[b]);
  }
  /* SEND/RECV_FLDFLX (EMF correction) and IntegrateField */
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < m->nb; ++b) {
    scratch *s = &ml->sb[b];
    double *const f[3] = {m->bb1 + b * m->nf1, m->bb2 + b * m->nf2, m->bb3 + b * m->nf3};
    double *const g[3] = {m->b1 + b * m->nf1, m->b2 + b * m->nf2, m->b3 + b * m->nf3};
    field_registers(m, &sw, f, g);
    ml_emf_correct_block(m, b, s->e1, s->e2, s->e3);
    double *const *t = sw.swap ? f : g;
    ct_update(m, b, sw.beta * m->dt, t[0], t[1], t[2], s);
  }
  if (sw.swap) {
    SWAP(m->u, m->u1);
    SWAP(m->b1, m->bb1);
    SWAP(m->b2, m->bb2);
    SWAP(m->b3, m->bb3);
  }
  /* SEND/RECV/SETB_HYD and _FLD, PROLONG, CONS2PRIM, PHY_BVAL */
  ml_exchange(m, m->u, NHYDRO, ml->ccons, m->b1, m->b2, m->b3);
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < m->nb; ++b) ml_prolongate_block(m, b, m->w);
  all_con2prim(m, m->w1);
  SWAP(m->w, m->w1);
  all_bcs(m, m->w);
}

/* the body of Mesh::Initialize's loop (mesh.cpp:1674-1930): exchange of U and B,
 * ProlongateBoundaries, W(U) over the ranges the neighbour levels give, physical
 * boundaries */
void orc_ml_boundaries(orc_mesh *m) {
  ml_exchange(m, m->u, NHYDRO, m->ml->ccons, m->b1, m->b2, m->b3);
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < m->nb; ++b) ml_prolongate_block(m, b, m->w);
  all_con2prim(m, m->w);
  all_bcs(m, m->w);
}

static void ml_initialize(orc_mesh *m) {
  /* Mesh::Initialize (mesh.cpp:1698-1964): the boundaries, then the first dt */
  orc_ml_boundaries(m);
  all_new_dt(m);
}

static void ml_free(orc_ml *ml, int nb) {
  if (!ml) return;
  free(ml->nbr); free(ml->nnbr); free(ml->nblev); free(ml->loc); free(ml->edge_flag);
  free(ml->nedge_fine); free(ml->ccons); free(ml->cprim); free(ml->cbcc); free(ml->cb1);
  free(ml->cb2); free(ml->cb3); free(ml->cdx1f); free(ml->cdx2f); free(ml->cdx3f);
  free(ml->cx1v); free(ml->cx2v); free(ml->cx3v);
  if (ml->sb)
    for (int b = 0; b < nb; ++b) scratch_free(&ml->sb[b]);
  free(ml->sb);
  free(ml);
}

int orc_set_multilevel(orc_mesh *m, const int *nbr_table, const int *nbr_count,
                       const int *nblevel, const long long *loc, const double *cx1f,
                       const double *cdx1f, const double *cx2f, const double *cdx2f,
                       const double *cx3f, const double *cdx3f) {
  if (m->p.relativistic) return -1;  /* the multi-level path is Newtonian MHD only */
  if (m->p.ng % 2) return -2;        /* mesh refinement needs an even NGHOST */
  orc_ml *ml = calloc(1, sizeof(orc_ml));
  long nb = m->nb;
  ml->nbr = malloc(sizeof(ml_nbr) * nb * ML_MAXNB);
  ml->nnbr = malloc(sizeof(int) * nb);
  ml->nblev = malloc(sizeof(int) * nb * 27);
  ml->loc = malloc(sizeof(long long) * nb * 4);
  ml->edge_flag = malloc(sizeof(int) * nb * 12);
  ml->nedge_fine = malloc(sizeof(int) * nb * 12);
  for (long b = 0; b < nb; ++b) {
    ml->nnbr[b] = nbr_count[b];
    for (int n = 0; n < ML_MAXNB; ++n) {
      const int *t = nbr_table + (b * ML_MAXNB + n) * ML_NF;
      ml_nbr *q = &ml->nbr[b * ML_MAXNB + n];
      q->gid = t[0]; q->level = t[1]; q->ox1 = t[2]; q->ox2 = t[3]; q->ox3 = t[4];
      q->type = t[5]; q->fi1 = t[6]; q->fi2 = t[7]; q->fid = t[8]; q->eid = t[9];
    }
  }
  memcpy(ml->nblev, nblevel, sizeof(int) * nb * 27);
  memcpy(ml->loc, loc, sizeof(long long) * nb * 4);
  int ng = m->p.ng;
  ml->cng = (ng + 1) / 2 + 1;  /* meshblock.cpp:93 */
  ml->ncc1 = m->p.nx1 / 2 + 2 * ng; ml->ncc2 = m->p.nx2 / 2 + 2 * ng;
  ml->ncc3 = m->p.nx3 / 2 + 2 * ng;
  ml->cis = ng; ml->cie = ng + m->p.nx1 / 2 - 1;
  ml->cjs = ng; ml->cje = ng + m->p.nx2 / 2 - 1;
  ml->cks = ng; ml->cke = ng + m->p.nx3 / 2 - 1;
  ml->nccell = (long)ml->ncc1 * ml->ncc2 * ml->ncc3;
  ml->ncf1 = (long)ml->ncc3 * ml->ncc2 * (ml->ncc1 + 1);
  ml->ncf2 = (long)ml->ncc3 * (ml->ncc2 + 1) * ml->ncc1;
  ml->ncf3 = (long)(ml->ncc3 + 1) * ml->ncc2 * ml->ncc1;
  ml->ccons = calloc(nb * NHYDRO * ml->nccell, sizeof(double));
  ml->cprim = calloc(nb * NHYDRO * ml->nccell, sizeof(double));
  ml->cbcc = calloc(nb * 3 * ml->nccell, sizeof(double));
  ml->cb1 = calloc(nb * ml->ncf1, sizeof(double));
  ml->cb2 = calloc(nb * ml->ncf2, sizeof(double));
  ml->cb3 = calloc(nb * ml->ncf3, sizeof(double));
  ml->cdx1f = malloc(sizeof(double) * nb * ml->ncc1);
  ml->cdx2f = malloc(sizeof(double) * nb * ml->ncc2);
  ml->cdx3f = malloc(sizeof(double) * nb * ml->ncc3);
  ml->cx1v = malloc(sizeof(double) * nb * ml->ncc1);
  ml->cx2v = malloc(sizeof(double) * nb * ml->ncc2);
  ml->cx3v = malloc(sizeof(double) * nb * ml->ncc3);
  memcpy(ml->cdx1f, cdx1f, sizeof(double) * nb * ml->ncc1);
  memcpy(ml->cdx2f, cdx2f, sizeof(double) * nb * ml->ncc2);
  memcpy(ml->cdx3f, cdx3f, sizeof(double) * nb * ml->ncc3);
  /* x?v = 0.5*(x?f(i+1) + x?f(i)) of the coarse coordinates (cartesian.cpp:26-28) */
  for (long b = 0; b < nb; ++b) {
    for (int i = 0; i < ml->ncc1; ++i)
      ml->cx1v[b * ml->ncc1 + i] = 0.5 * (cx1f[b * (ml->ncc1 + 1) + i + 1] +
                                          cx1f[b * (ml->ncc1 + 1) + i]);
    for (int j = 0; j < ml->ncc2; ++j)
      ml->cx2v[b * ml->ncc2 + j] = 0.5 * (cx2f[b * (ml->ncc2 + 1) + j + 1] +
                                          cx2f[b * (ml->ncc2 + 1) + j]);
    for (int k = 0; k < ml->ncc3; ++k)
      ml->cx3v[b * ml->ncc3 + k] = 0.5 * (cx3f[b * (ml->ncc3 + 1) + k + 1] +
                                          cx3f[b * (ml->ncc3 + 1) + k]);
  }
  ml->sb = malloc(sizeof(scratch) * nb);
  for (long b = 0; b < nb; ++b) scratch_alloc(m, &ml->sb[b]);
  ml_free(m->ml, m->nb);
  m->ml = ml;
  m->ml_nblev = ml->nblev;
  for (int b = 0; b < m->nb; ++b) ml_count_fine_edges(m, b);
  return 0;
}

void orc_set_integrator(orc_mesh *m, int integrator) { m->integ = integrator; }

/* ---- adaptive refinement ---------------------------------------------------------------- */

/* The blast problem's refinement measure (pgen/blast.cpp:413-443, 3-D branch): per block
 * the maximum over the interior and one ghost layer of |grad p| / p from centred
 * differences of the current primitives. */
void orc_refine_eps(const orc_mesh *m, double *maxeps) {
#pragma omp parallel for schedule(static)
  for (int b = 0; b < m->nb; ++b) {
    const double *p = m->w + ((long)b * NHYDRO + IPR) * m->ncell;
    double mx = 0.0;
    for (int k = m->ks - 1; k <= m->ke + 1; ++k)
      for (int j = m->js - 1; j <= m->je + 1; ++j)
        for (int i = m->is - 1; i <= m->ie + 1; ++i) {
          double a = 0.5 * (p[CIDX(m, 0, k, j, i + 1)] - p[CIDX(m, 0, k, j, i - 1)]);
          double c = 0.5 * (p[CIDX(m, 0, k, j + 1, i)] - p[CIDX(m, 0, k, j - 1, i)]);
          double e = 0.5 * (p[CIDX(m, 0, k + 1, j, i)] - p[CIDX(m, 0, k - 1, j, i)]);
          double eps = sqrt(SQR(a) + SQR(c) + SQR(e)) / p[CIDX(m, 0, k, j, i)];
          mx = smax(mx, eps);
        }
    maxeps[b] = mx;
  }
}

/* Mesh::RedistributeAndRefineMeshBlocks on one rank (amr_loadbalance.cpp:351-660): fill
 * the new mesh d (multi-level tables already set) from the old mesh s.  Per new block n,
 * kind[n] 0: the old block newtoold[n] is kept (all its arrays move); 1: restriction of the
 * eight old children newtoold[n]..+7 into the block's octants (FillSameRankFineToCoarseAMR,
 * :827-946); 2: the old parent's U and B with a one-cell halo into the coarse buffers
 * (FillSameRankCoarseToFineAMR, :948-1030), the face-field corrections ffc[nffc][3] =
 * (new block, receiving face, old block) from old same-level neighbours
 * (ReceiveAndSetFaceFieldCorrection, :1387-1444), then ProlongateMeshBlock (:1172-1222).
 * The new blocks start from zero arrays, as newly constructed MeshBlocks do. */
int orc_regrid(orc_mesh *d, orc_mesh *s, const int *newtoold, const int *kind, int nffc,
               const int *ffc) {
  if (!d->ml || !s->ml || d->ncell != s->ncell) return -1;
  orc_ml *dm = d->ml, *sm = s->ml;
  const int hx[3] = {d->p.nx1 / 2, d->p.nx2 / 2, d->p.nx3 / 2};
  double *sfb[3] = {s->b1, s->b2, s->b3}, *dfb[3] = {d->b1, d->b2, d->b3};
  double *scb[3] = {sm->cb1, sm->cb2, sm->cb3}, *dcb[3] = {dm->cb1, dm->cb2, dm->cb3};
  long nfs[3] = {d->nf1, d->nf2, d->nf3};
  const int clo[3] = {dm->cis, dm->cjs, dm->cks}, chi[3] = {dm->cie, dm->cje, dm->cke};
  const int flo[3] = {d->is, d->js, d->ks}, fhi[3] = {d->ie, d->je, d->ke};
  for (int n = 0; n < d->nb; ++n) {
    int on = newtoold[n];
    if (kind[n] == 0) {
      memcpy(d->u + (long)n * NHYDRO * d->ncell, s->u + (long)on * NHYDRO * s->ncell,
             sizeof(double) * NHYDRO * d->ncell);
      memcpy(d->w + (long)n * NHYDRO * d->ncell, s->w + (long)on * NHYDRO * s->ncell,
             sizeof(double) * NHYDRO * d->ncell);
      memcpy(d->bcc + (long)n * 3 * d->ncell, s->bcc + (long)on * 3 * s->ncell,
             sizeof(double) * 3 * d->ncell);
      for (int a = 0; a < 3; ++a)
        memcpy(dfb[a] + n * nfs[a], sfb[a] + on * nfs[a], sizeof(double) * nfs[a]);
      /* the kept MeshBlock keeps its coarse buffers too */
      long ncc = dm->nccell, ncf[3] = {dm->ncf1, dm->ncf2, dm->ncf3};
      memcpy(dm->ccons + n * NHYDRO * ncc, sm->ccons + on * NHYDRO * ncc,
             sizeof(double) * NHYDRO * ncc);
      memcpy(dm->cprim + n * NHYDRO * ncc, sm->cprim + on * NHYDRO * ncc,
             sizeof(double) * NHYDRO * ncc);
      memcpy(dm->cbcc + n * 3 * ncc, sm->cbcc + on * 3 * ncc, sizeof(double) * 3 * ncc);
      for (int a = 0; a < 3; ++a)
        memcpy(dcb[a] + n * ncf[a], scb[a] + on * ncf[a], sizeof(double) * ncf[a]);
    } else if (kind[n] == 1) {
      for (int l = 0; l < 8; ++l) {
        int c = on + l;
        int o[3];
        for (int a = 0; a < 3; ++a) o[a] = flo[a] + (int)(ml_lx(s, c, a) & 1LL) * hx[a];
        box3 cb = {{clo[0], clo[1], clo[2]}, {chi[0], chi[1], chi[2]}};
        box3 db = {{o[0], o[1], o[2]}, {o[0] + hx[0] - 1, o[1] + hx[1] - 1, o[2] + hx[2] - 1}};
        for (int v = 0; v < NHYDRO; ++v) {
          view3 cv = coarse_cc(sm, sm->ccons, c, NHYDRO, v);
          restrict_cc(s, c, fine_cc(s, s->u, c, NHYDRO, v), cv, cb);
          copy_box(fine_cc(d, d->u, n, NHYDRO, v), db, cv, cb);
        }
        for (int a = 0; a < 3; ++a) {
          box3 cf = cb, df = db;
          cf.e[a] += 1; df.e[a] += 1;
          view3 cv = coarse_fc(sm, a, scb[a], c);
          restrict_fc(s, c, a, fine_fc(s, a, sfb[a], c), cv, cf);
          copy_box(fine_fc(d, a, dfb[a], n), df, cv, cf);
        }
      }
    } else {
      int o[3];
      for (int a = 0; a < 3; ++a)
        o[a] = (int)(ml_lx(d, n, a) & 1LL) * hx[a] + flo[a] - 1;
      box3 cb = {{clo[0] - 1, clo[1] - 1, clo[2] - 1}, {chi[0] + 1, chi[1] + 1, chi[2] + 1}};
      box3 sb = {{o[0], o[1], o[2]}, {o[0] + hx[0] + 1, o[1] + hx[1] + 1, o[2] + hx[2] + 1}};
      for (int v = 0; v < NHYDRO; ++v)
        copy_box(coarse_cc(dm, dm->ccons, n, NHYDRO, v), cb, fine_cc(s, s->u, on, NHYDRO, v),
                 sb);
      for (int a = 0; a < 3; ++a) {
        box3 cf = cb, sf = sb;
        cf.e[a] += 1; sf.e[a] += 1;
        copy_box(coarse_fc(dm, a, dcb[a], n), cf, fine_fc(s, a, sfb[a], on), sf);
      }
    }
  }
  /* face-field corrections: the receiving face of the child from the facing face of the
   * old same-level neighbour */
  for (int t = 0; t < nffc; ++t) {
    int n = ffc[3 * t], f = ffc[3 * t + 1], i = ffc[3 * t + 2], a = f >> 1;
    box3 rb = {{flo[0], flo[1], flo[2]}, {fhi[0], fhi[1], fhi[2]}}, sb = rb;
    rb.s[a] = rb.e[a] = (f & 1) ? fhi[a] + 1 : flo[a];
    sb.s[a] = sb.e[a] = (f & 1) ? flo[a] : fhi[a] + 1;
    copy_box(fine_fc(d, a, dfb[a], n), rb, fine_fc(s, a, sfb[a], i), sb);
  }
  for (int n = 0; n < d->nb; ++n) {
    if (kind[n] != 2) continue;
    int got[6] = {0, 0, 0, 0, 0, 0};
    for (int t = 0; t < nffc; ++t)
      if (ffc[3 * t] == n) got[ffc[3 * t + 1]] = 1;
    box3 c = {{clo[0], clo[1], clo[2]}, {chi[0], chi[1], chi[2]}};
    for (int v = 0; v < NHYDRO; ++v)
      prolong_cc(d, n, coarse_cc(dm, dm->ccons, n, NHYDRO, v), fine_cc(d, d->u, n, NHYDRO, v),
                 c);
    for (int a = 0; a < 3; ++a) {
      box3 cf = c;
      cf.e[a] += 1;
      if (got[2 * a]) cf.s[a]++;
      if (got[2 * a + 1]) cf.e[a]--;
      prolong_shared(d, n, a, coarse_fc(dm, a, dcb[a], n), fine_fc(d, a, dfb[a], n), cf);
    }
    prolong_internal(d, n, fine_fc(d, 0, d->b1, n), fine_fc(d, 1, d->b2, n),
                     fine_fc(d, 2, d->b3, n), c);
  }
  d->time = s->time;
  d->dt = s->dt;
  return 0;
}
