/*
 * fvs_oracle.c — CPU oracle: a C restatement of fvs2d's residual-and-update
 * loop, in the reference's source loop order and operation order.
 *
 * TEST INFRASTRUCTURE ONLY (see fvs_oracle.h).  Parity against the
 * reference's own numbers is UNPINNED (the Fortran reference cannot be
 * built here and ships no golden outputs); the oracle is pinned by the
 * reference's built-in known-answer checks, exercised in tests/.
 *
 * Conventions: arrays are 1-based like the Fortran (slot 0 unused), so that
 * every loop below reads like the routine it restates.  Variables are
 * indexed 0..3 = (rho,u,v,p) / (rho,rho*u,rho*v,rho*E).  Every floating
 * expression keeps the Fortran evaluation order (left-to-right for * / + -,
 * x**2 as x*x, x**3 as (x*x)*x); the file must be compiled with
 * -ffp-contract=off so that no multiply-add is fused.
 *
 * Deviations from the reference, each guarded and reported as an error
 * instead of undefined behaviour or a program stop:
 *  - compute_residual allocates un(bndry(2)%nedges) even with one boundary
 *    (src/residual.f90:110): the array is unused and not restated.
 *  - the dead cfl_max loop (src/residual.f90:169-173) is not restated.
 *  - a boundary whose edge count differs from its cell count is rejected:
 *    the reference pairs edge i with bndry%cell(i) (src/residual.f90:114-125).
 *  - a limiter with GG gradients reads the unallocated LSQ stencil
 *    (src/gradient_limiter.f90:54): rejected.
 *  - RK coefficients exist only for 4 stages (src/runge_kutta.f90:36-51) and
 *    SSP only for order 2 (:57-67): other combinations are rejected, except
 *    the SSP-RK3 extension below.
 *  - time_integ_RK_steady allocates diff twice (src/runge_kutta.f90:270,321),
 *    a runtime error in the reference: the norms are computed as intended.
 *  - solid_wall and unknown BC types stop the reference (:206-220): rejected.
 * Extensions (not in the reference, used by the synthetic benchmark cases):
 *  - doubly periodic meshes (minimum-image geometry), SSP-RK3 (Shu-Osher),
 *    a CFL-derived global dt for unsteady runs.
 */
#include "fvs_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NV 4
static const double PI = 3.141592653589793238462643383279502884; /* acos(-1.d0) */

/* ========================================================================= */
/* kd-tree: restatement of kdtree2 (src/kdtree2.f90), 2-D, double precision,
 * bucket 12, mean split, sorted n-nearest search.                           */
/* ========================================================================= */
#define KD_BUCKET 12
typedef struct { double lower, upper; } kd_iv;
typedef struct kd_node {
  int cut_dim;
  double cut_val, cut_val_left, cut_val_right;
  int l, u;
  struct kd_node *left, *right;
  kd_iv box[2];
} kd_node;
typedef struct {
  int n;
  const double* data; /* the_data(1:2,1:n) as data[2*(i-1)+k] */
  int* ind;           /* 1-based */
  kd_node* root;
} kd_tree;
typedef struct { double dis; int idx; } kd_res;
typedef struct {
  const double* qv;
  int nn, nfound;
  double ballsize;
  kd_res* elems; /* 1-based heap over results(1:nn) */
  int heap_size;
  const kd_tree* tp;
} kd_search;

#define KDV(tp, c, i) ((tp)->data[2 * ((i) - 1) + ((c) - 1)])

/* spread_in_coordinate, src/kdtree2.f90:934-981 */
static kd_iv kd_spread(const kd_tree* tp, int c, int l, int u) {
  double smin = KDV(tp, c, tp->ind[l]), smax = smin, lmin, lmax, t, last;
  int i;
  for (i = l + 2; i <= u; i += 2) {
    lmin = KDV(tp, c, tp->ind[i - 1]);
    lmax = KDV(tp, c, tp->ind[i]);
    if (lmin > lmax) { t = lmin; lmin = lmax; lmax = t; }
    if (smin > lmin) smin = lmin;
    if (smax < lmax) smax = lmax;
  }
  if (i == u + 1) {
    last = KDV(tp, c, tp->ind[u]);
    if (smin > last) smin = last;
    if (smax < last) smax = last;
  }
  kd_iv r = {smin, smax};
  return r;
}

/* select_on_coordinate_value, src/kdtree2.f90:840-899 */
static int kd_select_value(kd_tree* tp, int c, double alpha, int li, int ui) {
  int lb = li, rb = ui, tmp;
  while (lb < rb) {
    if (KDV(tp, c, tp->ind[lb]) <= alpha) {
      lb = lb + 1;
    } else {
      tmp = tp->ind[lb]; tp->ind[lb] = tp->ind[rb]; tp->ind[rb] = tmp;
      rb = rb - 1;
    }
  }
  return (KDV(tp, c, tp->ind[lb]) <= alpha) ? lb : lb - 1;
}

/* build_tree_for_range, src/kdtree2.f90:702-838 */
static kd_node* kd_build(kd_tree* tp, int l, int u, kd_node* parent) {
  if (u < l) return NULL;
  kd_node* res = (kd_node*)calloc(1, sizeof(kd_node));
  if ((u - l) <= KD_BUCKET) {
    for (int i = 1; i <= 2; i++) res->box[i - 1] = kd_spread(tp, i, l, u);
    res->cut_dim = 0; res->cut_val = 0.0; res->l = l; res->u = u;
    return res;
  }
  for (int i = 1; i <= 2; i++) {
    int recompute = 1;
    if (parent && i != parent->cut_dim) recompute = 0;
    res->box[i - 1] = recompute ? kd_spread(tp, i, l, u) : parent->box[i - 1];
  }
  /* maxloc: first maximum */
  int c = 1;
  if (res->box[1].upper - res->box[1].lower > res->box[0].upper - res->box[0].lower) c = 2;
  double s = 0.0;
  for (int k = l; k <= u; k++) s = s + KDV(tp, c, tp->ind[k]);
  double average = s / (double)(u - l + 1);
  res->cut_val = average;
  int m = kd_select_value(tp, c, average, l, u);
  res->cut_dim = c; res->l = l; res->u = u;
  res->left = kd_build(tp, l, m, res);
  res->right = kd_build(tp, m + 1, u, res);
  if (!res->right) {
    res->box[0] = res->left->box[0]; res->box[1] = res->left->box[1];
    res->cut_val_left = res->left->box[c - 1].upper;
    res->cut_val = res->cut_val_left;
  } else if (!res->left) {
    res->box[0] = res->right->box[0]; res->box[1] = res->right->box[1];
    res->cut_val_right = res->right->box[c - 1].lower;
    res->cut_val = res->cut_val_right;
  } else {
    res->cut_val_right = res->right->box[c - 1].lower;
    res->cut_val_left = res->left->box[c - 1].upper;
    res->cut_val = (res->cut_val_left + res->cut_val_right) / 2;
    for (int i = 0; i < 2; i++) {
      res->box[i].upper = fmax(res->left->box[i].upper, res->right->box[i].upper);
      res->box[i].lower = fmin(res->left->box[i].lower, res->right->box[i].lower);
    }
  }
  return res;
}

static void kd_free_node(kd_node* n) {
  if (!n) return;
  kd_free_node(n->left); kd_free_node(n->right); free(n);
}

/* pq_insert, src/kdtree2.f90:295-337 */
static double kd_pq_insert(kd_search* sr, double dis, int idx) {
  sr->heap_size = sr->heap_size + 1;
  int i = sr->heap_size;
  while (i > 1) {
    int isparent = i / 2;
    double parentdis = sr->elems[isparent].dis;
    if (dis > parentdis) {
      sr->elems[i] = sr->elems[isparent];
      i = isparent;
    } else break;
  }
  sr->elems[i].dis = dis; sr->elems[i].idx = idx;
  return sr->elems[1].dis;
}

/* pq_replace_max, src/kdtree2.f90:380-449 */
static double kd_pq_replace_max(kd_search* sr, double dis, int idx) {
  int N = sr->heap_size;
  if (N >= 1) {
    int parent = 1, child = 2;
    while (child <= N) {
      double prichild = sr->elems[child].dis;
      if (child < N) {
        double p1 = sr->elems[child + 1].dis;
        if (prichild < p1) { child = child + 1; prichild = p1; }
      }
      if (dis >= prichild) break;
      sr->elems[parent] = sr->elems[child];
      parent = child; child = 2 * parent;
    }
    sr->elems[parent].dis = dis; sr->elems[parent].idx = idx;
    return sr->elems[1].dis;
  }
  sr->elems[1].dis = dis; sr->elems[1].idx = idx;
  return dis;
}

/* process_terminal_node, src/kdtree2.f90:1494-1597 (rearranged data holds
 * the same numbers as the_data(:,ind(i)), so both branches agree) */
static void kd_terminal(kd_search* sr, const kd_node* node) {
  const kd_tree* tp = sr->tp;
  double ballsize = sr->ballsize;
  for (int i = node->l; i <= node->u; i++) {
    int indexofi = tp->ind[i];
    double sd = 0.0, d;
    d = KDV(tp, 1, indexofi) - sr->qv[0];
    sd = sd + d * d;
    if (sd > ballsize) continue;
    d = KDV(tp, 2, indexofi) - sr->qv[1];
    sd = sd + d * d;
    if (sd > ballsize) continue;
    if (sr->nfound < sr->nn) {
      sr->nfound = sr->nfound + 1;
      double newpri = kd_pq_insert(sr, sd, indexofi);
      if (sr->nfound == sr->nn) ballsize = newpri;
    } else {
      ballsize = kd_pq_replace_max(sr, sd, indexofi);
    }
  }
  sr->ballsize = ballsize;
}

static double kd_dis2_from_bnd(double x, double amin, double amax) {
  if (x > amax) return (x - amax) * (x - amax);
  if (x < amin) return (amin - x) * (amin - x);
  return 0.0;
}

/* search, src/kdtree2.f90:1367-1441 */
static void kd_search_node(kd_search* sr, const kd_node* node) {
  if (!(node->left && node->right)) { kd_terminal(sr, node); return; }
  int cut_dim = node->cut_dim;
  double qval = sr->qv[cut_dim - 1], dis;
  const kd_node *ncloser, *nfarther;
  if (qval < node->cut_val) {
    ncloser = node->left; nfarther = node->right;
    dis = (node->cut_val_right - qval) * (node->cut_val_right - qval);
  } else {
    ncloser = node->right; nfarther = node->left;
    dis = (node->cut_val_left - qval) * (node->cut_val_left - qval);
  }
  if (ncloser) kd_search_node(sr, ncloser);
  if (nfarther) {
    double ballsize = sr->ballsize;
    if (dis <= ballsize) {
      for (int i = 1; i <= 2; i++) {
        if (i != cut_dim) {
          dis = dis + kd_dis2_from_bnd(sr->qv[i - 1], node->box[i - 1].lower, node->box[i - 1].upper);
          if (dis > ballsize) return;
        }
      }
      kd_search_node(sr, nfarther);
    }
  }
}

/* heapsort_struct, src/kdtree2.f90:1830-1900 (a is 1-based) */
static void kd_heapsort(kd_res* a, int n) {
  if (n == 1) return;
  int ileft = n / 2 + 1, iright = n, i, j;
  kd_res value;
  for (;;) {
    if (ileft > 1) {
      ileft = ileft - 1;
      value = a[ileft];
    } else {
      value = a[iright];
      a[iright] = a[1];
      iright = iright - 1;
      if (iright == 1) { a[1] = value; return; }
    }
    i = ileft; j = 2 * ileft;
    while (j <= iright) {
      if (j < iright) { if (a[j].dis < a[j + 1].dis) j = j + 1; }
      if (value.dis < a[j].dis) { a[i] = a[j]; i = j; j = j + j; }
      else j = iright + 1;
    }
    a[i] = value;
  }
}

/* kdtree2_n_nearest with sort=.true., src/kdtree2.f90:1026-1067;
 * res is 1-based with room for nn entries; returns nfound */
static int kd_n_nearest(const kd_tree* tp, const double qv[2], int nn, kd_res* res) {
  kd_search sr;
  sr.qv = qv; sr.nn = nn; sr.nfound = 0; sr.ballsize = 1.79769313486231570815e+308; /* huge(1.d0) */
  sr.elems = res; sr.heap_size = 0; sr.tp = tp;
  kd_search_node(&sr, tp->root);
  if (nn > 1) kd_heapsort(res, nn);
  return sr.nfound;
}

/* ========================================================================= */
/* oracle state                                                              */
/* ========================================================================= */
struct orc {
  fvs_options o;
  double Lx, Ly;
  /* grid (1-based) */
  int nnodes, ntri, nquad, ncells;
  double *xn, *yn;
  int* nvrt;
  int (*cnode)[5];
  int (*nghbr)[5];
  int (*nghbre)[5];
  int (*cedge)[5];
  double *xc, *yc, *vol;
  double (*nrmlsign)[5];
  int *nd_nc, *nd_ptr, *nd_cell; /* node -> cells: cells of node v are nd_cell[nd_ptr[v] .. nd_ptr[v]+nd_nc[v]-1] */
  int nedges;
  int *en1, *en2, *ec1, *ec2;
  double *ex, *ey, *ea, *enx, *eny, *etx, *ety;
  int ncells_intr, ncells_bndr, *cell_intr, *cell_bndr;
  int nedges_intr, nedges_bndr, *edge_intr, *edge_bndr, *bedge_cell;
  double heff1, heff2, vol1, vol2;
  int nb;
  int *b_ncells, *b_nedges, *b_type, *b_cptr, *b_eptr, *b_cell, *b_edge; /* concatenated, 1-based ids */
  double* kd_xy;
  kd_tree tree;
  /* gradient operator */
  int st_len;
  int *st_ptr, *st_cell; /* CSR over cells (st_ptr 0-based offsets, size ncells+2) */
  double *st_coef, *st_w; /* lsq: coef [len][2], w [len]; ggcb: coefnb [len][2]; ggnb: coefnb [len] */
  double (*coef0)[2];
  double (*coefedg)[5][2];
  double* eps2; /* limiter eps^2 per cell (venk / albada) */
  /* solution */
  double *pvar, *cvar, *grad, *resid, *phi, *ws;
  double pvar_inf[4];
  double *mms_sol, *mms_src;
  double mc[16];
  /* rk */
  double h_rk[5], rk_coef[5], dts[5], dte[5];
  double dt;
  int dt_ready;
  double* dt_local;
  int icont;
  /* race-free parallel residual */
  double* eflux; /* [nslots][5] */
  int* clist;    /* [ncells+1][8] signed slot+1 (negative: subtract) */
  int* ncl;
};

#define P(c, ic, v) ((c)->pvar[4 * (ic) + (v)])
#define U(c, ic, v) ((c)->cvar[4 * (ic) + (v)])
#define R(c, ic, v) ((c)->resid[4 * (ic) + (v)])
#define G(c, ic, v, d) ((c)->grad[(size_t)(d) * 4 * ((c)->ncells + 1) + 4 * (ic) + (v)])

static void set_err(char* err, int errlen, const char* fmt, ...) {
  if (!err || errlen <= 0) return;
  va_list ap; va_start(ap, fmt); vsnprintf(err, (size_t)errlen, fmt, ap); va_end(ap);
}

/* minimum-image helpers (identity for non-periodic meshes) */
static inline double mix(const orc* c, double d) { return c->Lx > 0 ? d - c->Lx * nearbyint(d / c->Lx) : d; }
static inline double miy(const orc* c, double d) { return c->Ly > 0 ? d - c->Ly * nearbyint(d / c->Ly) : d; }
static inline double unwx(const orc* c, double x, double xref) { return c->Lx > 0 ? x - c->Lx * nearbyint((x - xref) / c->Lx) : x; }
static inline double unwy(const orc* c, double y, double yref) { return c->Ly > 0 ? y - c->Ly * nearbyint((y - yref) / c->Ly) : y; }

/* tri_area, src/grid_procs.f90:800-808 */
static double tri_area(double x1, double x2, double x3, double y1, double y2, double y3) {
  return 0.5 * (((x1 * (y2 - y3)) + (x2 * (y3 - y1))) + (x3 * (y1 - y2)));
}

/* ========================================================================= */
/* grid_data, src/grid_procs.f90:170-794                                      */
/* ========================================================================= */
static int grid_data(orc* c, char* err, int errlen) {
  int nc = c->ncells;
  double xmin = 0, ymin = 0;
  if (c->Lx > 0 || c->Ly > 0) {
    xmin = c->xn[1]; ymin = c->yn[1];
    for (int i = 2; i <= c->nnodes; i++) { if (c->xn[i] < xmin) xmin = c->xn[i]; if (c->yn[i] < ymin) ymin = c->yn[i]; }
  }
  /* cell centroids :185-208 (vertices unwrapped against the first one) */
  for (int ic = 1; ic <= nc; ic++) {
    int nv = c->nvrt[ic];
    double x1 = c->xn[c->cnode[ic][1]], y1 = c->yn[c->cnode[ic][1]];
    double xs = 0.0, ys = 0.0;
    for (int iv = 1; iv <= nv; iv++) {
      int vp = c->cnode[ic][iv];
      xs = xs + unwx(c, c->xn[vp], x1);
      ys = ys + unwy(c, c->yn[vp], y1);
    }
    double xcv = xs / (double)nv, ycv = ys / (double)nv;
    if (c->Lx > 0) { if (xcv < xmin) xcv += c->Lx; else if (xcv >= xmin + c->Lx) xcv -= c->Lx; }
    if (c->Ly > 0) { if (ycv < ymin) ycv += c->Ly; else if (ycv >= ymin + c->Ly) ycv -= c->Ly; }
    c->xc[ic] = xcv; c->yc[ic] = ycv;
  }
  /* cell volume :214-227 */
  for (int ic = 1; ic <= nc; ic++) {
    double X[5], Y[5];
    int n1 = c->cnode[ic][1];
    for (int k = 1; k <= c->nvrt[ic]; k++) {
      int v = c->cnode[ic][k];
      X[k] = unwx(c, c->xn[v], c->xn[n1]); Y[k] = unwy(c, c->yn[v], c->yn[n1]);
    }
    if (c->nvrt[ic] == 3) c->vol[ic] = tri_area(X[1], X[2], X[3], Y[1], Y[2], Y[3]);
    else c->vol[ic] = tri_area(X[1], X[2], X[3], Y[1], Y[2], Y[3]) + tri_area(X[1], X[3], X[4], Y[1], Y[3], Y[4]);
  }
  /* heff :233-243 */
  double at = 0.0;
  for (int ic = 1; ic <= nc; ic++) at = at + c->vol[ic];
  c->heff1 = sqrt(at / (double)nc);
  at = 0.0;
  for (int ic = 1; ic <= nc; ic++) at = at + sqrt(c->vol[ic]);
  c->heff2 = at / (double)nc;
  /* kd-tree on cell centres :261-267 (only the LSQ-fn setup queries it) */
  c->kd_xy = (double*)malloc(sizeof(double) * 2 * (size_t)nc);
  for (int i = 1; i <= nc; i++) { c->kd_xy[2 * (i - 1)] = c->xc[i]; c->kd_xy[2 * (i - 1) + 1] = c->yc[i]; }
  c->tree.n = nc; c->tree.data = c->kd_xy;
  c->tree.ind = (int*)malloc(sizeof(int) * (size_t)(nc + 1));
  for (int j = 1; j <= nc; j++) c->tree.ind[j] = j;
  c->tree.root = kd_build(&c->tree, 1, nc, NULL);
  /* node -> cell :273-296 */
  c->nd_nc = (int*)calloc((size_t)c->nnodes + 1, sizeof(int));
  c->nd_ptr = (int*)calloc((size_t)c->nnodes + 2, sizeof(int));
  for (int ic = 1; ic <= nc; ic++)
    for (int iv = 1; iv <= c->nvrt[ic]; iv++) c->nd_nc[c->cnode[ic][iv]]++;
  c->nd_ptr[1] = 0;
  for (int i = 1; i <= c->nnodes; i++) c->nd_ptr[i + 1] = c->nd_ptr[i] + c->nd_nc[i];
  c->nd_cell = (int*)malloc(sizeof(int) * (size_t)(c->nd_ptr[c->nnodes + 1] + 1));
  for (int i = 1; i <= c->nnodes; i++) c->nd_nc[i] = 0;
  for (int ic = 1; ic <= nc; ic++)
    for (int iv = 1; iv <= c->nvrt[ic]; iv++) {
      int vp = c->cnode[ic][iv];
      c->nd_nc[vp]++;
      c->nd_cell[c->nd_ptr[vp] + c->nd_nc[vp] - 1] = ic;
    }
  /* edge neighbours :325-366 */
  for (int ic = 1; ic <= nc; ic++) {
    int nv = c->nvrt[ic];
    for (int iv = 1; iv <= nv; iv++) {
      int vL = (iv < nv) ? c->cnode[ic][iv + 1] : c->cnode[ic][1];
      int vR = c->cnode[ic][iv];
      int lfound = 0, jc = 0, im = 0;
      for (int j = 1; j <= c->nd_nc[vR]; j++) {
        jc = c->nd_cell[c->nd_ptr[vR] + j - 1];
        int nvj = c->nvrt[jc];
        for (int ii = 1; ii <= nvj; ii++) {
          int v2 = (ii > 1) ? c->cnode[jc][ii - 1] : c->cnode[jc][nvj];
          int v1 = c->cnode[jc][ii];
          if (v1 == vR && v2 == vL) {
            lfound = 1;
            im = ii + 1;
            if (im > nvj) im = im - nvj;
            break;
          }
        }
        if (lfound) break;
      }
      int in = iv + 2;
      if (in > nv) in = in - nv;
      if (lfound) { c->nghbr[ic][in] = jc; c->nghbr[jc][im] = ic; }
      else c->nghbr[ic][in] = 0;
    }
  }
  /* nghbre :373-395 */
  static const int loc_tri[4] = {0, 2, 3, 1}, loc_quad[5] = {0, 3, 4, 1, 2};
  for (int ic = 1; ic <= nc; ic++) {
    for (int k = 1; k <= 4; k++) c->nghbre[ic][k] = 0;
    for (int k = 1; k <= c->nvrt[ic]; k++) {
      int ie = (c->nvrt[ic] == 3) ? loc_tri[k] : loc_quad[k];
      c->nghbre[ic][ie] = c->nghbr[ic][k];
    }
  }
  /* count edges :401-407 */
  int ne = 0;
  for (int ic = 1; ic <= nc; ic++)
    for (int j = 1; j <= c->nvrt[ic]; j++)
      if (c->nghbr[ic][j] > ic || c->nghbr[ic][j] == 0) ne++;
  c->nedges = ne;
  c->en1 = (int*)calloc((size_t)ne + 1, sizeof(int)); c->en2 = (int*)calloc((size_t)ne + 1, sizeof(int));
  c->ec1 = (int*)calloc((size_t)ne + 1, sizeof(int)); c->ec2 = (int*)calloc((size_t)ne + 1, sizeof(int));
  /* edge nodes and cells :413-486; local edge k of a cell runs node(k)->node(k+1)
   * and its neighbour sits at nghbr(k+2 wrapped): tri order (3,1,2), quad (3,4,1,2) */
  static const int tri_nb[4] = {0, 3, 1, 2}, quad_nb[5] = {0, 3, 4, 1, 2};
  ne = 0;
  for (int pass = 0; pass < 2; pass++) {
    int lo = pass == 0 ? 1 : c->ntri + 1, hi = pass == 0 ? c->ntri : nc;
    for (int ic = lo; ic <= hi; ic++) {
      int nv = c->nvrt[ic];
      for (int k = 1; k <= nv; k++) {
        int nb = nv == 3 ? tri_nb[k] : quad_nb[k];
        if (c->nghbr[ic][nb] > ic || c->nghbr[ic][nb] == 0) {
          ne++;
          c->en1[ne] = c->cnode[ic][k];
          c->en2[ne] = c->cnode[ic][k < nv ? k + 1 : 1];
          c->ec1[ne] = ic;
          c->ec2[ne] = c->nghbr[ic][nb];
        }
      }
    }
  }
  /* cell -> edge :492-624 */
  static const int tri_v2e[5] = {0, 2, 3, 1, 0}, qud_v2e[5] = {0, 3, 4, 1, 2};
  ne = 0;
  for (int pass = 0; pass < 2; pass++) {
    int lo = pass == 0 ? 1 : c->ntri + 1, hi = pass == 0 ? c->ntri : nc;
    for (int ic = lo; ic <= hi; ic++) {
      int nv = c->nvrt[ic];
      for (int k = 1; k <= nv; k++) {
        int nb = nv == 3 ? tri_nb[k] : quad_nb[k];
        if (c->nghbr[ic][nb] > ic || c->nghbr[ic][nb] == 0) {
          ne++;
          c->cedge[ic][k] = ne;
        } else {
          int jc = c->nghbr[ic][nb];
          const int* idum4 = c->nvrt[jc] == 3 ? tri_v2e : qud_v2e;
          for (int kk = 1; kk <= c->nvrt[jc]; kk++) {
            if (c->nghbr[jc][kk] == ic) { c->cedge[ic][k] = c->cedge[jc][idum4[kk]]; break; }
          }
        }
      }
    }
  }
  /* edge geometry :630-647 (second node unwrapped against the first) */
  c->ex = (double*)calloc((size_t)ne + 1, sizeof(double)); c->ey = (double*)calloc((size_t)ne + 1, sizeof(double));
  c->ea = (double*)calloc((size_t)ne + 1, sizeof(double)); c->enx = (double*)calloc((size_t)ne + 1, sizeof(double));
  c->eny = (double*)calloc((size_t)ne + 1, sizeof(double)); c->etx = (double*)calloc((size_t)ne + 1, sizeof(double));
  c->ety = (double*)calloc((size_t)ne + 1, sizeof(double));
  for (int i = 1; i <= ne; i++) {
    int v1 = c->en1[i], v2 = c->en2[i];
    double x1 = c->xn[v1], y1 = c->yn[v1];
    double x2 = unwx(c, c->xn[v2], x1), y2 = unwy(c, c->yn[v2], y1);
    double dx = x2 - x1, dy = y2 - y1;
    c->ea[i] = sqrt(dx * dx + dy * dy);
    double xf = 0.5 * (x1 + x2), yf = 0.5 * (y1 + y2);
    if (c->Lx > 0) { if (xf < xmin) xf += c->Lx; else if (xf >= xmin + c->Lx) xf -= c->Lx; }
    if (c->Ly > 0) { if (yf < ymin) yf += c->Ly; else if (yf >= ymin + c->Ly) yf -= c->Ly; }
    c->ex[i] = xf; c->ey[i] = yf;
    c->enx[i] = dy / c->ea[i];
    c->eny[i] = -dx / c->ea[i];
    c->etx[i] = dx / c->ea[i];
    c->ety[i] = dy / c->ea[i];
  }
  /* nrmlsign :672-691 */
  for (int ic = 1; ic <= nc; ic++)
    for (int ie = 1; ie <= 4; ie++)
      c->nrmlsign[ic][ie] = (ie <= c->nvrt[ic] && c->ec1[c->cedge[ic][ie]] != ic) ? -1.0 : 1.0;
  /* interior / boundary cells :697-728 */
  c->cell_intr = (int*)calloc((size_t)nc + 1, sizeof(int));
  c->cell_bndr = (int*)calloc((size_t)nc + 1, sizeof(int));
  c->ncells_intr = c->ncells_bndr = 0;
  for (int ic = 1; ic <= nc; ic++) {
    int im = 1;
    for (int ie = 1; ie <= c->nvrt[ic]; ie++) if (c->nghbre[ic][ie] == 0) im = 0;
    if (im == 1) c->cell_intr[++c->ncells_intr] = ic;
    else c->cell_bndr[++c->ncells_bndr] = ic;
  }
  int sumb = 0;
  for (int ib = 1; ib <= c->nb; ib++) sumb += c->b_ncells[ib];
  if (c->ncells_bndr != sumb) {
    set_err(err, errlen, "boundary cells determined %d != %d listed in .bc (grid_data)", c->ncells_bndr, sumb);
    return FVS_ERR_MESH;
  }
  /* interior / boundary edges :733-791 */
  c->edge_intr = (int*)calloc((size_t)ne + 1, sizeof(int));
  c->edge_bndr = (int*)calloc((size_t)ne + 1, sizeof(int));
  c->bedge_cell = (int*)calloc((size_t)ne + 1, sizeof(int));
  c->nedges_intr = c->nedges_bndr = 0;
  for (int ie = 1; ie <= ne; ie++) {
    if (c->ec1[ie] == 0 && c->ec2[ie] > 0) {
      c->nedges_bndr++; c->edge_bndr[c->nedges_bndr] = ie; c->bedge_cell[c->nedges_bndr] = c->ec2[ie];
    } else if (c->ec1[ie] > 0 && c->ec2[ie] == 0) {
      c->nedges_bndr++; c->edge_bndr[c->nedges_bndr] = ie; c->bedge_cell[c->nedges_bndr] = c->ec1[ie];
    } else if (c->ec1[ie] > 0 && c->ec2[ie] > 0) {
      c->nedges_intr++; c->edge_intr[c->nedges_intr] = ie;
    } else {
      set_err(err, errlen, "edge %d has no cell (grid_data)", ie);
      return FVS_ERR_MESH;
    }
  }
  c->b_nedges = (int*)calloc((size_t)c->nb + 1, sizeof(int));
  c->b_eptr = (int*)calloc((size_t)c->nb + 2, sizeof(int));
  c->b_edge = (int*)calloc((size_t)ne + 1, sizeof(int));
  int pos = 0;
  for (int ib = 1; ib <= c->nb; ib++) {
    c->b_eptr[ib] = pos;
    for (int i = 1; i <= c->b_ncells[ib]; i++) {
      int ic = c->b_cell[c->b_cptr[ib] + i - 1];
      if (ic < 1 || ic > nc) { set_err(err, errlen, "boundary %d lists cell %d out of range", ib, ic); return FVS_ERR_MESH; }
      for (int ie = 1; ie <= c->nvrt[ic]; ie++) {
        int je = c->cedge[ic][ie];
        if ((c->ec1[je] == ic && c->ec2[je] == 0) || (c->ec1[je] == 0 && c->ec2[je] == ic)) {
          if (pos >= ne) { set_err(err, errlen, "too many boundary edges"); return FVS_ERR_MESH; }
          c->b_edge[++pos] = je;
          c->b_nedges[ib]++;
        }
      }
    }
  }
  c->b_eptr[c->nb + 1] = pos;
  if (c->nedges_bndr != pos) {
    set_err(err, errlen, "boundary edges determined %d != %d read (grid_data)", c->nedges_bndr, pos);
    return FVS_ERR_MESH;
  }
  for (int ib = 1; ib <= c->nb; ib++)
    if (c->b_nedges[ib] != c->b_ncells[ib]) {
      set_err(err, errlen, "boundary %d has %d edges for %d cells: the reference pairs edge i with cell i "
              "(src/residual.f90:114-125)", ib, c->b_nedges[ib], c->b_ncells[ib]);
      return FVS_ERR_MESH;
    }
  /* grid_data_verify :814-852 */
  c->vol1 = 0.0;
  for (int ic = 1; ic <= nc; ic++) c->vol1 = c->vol1 + c->vol[ic];
  c->vol2 = 0.0;
  for (int ic = 1; ic <= nc; ic++) {
    double v = 0.0;
    for (int ie = 1; ie <= c->nvrt[ic]; ie++) {
      int je = c->cedge[ic][ie];
      double nx = c->enx[je] * c->nrmlsign[ic][ie];
      v = v + ((nx * c->ex[je]) * c->ea[je]);
    }
    c->vol2 = c->vol2 + v;
  }
  for (int ie = 1; ie <= ne; ie++)
    if (c->ec1[ie] <= 0) { set_err(err, errlen, "edge(%d)%%c1 <= 0 (grid_data_verify)", ie); return FVS_ERR_MESH; }
  return FVS_OK;
}

/* ========================================================================= */
/* gradient operators                                                        */
/* ========================================================================= */
/* LSQ coefficients for one cell, shared by setup_fn :137-201 and setup_nn
 * :292-338 (identical arithmetic) */
static int lsq_coeffs(orc* c, int ic) {
  double xc = c->xc[ic], yc = c->yc[ic];
  int b = c->st_ptr[ic], n = c->st_ptr[ic + 1] - b;
  double d[64][2];
  if (n > 64) return FVS_ERR_MESH;
  for (int in = 0; in < n; in++) {
    int jc = c->st_cell[b + in];
    double dxx = mix(c, c->xc[jc] - xc), dyy = miy(c, c->yc[jc] - yc);
    double dis = sqrt(dxx * dxx + dyy * dyy);
    double w = 0.0;
    c->st_w[b + in] = 0.0;
    if (dis > 0.0) { w = 1.0 / pow(dis, c->o.lsq_pow); c->st_w[b + in] = w; }
    d[in][0] = w * dxx;
    d[in][1] = w * dyy;
  }
  double g[2][2];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      g[i][j] = 0.0;
      for (int in = 0; in < n; in++) g[i][j] = g[i][j] + d[in][i] * d[in][j];
    }
  double det = g[0][0] * g[1][1] - g[0][1] * g[1][0];
  double gi[2][2];
  gi[0][0] = 1.0 / det * g[1][1];
  gi[1][1] = 1.0 / det * g[0][0];
  gi[0][1] = -1.0 / det * g[0][1];
  gi[1][0] = -1.0 / det * g[1][0];
  for (int in = 0; in < n; in++)
    for (int i = 0; i < 2; i++) {
      double s = 0.0;
      for (int k = 0; k < 2; k++) s = s + gi[i][k] * d[in][k];
      c->st_coef[2 * (b + in) + i] = s;
    }
  return FVS_OK;
}

/* setup_fn, src/gradient_lsq.f90:70-208 */
static int setup_fn(orc* c, char* err, int errlen) {
  int nc = c->ncells;
  c->st_ptr = (int*)calloc((size_t)nc + 2, sizeof(int));
  for (int ic = 1; ic <= nc; ic++) c->st_ptr[ic + 1] = c->st_ptr[ic] + c->nvrt[ic];
  c->st_len = c->st_ptr[nc + 1];
  c->st_cell = (int*)calloc((size_t)c->st_len + 1, sizeof(int));
  c->st_coef = (double*)calloc(2 * (size_t)c->st_len + 2, sizeof(double));
  c->st_w = (double*)calloc((size_t)c->st_len + 1, sizeof(double));
  kd_res fnearest[9];
  const int num_nearests = 8;
  for (int ic = 1; ic <= nc; ic++) {
    int b = c->st_ptr[ic], nv = c->nvrt[ic], izb = 0, tmpi[5] = {0, 0, 0, 0, 0};
    for (int in = 1; in <= nv; in++) {
      int jc = c->nghbr[ic][in];
      if (jc == 0) tmpi[++izb] = in;
      else c->st_cell[b + in - 1] = jc;
    }
    if (izb > 0 && izb < 3) {
      double r[2] = {c->xc[ic], c->yc[ic]};
      kd_n_nearest(&c->tree, r, num_nearests, fnearest);
      int nt = 0;
      for (int i = 1; i <= num_nearests; i++) {
        int jc = fnearest[i].idx;
        if (jc != ic) {
          double dum = 1.0;
          for (int in = 1; in <= nv; in++) {
            int dd = abs(c->nghbr[ic][in] - jc);
            dum = dum * (double)(dd > 0 ? dd : 0);
          }
          if (dum > 0.0) {
            nt++;
            c->st_cell[b + tmpi[nt] - 1] = jc;
          }
          if (nt == izb) break;
        }
      }
      if (nt < izb) { set_err(err, errlen, "setup_fn: cell %d found %d of %d padding cells", ic, nt, izb); return FVS_ERR_MESH; }
    } else if (izb > 2) {
      set_err(err, errlen, "setup_fn: cell %d has %d boundary edges (>2)", ic, izb);
      return FVS_ERR_MESH;
    }
  }
  for (int ic = 1; ic <= nc; ic++)
    if (lsq_coeffs(c, ic) != FVS_OK) { set_err(err, errlen, "lsq stencil too long"); return FVS_ERR_MESH; }
  return FVS_OK;
}

static int cmp_int(const void* a, const void* b) { int x = *(const int*)a, y = *(const int*)b; return (x > y) - (x < y); }

/* setup_nn, src/gradient_lsq.f90:214-365: node-neighbour cells, ascending,
 * duplicates removed */
static int setup_nn(orc* c, char* err, int errlen) {
  int nc = c->ncells;
  c->st_ptr = (int*)calloc((size_t)nc + 2, sizeof(int));
  int* tmp = (int*)malloc(sizeof(int) * 256);
  int total = 0;
  int** lists = (int**)calloc((size_t)nc + 1, sizeof(int*));
  for (int ic = 1; ic <= nc; ic++) {
    int nt = 0;
    for (int in = 1; in <= c->nvrt[ic]; in++) {
      int iv = c->cnode[ic][in];
      for (int i = 1; i <= c->nd_nc[iv]; i++) {
        int jc = c->nd_cell[c->nd_ptr[iv] + i - 1];
        if (jc != ic) { if (nt >= 256) { free(tmp); set_err(err, errlen, "setup_nn: stencil > 256"); return FVS_ERR_MESH; } tmp[nt++] = jc; }
      }
    }
    qsort(tmp, (size_t)nt, sizeof(int), cmp_int);
    int nu = 0;
    for (int i = 0; i < nt; i++) if (nu == 0 || tmp[i] != tmp[nu - 1]) tmp[nu++] = tmp[i];
    lists[ic] = (int*)malloc(sizeof(int) * (size_t)(nu + 1));
    memcpy(lists[ic], tmp, sizeof(int) * (size_t)nu);
    c->st_ptr[ic + 1] = c->st_ptr[ic] + nu;
    total += nu;
  }
  free(tmp);
  c->st_len = total;
  c->st_cell = (int*)calloc((size_t)total + 1, sizeof(int));
  c->st_coef = (double*)calloc(2 * (size_t)total + 2, sizeof(double));
  c->st_w = (double*)calloc((size_t)total + 1, sizeof(double));
  for (int ic = 1; ic <= nc; ic++) {
    memcpy(c->st_cell + c->st_ptr[ic], lists[ic], sizeof(int) * (size_t)(c->st_ptr[ic + 1] - c->st_ptr[ic]));
    free(lists[ic]);
  }
  free(lists);
  for (int ic = 1; ic <= nc; ic++)
    if (lsq_coeffs(c, ic) != FVS_OK) { set_err(err, errlen, "lsq stencil too long (>64)"); return FVS_ERR_MESH; }
  return FVS_OK;
}

/* grad_lsq_verify, src/gradient_lsq.f90:490-529 */
static int lsq_verify(orc* c, char* err, int errlen) {
  const double cstx = 2.0, csty = 1.0;
  for (int ic = 1; ic <= c->ncells; ic++) {
    double dfx = 0.0, dfy = 0.0;
    for (int k = c->st_ptr[ic]; k < c->st_ptr[ic + 1]; k++) {
      int jc = c->st_cell[k];
      double diff;
      if (c->Lx > 0 || c->Ly > 0)
        diff = csty * miy(c, c->yc[jc] - c->yc[ic]) + cstx * mix(c, c->xc[jc] - c->xc[ic]);
      else
        diff = csty * c->yc[jc] + cstx * c->xc[jc] - (csty * c->yc[ic] + cstx * c->xc[ic]);
      dfx = dfx + c->st_coef[2 * k] * diff * c->st_w[k];
      dfy = dfy + c->st_coef[2 * k + 1] * diff * c->st_w[k];
    }
    if (fabs(dfx - cstx) > 1.0e-10 || fabs(dfy - csty) > 1.0e-10) {
      set_err(err, errlen, "LSQ coefficients are not correct at cell %d: df/dx=%.17g df/dy=%.17g (grad_lsq_verify)", ic, dfx, dfy);
      return FVS_ERR_MESH;
    }
  }
  return FVS_OK;
}

/* grad_ggcb setup, src/gradient_ggcb.f90:48-110 */
static void setup_ggcb(orc* c) {
  int nc = c->ncells;
  c->st_ptr = (int*)calloc((size_t)nc + 2, sizeof(int));
  for (int ic = 1; ic <= nc; ic++) c->st_ptr[ic + 1] = c->st_ptr[ic] + c->nvrt[ic];
  c->st_len = c->st_ptr[nc + 1];
  c->st_cell = (int*)calloc((size_t)c->st_len + 1, sizeof(int));
  c->st_coef = (double*)calloc(2 * (size_t)c->st_len + 2, sizeof(double));
  c->coef0 = calloc((size_t)nc + 1, sizeof(*c->coef0));
  for (int ic = 1; ic <= nc; ic++) {
    double xc = c->xc[ic], yc = c->yc[ic];
    c->coef0[ic][0] = 0.0; c->coef0[ic][1] = 0.0;
    for (int ie = 1; ie <= c->nvrt[ic]; ie++) {
      int je = c->cedge[ic][ie], k = c->st_ptr[ic] + ie - 1;
      int ic1 = c->ec1[je], ic2 = c->ec2[je];
      double af = c->ea[je];
      double nxf = c->enx[je] * c->nrmlsign[ic][ie];
      double nyf = c->eny[je] * c->nrmlsign[ic][ie];
      double xf = c->ex[je], yf = c->ey[je];
      double dx = mix(c, xf - xc), dy = miy(c, yf - yc);
      double d0 = sqrt(dx * dx + dy * dy);
      double xc1 = xc, yc1 = yc;
      c->st_cell[k] = ic;
      if (ic1 > 0 && ic1 != ic) { xc1 = c->xc[ic1]; yc1 = c->yc[ic1]; c->st_cell[k] = ic1; }
      else if (ic2 > 0 && ic2 != ic) { xc1 = c->xc[ic2]; yc1 = c->yc[ic2]; c->st_cell[k] = ic2; }
      dx = mix(c, xf - xc1); dy = miy(c, yf - yc1);
      double d1 = sqrt(dx * dx + dy * dy);
      c->coef0[ic][0] = c->coef0[ic][0] + d1 / (d0 + d1) * nxf * af;
      c->coef0[ic][1] = c->coef0[ic][1] + d1 / (d0 + d1) * nyf * af;
      c->st_coef[2 * k] = d0 / (d0 + d1) * nxf * af;
      c->st_coef[2 * k + 1] = d0 / (d0 + d1) * nyf * af;
    }
  }
}

/* grad_ggnb setup, src/gradient_ggnb.f90:49-177 */
static void setup_ggnb(orc* c) {
  int nc = c->ncells;
  double* idw = (double*)calloc((size_t)c->nnodes + 1, sizeof(double));
  for (int in = 1; in <= c->nnodes; in++) {
    double xv = c->xn[in], yv = c->yn[in], idt = 0.0;
    for (int i = 1; i <= c->nd_nc[in]; i++) {
      int ic = c->nd_cell[c->nd_ptr[in] + i - 1];
      double dx = mix(c, c->xc[ic] - xv), dy = miy(c, c->yc[ic] - yv);
      double d = sqrt(dx * dx + dy * dy);
      idt = idt + 1.0 / d;
    }
    idw[in] = 1.0 / idt;
  }
  c->coef0 = calloc((size_t)nc + 1, sizeof(*c->coef0));
  for (int ic = 1; ic <= nc; ic++) {
    c->coef0[ic][0] = 0.0; c->coef0[ic][1] = 0.0;
    for (int ie = 1; ie <= c->nvrt[ic]; ie++) {
      int je = c->cedge[ic][ie];
      double af = c->ea[je];
      double nxf = c->enx[je] * c->nrmlsign[ic][ie];
      double nyf = c->eny[je] * c->nrmlsign[ic][ie];
      int iv1 = c->en1[je], iv2 = c->en2[je];
      double dx = mix(c, c->xc[ic] - c->xn[iv1]), dy = miy(c, c->yc[ic] - c->yn[iv1]);
      double w1 = 1.0 / sqrt(dx * dx + dy * dy);
      dx = mix(c, c->xc[ic] - c->xn[iv2]); dy = miy(c, c->yc[ic] - c->yn[iv2]);
      double w2 = 1.0 / sqrt(dx * dx + dy * dy);
      double wt1 = idw[iv1], wt2 = idw[iv2];
      c->coef0[ic][0] = c->coef0[ic][0] + af * nxf / 2.0 * (w1 * wt1 + w2 * wt2);
      c->coef0[ic][1] = c->coef0[ic][1] + af * nyf / 2.0 * (w1 * wt1 + w2 * wt2);
    }
  }
  c->st_ptr = (int*)calloc((size_t)nc + 2, sizeof(int));
  for (int ic = 1; ic <= nc; ic++) {
    int i = 0;
    for (int in = 1; in <= c->nvrt[ic]; in++) i += c->nd_nc[c->cnode[ic][in]];
    c->st_ptr[ic + 1] = c->st_ptr[ic] + i;
  }
  c->st_len = c->st_ptr[nc + 1];
  c->st_cell = (int*)calloc((size_t)c->st_len + 1, sizeof(int));
  c->st_coef = (double*)calloc((size_t)c->st_len + 1, sizeof(double));
  for (int ic = 1; ic <= nc; ic++) {
    int i = c->st_ptr[ic];
    for (int in = 1; in <= c->nvrt[ic]; in++) {
      int iv = c->cnode[ic][in];
      double xv = c->xn[iv], yv = c->yn[iv];
      for (int j = 1; j <= c->nd_nc[iv]; j++) {
        int jc = c->nd_cell[c->nd_ptr[iv] + j - 1];
        double dx = mix(c, c->xc[jc] - xv), dy = miy(c, c->yc[jc] - yv);
        double d = sqrt(dx * dx + dy * dy);
        c->st_cell[i] = jc;
        c->st_coef[i] = idw[iv] / d;
        if (jc == ic) c->st_coef[i] = 0.0;
        i++;
      }
    }
  }
  c->coefedg = calloc((size_t)nc + 1, sizeof(*c->coefedg));
  for (int ic = 1; ic <= nc; ic++) {
    for (int in = 1; in <= c->nvrt[ic]; in++) {
      int iv = c->cnode[ic][in];
      c->coefedg[ic][in][0] = 0.0; c->coefedg[ic][in][1] = 0.0;
      for (int ie = 1; ie <= c->nvrt[ic]; ie++) {
        int je = c->cedge[ic][ie];
        for (int j = 1; j <= 2; j++) {
          int jv = (j == 1) ? c->en1[je] : c->en2[je];
          if (jv == iv) {
            double af = c->ea[je];
            double nxf = c->enx[je] * c->nrmlsign[ic][ie];
            double nyf = c->eny[je] * c->nrmlsign[ic][ie];
            c->coefedg[ic][in][0] = c->coefedg[ic][in][0] + af * nxf / 2.0;
            c->coefedg[ic][in][1] = c->coefedg[ic][in][1] + af * nyf / 2.0;
          }
        }
      }
    }
  }
  free(idw);
}

/* ========================================================================= */
/* solution data, MMS, vortex                                                */
/* ========================================================================= */
/* cvar2pvar for one cell, src/data_solution.f90:72-86 */
static inline void cvar2pvar_cell(orc* c, int ic) {
  double g = c->o.gamma;
  P(c, ic, 0) = U(c, ic, 0);
  P(c, ic, 1) = U(c, ic, 1) / U(c, ic, 0);
  P(c, ic, 2) = U(c, ic, 2) / U(c, ic, 0);
  P(c, ic, 3) = (g - 1.0) * (U(c, ic, 3) - 0.5 * P(c, ic, 0) * (P(c, ic, 1) * P(c, ic, 1) + P(c, ic, 2) * P(c, ic, 2)));
}

/* pvar2cvar / prim2cnsr, src/data_solution.f90:92-124 */
static inline void prim2cnsr(double g, const double* w, double* u) {
  u[0] = w[0];
  u[1] = w[0] * w[1];
  u[2] = w[0] * w[2];
  u[3] = w[3] / (g - 1.0) + 0.5 * w[0] * (w[1] * w[1] + w[2] * w[2]);
}

/* manufactured_sol, src/mms.f90:187-213 */
static double manufactured_sol(double a0, double as, double ax, double ay, int nx, int ny, double x, double y) {
  double f;
  if (nx + ny == 0) return a0 + as * sin(ax * x + ay * y);
  double pw = pow(ax, (double)nx) * pow(ay, (double)ny);
  if ((nx + ny) % 2 == 0) {
    f = -pw * as * sin(ax * x + ay * y);
    if ((nx + ny) % 4 == 0) f = -f;
  } else {
    f = pw * as * cos(ax * x + ay * y);
    if ((nx + ny + 1) % 4 == 0) f = -f;
  }
  return f;
}

/* mms constants, src/mms.f90:79-101 */
static void mms_constants(double* mc) {
  mc[0] = 1.12; mc[1] = 0.15; mc[2] = 3.12 * PI; mc[3] = 2.92 * PI;
  mc[4] = 1.32; mc[5] = 0.06; mc[6] = 2.09 * PI; mc[7] = 3.12 * PI;
  mc[8] = 1.18; mc[9] = 0.03; mc[10] = 2.15 * PI; mc[11] = 3.32 * PI;
  mc[12] = 1.62; mc[13] = 0.31; mc[14] = 3.79 * PI; mc[15] = 2.98 * PI;
}

/* mms_compute_euler2d, src/mms.f90:124-181 */
static void mms_euler2d(const orc* c, double xc, double yc, double* sol, double* rhs) {
  const double* m = c->mc;
  double g = c->o.gamma;
  double r = manufactured_sol(m[0], m[1], m[2], m[3], 0, 0, xc, yc);
  double u = manufactured_sol(m[4], m[5], m[6], m[7], 0, 0, xc, yc);
  double v = manufactured_sol(m[8], m[9], m[10], m[11], 0, 0, xc, yc);
  double p = manufactured_sol(m[12], m[13], m[14], m[15], 0, 0, xc, yc);
  sol[0] = r; sol[1] = u; sol[2] = v; sol[3] = p;
  double rx = manufactured_sol(m[0], m[1], m[2], m[3], 1, 0, xc, yc);
  double ux = manufactured_sol(m[4], m[5], m[6], m[7], 1, 0, xc, yc);
  double vx = manufactured_sol(m[8], m[9], m[10], m[11], 1, 0, xc, yc);
  double px = manufactured_sol(m[12], m[13], m[14], m[15], 1, 0, xc, yc);
  double ry = manufactured_sol(m[0], m[1], m[2], m[3], 0, 1, xc, yc);
  double uy = manufactured_sol(m[4], m[5], m[6], m[7], 0, 1, xc, yc);
  double vy = manufactured_sol(m[8], m[9], m[10], m[11], 0, 1, xc, yc);
  double py = manufactured_sol(m[12], m[13], m[14], m[15], 0, 1, xc, yc);
  double rH = g / (g - 1.0) * p + r * u * u / 2.0 + r * v * v / 2.0;
  double rHx = g / (g - 1.0) * px + rx * (u * u + v * v) / 2.0 + r * (u * ux + v * vx);
  double rHy = g / (g - 1.0) * py + ry * (u * u + v * v) / 2.0 + r * (u * uy + v * vy);
  rhs[0] = rx * u + u * rx + ry * v + r * vy;
  rhs[1] = rx * u * u + 2.0 * r * u * ux + ry * u * v + r * uy * v + r * u * vy + px;
  rhs[2] = rx * u * v + r * ux * v + r * u * vx + ry * v * v + 2.0 * r * v * vy + py;
  rhs[3] = u * rHx + ux * rH + v * rHy + vy * rH;
}

/* compute_isentropic_vortex, src/mms.f90:219-265 */
static void vortex_state(const orc* c, double t, double x, double y, double* pv) {
  double g = c->o.gamma, K = c->o.vortex_kappa;
  double rho_inf = c->o.vortex_inf[0], u_inf = c->o.vortex_inf[1], v_inf = c->o.vortex_inf[2], p_inf = c->o.vortex_inf[3];
  double T_inf = p_inf / rho_inf;
  double xc = c->o.vortex_x + u_inf * t;
  double yc = c->o.vortex_y + v_inf * t;
  double dx = x - xc, dy = y - yc;
  double r = sqrt(dx * dx + dy * dy);
  double u = u_inf - K / (2.0 * PI) * dy * exp(0.5 * (1.0 - r * r));
  double v = v_inf + K / (2.0 * PI) * dx * exp(0.5 * (1.0 - r * r));
  double q = K / (2.0 * PI);
  double temp = T_inf - (q * q) * (g - 1.0) / (2.0 * g) * exp(1.0 - r * r);
  double rho = pow(temp, 1.0 / (g - 1.0));
  double p = pow(rho, g);
  pv[0] = rho; pv[1] = u; pv[2] = v; pv[3] = p;
}

/* ========================================================================= */
/* residual: gradient, limiter, Roe flux, bc_flux                            */
/* ========================================================================= */
static void gradient_cell(orc* c, int ic) {
  int m = c->o.grad_method;
  if (m == FVS_GRAD_LSQ) { /* grad_lsq, src/gradient_lsq.f90:371-419 (in-outer, ivar-inner) */
    for (int v = 0; v < NV; v++) { G(c, ic, v, 0) = 0.0; G(c, ic, v, 1) = 0.0; }
    for (int k = c->st_ptr[ic]; k < c->st_ptr[ic + 1]; k++) {
      int jc = c->st_cell[k];
      for (int v = 0; v < NV; v++) {
        G(c, ic, v, 0) = G(c, ic, v, 0) + c->st_coef[2 * k] * (P(c, jc, v) - P(c, ic, v)) * c->st_w[k];
        G(c, ic, v, 1) = G(c, ic, v, 1) + c->st_coef[2 * k + 1] * (P(c, jc, v) - P(c, ic, v)) * c->st_w[k];
      }
    }
  } else if (m == FVS_GRAD_GGCB) { /* grad_ggcb, src/gradient_ggcb.f90:116-138 */
    for (int v = 0; v < NV; v++) {
      double gx = c->coef0[ic][0] * P(c, ic, v), gy = c->coef0[ic][1] * P(c, ic, v);
      for (int k = c->st_ptr[ic]; k < c->st_ptr[ic + 1]; k++) {
        int ic1 = c->st_cell[k];
        gx = gx + c->st_coef[2 * k] * P(c, ic1, v);
        gy = gy + c->st_coef[2 * k + 1] * P(c, ic1, v);
      }
      G(c, ic, v, 0) = gx / c->vol[ic];
      G(c, ic, v, 1) = gy / c->vol[ic];
    }
  } else { /* grad_ggnb, src/gradient_ggnb.f90:183-210 */
    for (int v = 0; v < NV; v++) {
      double gx = c->coef0[ic][0] * P(c, ic, v), gy = c->coef0[ic][1] * P(c, ic, v);
      int i = c->st_ptr[ic];
      for (int in = 1; in <= c->nvrt[ic]; in++) {
        int iv = c->cnode[ic][in];
        for (int j = 1; j <= c->nd_nc[iv]; j++) {
          int jc = c->st_cell[i];
          gx = gx + c->coefedg[ic][in][0] * c->st_coef[i] * P(c, jc, v);
          gy = gy + c->coefedg[ic][in][1] * c->st_coef[i] * P(c, jc, v);
          i++;
        }
      }
      G(c, ic, v, 0) = gx / c->vol[ic];
      G(c, ic, v, 1) = gy / c->vol[ic];
    }
  }
}

/* limiter, src/gradient_limiter.f90:103-134; eps2 precomputed per cell */
static inline double limiter_fn(int type, double a, double b, double eps2) {
  if (type == FVS_LIM_VENK) return ((a * a + eps2) + 2.0 * b * a) / (a * a + 2.0 * (b * b) + a * b + eps2);
  if (type == FVS_LIM_BARTH) { double q = a / b; return q < 1.0 ? q : 1.0; }
  double l = ((b * b + eps2) * a + (a * a + eps2) * b) / (a * a + b * b + 2.0 * eps2);
  return l / (b + eps2);
}

/* compute_gradient_limiter for one cell, src/gradient_limiter.f90:47-88 */
static void limiter_cell(orc* c, int ic) {
  double phimin = 0.0;
  for (int v = 0; v < NV; v++) {
    double pc = P(c, ic, v), pmin = pc, pmax = pc;
    for (int k = c->st_ptr[ic]; k < c->st_ptr[ic + 1]; k++) {
      double pj = P(c, c->st_cell[k], v);
      pmin = pj < pmin ? pj : pmin;
      pmax = pj > pmax ? pj : pmax;
    }
    double phi_edge[4] = {100.0, 100.0, 100.0, 100.0};
    for (int ie = 1; ie <= c->nvrt[ic]; ie++) {
      int je = c->cedge[ic][ie];
      double pf = pc + mix(c, c->ex[je] - c->xc[ic]) * G(c, ic, v, 0) + miy(c, c->ey[je] - c->yc[ic]) * G(c, ic, v, 1);
      double dmax = pmax - pc, dmin = pmin - pc, diff = pf - pc;
      if (diff > 0.0) phi_edge[ie - 1] = limiter_fn(c->o.limiter, dmax, diff, c->eps2[ic]);
      else if (diff < 0.0) phi_edge[ie - 1] = limiter_fn(c->o.limiter, dmin, diff, c->eps2[ic]);
      else phi_edge[ie - 1] = 1.0;
    }
    double mv = phi_edge[0];
    for (int k = 1; k < 4; k++) if (phi_edge[k] < mv) mv = phi_edge[k];
    double ph = mv < 1.0 ? mv : 1.0;
    if (v == 0 || ph < phimin) phimin = ph;
  }
  c->phi[ic] = phimin;
}

/* flux_invscid_roe, src/flux_invscid.f90:37-136 */
static void roe_flux(double gamma, const double* pL_, const double* pR_, double nx, double ny, double* flux, double* ws_max) {
  double tx = -ny, ty = nx;
  double rhoL = pL_[0], uL = pL_[1], vL = pL_[2], pL = pL_[3];
  double rhoR = pR_[0], uR = pR_[1], vR = pR_[2], pR = pR_[3];
  double unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
  double utL = uL * tx + vL * ty, utR = uR * tx + vR * ty;
  double aL = sqrt(gamma * pL / rhoL), aR = sqrt(gamma * pR / rhoR);
  double kL = 0.5 * (uL * uL + vL * vL), kR = 0.5 * (uR * uR + vR * vR);
  double HL = aL * aL / (gamma - 1.0) + kL, HR = aR * aR / (gamma - 1.0) + kR;
  double RT = sqrt(rhoR / rhoL);
  double rho = RT * rhoL;
  double u = (uL + RT * uR) / (1.0 + RT);
  double v = (vL + RT * vR) / (1.0 + RT);
  double H = (HL + RT * HR) / (1.0 + RT);
  double a = sqrt((gamma - 1.0) * (H - 0.5 * (u * u + v * v)));
  double un = u * nx + v * ny;
  double ut = u * tx + v * ty;
  double drho = rhoR - rhoL, dp = pR - pL, dun = unR - unL, dut = utR - utL;
  double LdU[4], ws[4], Rv[4][4], diss[4], fL[4], fR[4];
  LdU[0] = (dp - rho * a * dun) / (2.0 * a * a);
  LdU[1] = rho * dut;
  LdU[2] = drho - dp / (a * a);
  LdU[3] = (dp + rho * a * dun) / (2.0 * a * a);
  ws[0] = fabs(un - a); ws[1] = fabs(un); ws[2] = fabs(un); ws[3] = fabs(un + a);
  double dws = 1.0 / 5.0;
  if (ws[0] < dws) ws[0] = 0.5 * (ws[0] * ws[0] / dws + dws);
  if (ws[3] < dws) ws[3] = 0.5 * (ws[3] * ws[3] / dws + dws);
  double tke = 0.5 * (u * u + v * v);
  Rv[0][0] = 1.0;          Rv[0][1] = 0.0; Rv[0][2] = 1.0; Rv[0][3] = 1.0;
  Rv[1][0] = u - a * nx;   Rv[1][1] = tx;  Rv[1][2] = u;   Rv[1][3] = u + a * nx;
  Rv[2][0] = v - a * ny;   Rv[2][1] = ty;  Rv[2][2] = v;   Rv[2][3] = v + a * ny;
  Rv[3][0] = H - un * a;   Rv[3][1] = ut;  Rv[3][2] = tke; Rv[3][3] = H + un * a;
  for (int i = 0; i < 4; i++) {
    diss[i] = 0.0;
    for (int j = 0; j < 4; j++) diss[i] = diss[i] + ws[j] * LdU[j] * Rv[i][j];
  }
  fL[0] = rhoL * unL;
  fL[1] = rhoL * unL * uL + pL * nx;
  fL[2] = rhoL * unL * vL + pL * ny;
  fL[3] = rhoL * unL * HL;
  fR[0] = rhoR * unR;
  fR[1] = rhoR * unR * uR + pR * nx;
  fR[2] = rhoR * unR * vR + pR * ny;
  fR[3] = rhoR * unR * HR;
  for (int i = 0; i < 4; i++) flux[i] = 0.5 * (fL[i] + fR[i] - 1.0 * diss[i]);
  *ws_max = 0.5 * (fabs(un) + a);
}

/* bc_flux, src/residual.f90:183-255 */
static void bc_state(const orc* c, double time, double x, double y, double nx, double ny, int type,
                     const double* pfL, double* pfR) {
  for (int k = 0; k < 4; k++) pfR[k] = 0.0;
  if (type == FVS_BC_FREESTREAM) {
    for (int k = 0; k < 4; k++) pfR[k] = c->pvar_inf[k];
  } else if (type == FVS_BC_SLIP_WALL) {
    for (int k = 0; k < 4; k++) pfR[k] = pfL[k];
    double un = pfL[1] * nx + pfL[2] * ny;
    pfR[1] = pfL[1] - 2.0 * un * nx;
    pfR[2] = pfL[2] - 2.0 * un * ny;
  } else { /* dirichlet */
    if (c->o.vortex) vortex_state(c, time, x, y, pfR);
    else { double rhs[4]; mms_euler2d(c, x, y, pfR, rhs); }
  }
}

/* face reconstruction + flux of interior edge ie, src/residual.f90:67-95 */
static void interior_flux(const orc* c, int ie, double* flux, double* ws_max) {
  double xf = c->ex[ie], yf = c->ey[ie], nxf = c->enx[ie], nyf = c->eny[ie];
  int icL = c->ec1[ie], icR = c->ec2[ie];
  double dxL = mix(c, xf - c->xc[icL]), dyL = miy(c, yf - c->yc[icL]);
  double dxR = mix(c, xf - c->xc[icR]), dyR = miy(c, yf - c->yc[icR]);
  double k = c->o.umuscl, pfL[4], pfR[4];
  const double* pl = &c->pvar[4 * icL];
  const double* pr = &c->pvar[4 * icR];
  for (int v = 0; v < NV; v++) {
    double gradC = pr[v] - pl[v];
    double gradL = dxL * G(c, icL, v, 0) + dyL * G(c, icL, v, 1);
    double gradR = dxR * G(c, icR, v, 0) + dyR * G(c, icR, v, 1);
    pfL[v] = pl[v] + c->phi[icL] * (k / 2.0 * gradC + (1.0 - k) * gradL);
    pfR[v] = pr[v] + c->phi[icR] * (-k / 2.0 * gradC + (1.0 - k) * gradR);
  }
  roe_flux(c->o.gamma, pfL, pfR, nxf, nyf, flux, ws_max);
}

/* boundary edge i of boundary ib (1-based), src/residual.f90:116-142 */
static void boundary_flux(const orc* c, double time, int ib, int i, int* icL_out, double* flux, double* ws_max) {
  int ie = c->b_edge[c->b_eptr[ib] + i];
  int icL = c->b_cell[c->b_cptr[ib] + i - 1];
  double xf = c->ex[ie], yf = c->ey[ie], nxf = c->enx[ie], nyf = c->eny[ie];
  double dx = mix(c, xf - c->xc[icL]), dy = miy(c, yf - c->yc[icL]);
  double pfL[4], pfR[4];
  for (int v = 0; v < NV; v++)
    pfL[v] = P(c, icL, v) + c->phi[icL] * (dx * G(c, icL, v, 0) + dy * G(c, icL, v, 1));
  bc_state(c, time, xf, yf, nxf, nyf, c->b_type[ib], pfL, pfR);
  roe_flux(c->o.gamma, pfL, pfR, nxf, nyf, flux, ws_max);
  *icL_out = icL;
}

static int nthreads_eff(int n) { return n < 1 ? 1 : n; }

/* compute_residual, src/residual.f90:23-177 */
static void compute_residual(orc* c, double time, int nthreads) {
  int nc = c->ncells;
  int nt = nthreads_eff(nthreads);
  (void)nt;
  int first_order = (c->o.reconst == FVS_RECON_UPWIND1);
  /* zero :37-40, cvar2pvar :46 */
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
  for (int ic = 1; ic <= nc; ic++) {
    for (int v = 0; v < NV; v++) { R(c, ic, v) = 0.0; G(c, ic, v, 0) = 0.0; G(c, ic, v, 1) = 0.0; }
    c->phi[ic] = 0.0; c->ws[ic] = 0.0;
    cvar2pvar_cell(c, ic);
  }
  /* gradient :52 (no-op for first order, src/gradient.f90:49) */
  if (!first_order) {
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
    for (int ic = 1; ic <= nc; ic++) gradient_cell(c, ic);
  }
  /* limiter :58 */
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
  for (int ic = 1; ic <= nc; ic++) {
    if (first_order) c->phi[ic] = 0.0;
    else if (c->o.limiter == FVS_LIM_NONE) c->phi[ic] = 1.0;
    else limiter_cell(c, ic);
  }
  if (nthreads <= 1) {
    /* the reference's sequential edge loops :66-157 */
    for (int i = 1; i <= c->nedges_intr; i++) {
      int ie = c->edge_intr[i];
      double flux[4], ws_max;
      interior_flux(c, ie, flux, &ws_max);
      double af = c->ea[ie];
      int icL = c->ec1[ie], icR = c->ec2[ie];
      for (int v = 0; v < NV; v++) {
        R(c, icL, v) = R(c, icL, v) + flux[v] * af;
        R(c, icR, v) = R(c, icR, v) - flux[v] * af;
      }
      c->ws[icL] = c->ws[icL] + ws_max * af;
      c->ws[icR] = c->ws[icR] + ws_max * af;
    }
    for (int ib = 1; ib <= c->nb; ib++)
      for (int i = 1; i <= c->b_nedges[ib]; i++) {
        int icL, ie = c->b_edge[c->b_eptr[ib] + i];
        double flux[4], ws_max;
        boundary_flux(c, time, ib, i, &icL, flux, &ws_max);
        double af = c->ea[ie];
        for (int v = 0; v < NV; v++) R(c, icL, v) = R(c, icL, v) + flux[v] * af;
        c->ws[icL] = c->ws[icL] + ws_max * af;
      }
  } else {
    /* race-free variant: fluxes into per-edge slots, then a per-cell gather
     * in the same summation order as the loops above (bit-identical) */
    int nint = c->nedges_intr;
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int i = 1; i <= nint; i++) {
      int ie = c->edge_intr[i];
      double flux[4], ws_max, af = c->ea[ie];
      interior_flux(c, ie, flux, &ws_max);
      double* s = &c->eflux[5 * (i - 1)];
      for (int v = 0; v < NV; v++) s[v] = flux[v] * af;
      s[4] = ws_max * af;
    }
    int nbe = c->b_eptr[c->nb + 1];
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int k = 0; k < nbe; k++) {
      int ib = 1;
      while (c->b_eptr[ib + 1] <= k) ib++;
      int i = k - c->b_eptr[ib] + 1, icL, ie = c->b_edge[k + 1];
      double flux[4], ws_max, af = c->ea[ie];
      boundary_flux(c, time, ib, i, &icL, flux, &ws_max);
      double* s = &c->eflux[5 * (nint + k)];
      for (int v = 0; v < NV; v++) s[v] = flux[v] * af;
      s[4] = ws_max * af;
    }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int ic = 1; ic <= nc; ic++) {
      for (int j = 0; j < c->ncl[ic]; j++) {
        int e = c->clist[8 * ic + j];
        const double* s = &c->eflux[5 * ((e > 0 ? e : -e) - 1)];
        if (e > 0) for (int v = 0; v < NV; v++) R(c, ic, v) = R(c, ic, v) + s[v];
        else for (int v = 0; v < NV; v++) R(c, ic, v) = R(c, ic, v) - s[v];
        c->ws[ic] = c->ws[ic] + s[4];
      }
    }
  }
  /* resid = -resid/vol :164-166 */
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
  for (int ic = 1; ic <= nc; ic++)
    for (int v = 0; v < NV; v++) R(c, ic, v) = -R(c, ic, v) / c->vol[ic];
}

/* ========================================================================= */
/* Runge-Kutta, src/runge_kutta.f90                                          */
/* ========================================================================= */
static void rk_coeffs(orc* c) {
  double dt = c->dt;
  int ns = c->o.rk_nstages, ord = c->o.rk_order;
  if (ns == 4) { /* :36-51 */
    double ak = 0, bk = 0, ck = 0, dk = 0;
    if (ord == 1) { ak = 3.60897; bk = 2.04; ck = 0.34206; dk = 0.00897; }
    else if (ord == 2) { ak = 0.11; bk = 3.92; ck = 1.86; dk = 0.11; }
    else if (ord == 3) { ak = 0.65; bk = 2.7; ck = 2.0; dk = 0.65; }
    else if (ord == 4) { ak = 1.0; bk = 2.0; ck = 2.0; dk = 1.0; }
    c->h_rk[1] = dt / 2.0; c->rk_coef[1] = ak;
    c->h_rk[2] = dt / 2.0; c->rk_coef[2] = bk;
    c->h_rk[3] = dt;       c->rk_coef[3] = ck;
    c->h_rk[4] = dt / 6.0; c->rk_coef[4] = dk;
  }
  if (ns == 4 && ord == 2 && c->o.ssprk) { /* :57-67 */
    c->h_rk[1] = dt / 3.0; c->rk_coef[1] = 1.0;
    c->h_rk[2] = dt / 3.0; c->rk_coef[2] = 1.0;
    c->h_rk[3] = dt / 3.0; c->rk_coef[3] = 1.0;
    c->h_rk[4] = dt / 4.0; c->rk_coef[4] = 1.0;
    c->dts[1] = 0.0;            c->dte[1] = dt / 3.0;
    c->dts[2] = dt / 3.0;       c->dte[2] = dt * 2.0 / 3.0;
    c->dts[3] = dt * 2.0 / 3.0; c->dte[3] = dt;
    c->dts[4] = dt;             c->dte[4] = dt;
  }
  if (ns == 3 && c->o.ssprk) { /* extension: Shu-Osher SSP-RK3 stage times */
    c->dts[1] = 0.0; c->dts[2] = dt; c->dts[3] = dt / 2.0;
  }
}

/* compute_local_time, src/runge_kutta.f90:424-437 */
static void compute_local_time(orc* c, int nt) {
  (void)nt;
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
  for (int ic = 1; ic <= c->ncells; ic++) c->dt_local[ic] = c->o.cfl * c->vol[ic] / (0.5 * c->ws[ic]);
}

static void rms_norm(const orc* c, const double* cvar0, double* out4) {
  for (int v = 0; v < NV; v++) {
    double s = 0.0;
    for (int ic = 1; ic <= c->ncells; ic++) {
      double d = fabs(U(c, ic, v) - cvar0[4 * ic + v]);
      s = s + d * d;
    }
    out4[v] = sqrt(s / (double)c->ncells);
  }
}

static void ensure_dt(orc* c, double t1, int nt) {
  if (c->dt_ready) return;
  if (c->o.dt_from_cfl && !c->o.steady) {
    compute_residual(c, t1, nt);
    double dmin = 0.0;
    for (int ic = 1; ic <= c->ncells; ic++) {
      double d = c->o.cfl * c->vol[ic] / (0.5 * c->ws[ic]);
      if (ic == 1 || d < dmin) dmin = d;
    }
    c->dt = dmin;
  }
  rk_coeffs(c);
  c->dt_ready = 1;
}

int orc_time_integration(orc* c, double t1, int nsteps, double* resnorm, int nthreads) {
  int nc = c->ncells, nt = nthreads_eff(nthreads);
  (void)nt;
  ensure_dt(c, t1, nthreads);
  int ns = c->o.rk_nstages, steady = c->o.steady, ssp = c->o.ssprk;
  size_t n4 = 4 * (size_t)(nc + 1);
  double* cvar0 = (double*)malloc(sizeof(double) * n4);
  double* fcvar = (double*)malloc(sizeof(double) * n4);
  double dt = c->dt;
  for (int istep = 1; istep <= nsteps; istep++) {
    double told = t1 + (double)(istep - 1) * dt;
    double tst[5] = {0, told, told + 0.5 * dt, told + 0.5 * dt, told + dt};
    c->icont++;
    memcpy(cvar0, c->cvar, sizeof(double) * n4);
    memset(fcvar, 0, sizeof(double) * n4);
    for (int rk = 1; rk <= ns; rk++) {
      double tstart = ssp ? told + c->dts[rk] : tst[rk];
      compute_residual(c, tstart, nthreads);
      if (steady && rk == 1) compute_local_time(c, nthreads);
      if (ns == 3) {
        /* extension: SSP-RK3, U_k+1 = a*U0 + b*(U_k + h*R) */
        static const double A[4] = {0, 0.0, 0.75, 1.0 / 3.0}, B[4] = {0, 1.0, 0.25, 2.0 / 3.0};
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
        for (int ic = 1; ic <= nc; ic++) {
          double h = steady ? c->dt_local[ic] : dt;
          for (int v = 0; v < NV; v++) {
            double s = U(c, ic, v) + h * R(c, ic, v);
            U(c, ic, v) = rk == 1 ? s : A[rk] * cvar0[4 * ic + v] + B[rk] * s;
          }
        }
      } else if (ssp && !steady) { /* time_integ_SSPRK :223-226 */
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
        for (int ic = 1; ic <= nc; ic++)
          for (int v = 0; v < NV; v++) {
            size_t k = 4 * (size_t)ic + v;
            c->cvar[k] = cvar0[k] + c->h_rk[rk] * (c->rk_coef[rk] * c->resid[k] + fcvar[k]);
            fcvar[k] = fcvar[k] + c->resid[k];
          }
      } else if (ssp && steady) { /* time_integ_SSPRK_steady :381-387 */
        double cst = 1.0 / 3.0;
        if (rk == 4) cst = 1.0 / 4.0;
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
        for (int ic = 1; ic <= nc; ic++)
          for (int v = 0; v < NV; v++) {
            size_t k = 4 * (size_t)ic + v;
            c->cvar[k] = cvar0[k] + c->dt_local[ic] * cst * (c->rk_coef[rk] * c->resid[k] + fcvar[k]);
            fcvar[k] = fcvar[k] + c->resid[k];
          }
      } else if (!steady) { /* time_integ_RK :154-162 */
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
        for (int ic = 1; ic <= nc; ic++)
          for (int v = 0; v < NV; v++) {
            size_t k = 4 * (size_t)ic + v;
            fcvar[k] = fcvar[k] + c->rk_coef[rk] * c->resid[k];
            if (rk < ns) c->cvar[k] = cvar0[k] + c->h_rk[rk] * c->resid[k];
            else c->cvar[k] = cvar0[k] + c->h_rk[rk] * fcvar[k];
          }
      } else { /* time_integ_RK_steady :296-313 */
        double cst = 1.0 / 2.0;
        if (rk == 3) cst = 1.0;
        if (rk == 4) cst = 1.0 / 6.0;
#pragma omp parallel for num_threads(nt) if (nt > 1) schedule(static)
        for (int ic = 1; ic <= nc; ic++)
          for (int v = 0; v < NV; v++) {
            size_t k = 4 * (size_t)ic + v;
            fcvar[k] = fcvar[k] + c->rk_coef[rk] * c->resid[k];
            if (rk < ns) c->cvar[k] = cvar0[k] + c->dt_local[ic] * cst * c->resid[k];
            else c->cvar[k] = cvar0[k] + c->dt_local[ic] * cst * fcvar[k];
          }
      }
    }
    if (resnorm) rms_norm(c, cvar0, resnorm + 4 * (size_t)(istep - 1));
  }
  free(cvar0); free(fcvar);
  return FVS_OK;
}

/* ========================================================================= */
/* public API                                                                */
/* ========================================================================= */
double orc_dt(const orc* c) { return c->dt; }

int orc_create(const fvs_mesh* m, const fvs_options* o, orc** out, char* err, int errlen) {
  *out = NULL;
  if (!m || !o || m->nnodes <= 0 || m->ncells_tri < 0 || m->ncells_quad < 0 || m->ncells_tri + m->ncells_quad <= 0) {
    set_err(err, errlen, "invalid mesh sizes"); return FVS_ERR_INVALID;
  }
  if (o->flux != 1) { set_err(err, errlen, "only the Roe flux (1) exists"); return FVS_ERR_INVALID; }
  if (o->grad_method < 1 || o->grad_method > 3) { set_err(err, errlen, "grad_method must be 1..3"); return FVS_ERR_INVALID; }
  if (o->limiter < 0 || o->limiter > 3) { set_err(err, errlen, "limiter must be 0..3"); return FVS_ERR_INVALID; }
  if (o->limiter != FVS_LIM_NONE && o->grad_method != FVS_GRAD_LSQ && o->reconst != FVS_RECON_UPWIND1) {
    set_err(err, errlen, "the limiter reads the LSQ stencil (src/gradient_limiter.f90:54): use LSQ gradients");
    return FVS_ERR_INVALID;
  }
  if (o->reconst < 1 || o->reconst > 3) { set_err(err, errlen, "reconst must be 1..3"); return FVS_ERR_INVALID; }
  int ns = o->rk_nstages;
  if (!((ns == 4 && o->rk_order >= 1 && o->rk_order <= 4 && (!o->ssprk || o->rk_order == 2)) || (ns == 3 && o->ssprk))) {
    set_err(err, errlen, "RK coefficients exist for 4 stages (SSP: order 2) and the SSP-RK3 extension only");
    return FVS_ERR_INVALID;
  }
  orc* c = (orc*)calloc(1, sizeof(orc));
  c->o = *o;
  if (o->reconst != FVS_RECON_UMUSCL) c->o.umuscl = 0.0; /* src/input.f90:250,254 */
  c->Lx = m->period_x > 0 ? m->period_x : 0.0;
  c->Ly = m->period_y > 0 ? m->period_y : 0.0;
  c->nnodes = m->nnodes; c->ntri = m->ncells_tri; c->nquad = m->ncells_quad;
  int nc = c->ncells = c->ntri + c->nquad;
  c->xn = (double*)calloc((size_t)c->nnodes + 1, sizeof(double));
  c->yn = (double*)calloc((size_t)c->nnodes + 1, sizeof(double));
  for (int i = 1; i <= c->nnodes; i++) { c->xn[i] = m->node_xy[2 * (i - 1)]; c->yn[i] = m->node_xy[2 * (i - 1) + 1]; }
  c->nvrt = (int*)calloc((size_t)nc + 1, sizeof(int));
  c->cnode = calloc((size_t)nc + 1, sizeof(*c->cnode));
  c->nghbr = calloc((size_t)nc + 1, sizeof(*c->nghbr));
  c->nghbre = calloc((size_t)nc + 1, sizeof(*c->nghbre));
  c->cedge = calloc((size_t)nc + 1, sizeof(*c->cedge));
  c->nrmlsign = calloc((size_t)nc + 1, sizeof(*c->nrmlsign));
  c->xc = (double*)calloc((size_t)nc + 1, sizeof(double));
  c->yc = (double*)calloc((size_t)nc + 1, sizeof(double));
  c->vol = (double*)calloc((size_t)nc + 1, sizeof(double));
  for (int i = 1; i <= c->ntri; i++) {
    c->nvrt[i] = 3;
    for (int k = 1; k <= 3; k++) c->cnode[i][k] = m->tri_nodes[3 * (i - 1) + k - 1];
  }
  for (int i = 1; i <= c->nquad; i++) {
    int ic = c->ntri + i;
    c->nvrt[ic] = 4;
    for (int k = 1; k <= 4; k++) c->cnode[ic][k] = m->quad_nodes[4 * (i - 1) + k - 1];
  }
  for (int ic = 1; ic <= nc; ic++)
    for (int k = 1; k <= c->nvrt[ic]; k++)
      if (c->cnode[ic][k] < 1 || c->cnode[ic][k] > c->nnodes) {
        set_err(err, errlen, "cell %d node %d out of range", ic, c->cnode[ic][k]); orc_destroy(c); return FVS_ERR_MESH;
      }
  c->nb = m->nbndries;
  c->b_ncells = (int*)calloc((size_t)c->nb + 1, sizeof(int));
  c->b_type = (int*)calloc((size_t)c->nb + 1, sizeof(int));
  c->b_cptr = (int*)calloc((size_t)c->nb + 2, sizeof(int));
  int tot = 0;
  for (int ib = 1; ib <= c->nb; ib++) {
    c->b_ncells[ib] = m->bndry_ncells[ib - 1];
    c->b_type[ib] = m->bndry_type[ib - 1];
    c->b_cptr[ib] = tot;
    tot += c->b_ncells[ib];
    int t = c->b_type[ib];
    if (t != FVS_BC_FREESTREAM && t != FVS_BC_SLIP_WALL && t != FVS_BC_DIRICHLET) {
      set_err(err, errlen, "boundary %d: type %d not implemented (src/residual.f90:206-220)", ib, t);
      orc_destroy(c); return FVS_ERR_INVALID;
    }
  }
  c->b_cell = (int*)calloc((size_t)tot + 1, sizeof(int));
  for (int i = 0; i < tot; i++) c->b_cell[i] = m->bndry_cells[i];
  int rc = grid_data(c, err, errlen);
  if (rc != FVS_OK) { orc_destroy(c); return rc; }
  /* solution arrays, src/data_solution.f90:41-66 */
  size_t n4 = 4 * (size_t)(nc + 1);
  c->pvar = (double*)calloc(n4, sizeof(double));
  c->cvar = (double*)calloc(n4, sizeof(double));
  c->resid = (double*)calloc(n4, sizeof(double));
  c->grad = (double*)calloc(2 * n4, sizeof(double));
  c->phi = (double*)calloc((size_t)nc + 1, sizeof(double));
  c->ws = (double*)calloc((size_t)nc + 1, sizeof(double));
  c->dt_local = (double*)calloc((size_t)nc + 1, sizeof(double));
  double aoa = o->aoa_inf_deg * PI / 180.0;
  c->pvar_inf[0] = 1.0;
  c->pvar_inf[1] = o->mach_inf * cos(aoa);
  c->pvar_inf[2] = o->mach_inf * sin(aoa);
  c->pvar_inf[3] = 1.0 / o->gamma;
  /* gradient operator, src/gradient.f90:18-38 */
  if (o->grad_method == FVS_GRAD_LSQ) {
    rc = o->lsq_stencil == FVS_LSQ_NN ? setup_nn(c, err, errlen) : setup_fn(c, err, errlen);
    if (rc == FVS_OK) rc = lsq_verify(c, err, errlen);
  } else if (o->grad_method == FVS_GRAD_GGCB) setup_ggcb(c);
  else setup_ggnb(c);
  if (rc != FVS_OK) { orc_destroy(c); return rc; }
  /* limiter eps^2 per cell, src/gradient_limiter.f90:113-126 */
  c->eps2 = (double*)calloc((size_t)nc + 1, sizeof(double));
  for (int ic = 1; ic <= nc; ic++) {
    double h = 2.0 * sqrt(c->vol[ic] / PI);
    double t = (o->limiter == FVS_LIM_ALBADA ? 0.3 : 5.0) * h;
    c->eps2[ic] = t * t * t;
  }
  /* MMS, src/mms.f90:32-118 */
  mms_constants(c->mc);
  c->mms_sol = (double*)calloc(n4, sizeof(double));
  c->mms_src = (double*)calloc(n4, sizeof(double));
  for (int ic = 1; ic <= nc; ic++) mms_euler2d(c, c->xc[ic], c->yc[ic], &c->mms_sol[4 * ic], &c->mms_src[4 * ic]);
  /* RK, src/runge_kutta.f90:25-88 */
  c->dt = o->dt;
  for (int ic = 1; ic <= nc; ic++) c->dt_local[ic] = o->dt;
  /* race-free residual gather lists (same order as the sequential loops) */
  int nbe = c->b_eptr[c->nb + 1];
  c->eflux = (double*)calloc(5 * (size_t)(c->nedges_intr + nbe) + 5, sizeof(double));
  c->clist = (int*)calloc(8 * (size_t)(nc + 1), sizeof(int));
  c->ncl = (int*)calloc((size_t)nc + 1, sizeof(int));
  for (int i = 1; i <= c->nedges_intr; i++) {
    int ie = c->edge_intr[i];
    int a = c->ec1[ie], b = c->ec2[ie];
    c->clist[8 * a + c->ncl[a]++] = i;
    c->clist[8 * b + c->ncl[b]++] = -i;
  }
  for (int k = 0; k < nbe; k++) {
    int ib = 1;
    while (c->b_eptr[ib + 1] <= k) ib++;
    int i = k - c->b_eptr[ib] + 1;
    int a = c->b_cell[c->b_cptr[ib] + i - 1];
    if (c->ncl[a] >= 8) { set_err(err, errlen, "cell %d has more than 8 flux contributions", a); orc_destroy(c); return FVS_ERR_MESH; }
    c->clist[8 * a + c->ncl[a]++] = c->nedges_intr + k + 1;
  }
  *out = c;
  return FVS_OK;
}

void orc_destroy(orc* c) {
  if (!c) return;
  kd_free_node(c->tree.root); free(c->tree.ind); free(c->kd_xy);
  void* ptrs[] = {c->xn, c->yn, c->nvrt, c->cnode, c->nghbr, c->nghbre, c->cedge, c->xc, c->yc, c->vol, c->nrmlsign,
                  c->nd_nc, c->nd_ptr, c->nd_cell, c->en1, c->en2, c->ec1, c->ec2, c->ex, c->ey, c->ea, c->enx,
                  c->eny, c->etx, c->ety, c->cell_intr, c->cell_bndr, c->edge_intr, c->edge_bndr, c->bedge_cell,
                  c->b_ncells, c->b_nedges, c->b_type, c->b_cptr, c->b_eptr, c->b_cell, c->b_edge, c->st_ptr,
                  c->st_cell, c->st_coef, c->st_w, c->coef0, c->coefedg, c->eps2, c->pvar, c->cvar, c->grad,
                  c->resid, c->phi, c->ws, c->mms_sol, c->mms_src, c->dt_local, c->eflux, c->clist, c->ncl};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
  free(c);
}

int orc_sizes(const orc* c, fvs_sizes* s) {
  memset(s, 0, sizeof(*s));
  s->nnodes = c->nnodes; s->ncells = c->ncells; s->ncells_tri = c->ntri; s->ncells_quad = c->nquad;
  s->nedges = c->nedges; s->nedges_intr = c->nedges_intr; s->nedges_bndr = c->nedges_bndr;
  s->ncells_intr = c->ncells_intr; s->ncells_bndr = c->ncells_bndr; s->nbndries = c->nb;
  s->stencil_len = c->st_len; s->nstages = c->o.rk_nstages;
  s->heff1 = c->heff1; s->heff2 = c->heff2; s->vol_sum = c->vol1; s->vol_green = c->vol2; s->dt = c->dt;
  return FVS_OK;
}

/* named exports: reference-order arrays, 1-based ids, 0-based CSR offsets */
static int export_impl(const orc* c, const char* name, void* dst, int64_t* nbytes) {
  int nc = c->ncells, ne = c->nedges;
#define EXP(cond, bytes, fill) \
  if (cond) { int64_t nb_ = (int64_t)(bytes); if (!dst) { *nbytes = nb_; return FVS_OK; } if (*nbytes < nb_) return FVS_ERR_INVALID; fill; return FVS_OK; }
  int32_t* I = (int32_t*)dst;
  double* D = (double*)dst;
  EXP(!strcmp(name, "cell_xy"), 16 * nc, for (int i = 1; i <= nc; i++) { D[2 * i - 2] = c->xc[i]; D[2 * i - 1] = c->yc[i]; })
  EXP(!strcmp(name, "cell_vol"), 8 * nc, for (int i = 1; i <= nc; i++) D[i - 1] = c->vol[i])
  EXP(!strcmp(name, "cell_nghbr"), 16 * nc, for (int i = 1; i <= nc; i++) for (int k = 1; k <= 4; k++) I[4 * (i - 1) + k - 1] = k <= c->nvrt[i] ? c->nghbr[i][k] : -1)
  EXP(!strcmp(name, "cell_nghbre"), 16 * nc, for (int i = 1; i <= nc; i++) for (int k = 1; k <= 4; k++) I[4 * (i - 1) + k - 1] = k <= c->nvrt[i] ? c->nghbre[i][k] : -1)
  EXP(!strcmp(name, "cell_edge"), 16 * nc, for (int i = 1; i <= nc; i++) for (int k = 1; k <= 4; k++) I[4 * (i - 1) + k - 1] = k <= c->nvrt[i] ? c->cedge[i][k] : -1)
  EXP(!strcmp(name, "cell_nrmlsign"), 32 * nc, for (int i = 1; i <= nc; i++) for (int k = 1; k <= 4; k++) D[4 * (i - 1) + k - 1] = k <= c->nvrt[i] ? c->nrmlsign[i][k] : 0.0)
  EXP(!strcmp(name, "edge_nodes"), 8 * ne, for (int i = 1; i <= ne; i++) { I[2 * i - 2] = c->en1[i]; I[2 * i - 1] = c->en2[i]; })
  EXP(!strcmp(name, "edge_cells"), 8 * ne, for (int i = 1; i <= ne; i++) { I[2 * i - 2] = c->ec1[i]; I[2 * i - 1] = c->ec2[i]; })
  EXP(!strcmp(name, "edge_geom"), 56 * ne, for (int i = 1; i <= ne; i++) { double* g = D + 7 * (i - 1); g[0] = c->ex[i]; g[1] = c->ey[i]; g[2] = c->ea[i]; g[3] = c->enx[i]; g[4] = c->eny[i]; g[5] = c->etx[i]; g[6] = c->ety[i]; })
  EXP(!strcmp(name, "edge_intr"), 4 * c->nedges_intr, for (int i = 1; i <= c->nedges_intr; i++) I[i - 1] = c->edge_intr[i])
  EXP(!strcmp(name, "edge_bndr"), 4 * c->nedges_bndr, for (int i = 1; i <= c->nedges_bndr; i++) I[i - 1] = c->edge_bndr[i])
  EXP(!strcmp(name, "bedge_cell"), 4 * c->nedges_bndr, for (int i = 1; i <= c->nedges_bndr; i++) I[i - 1] = c->bedge_cell[i])
  EXP(!strcmp(name, "cell_intr"), 4 * c->ncells_intr, for (int i = 1; i <= c->ncells_intr; i++) I[i - 1] = c->cell_intr[i])
  EXP(!strcmp(name, "cell_bndr"), 4 * c->ncells_bndr, for (int i = 1; i <= c->ncells_bndr; i++) I[i - 1] = c->cell_bndr[i])
  EXP(!strcmp(name, "bndry_edges"), 4 * c->b_eptr[c->nb + 1], for (int i = 1; i <= c->b_eptr[c->nb + 1]; i++) I[i - 1] = c->b_edge[i])
  EXP(!strcmp(name, "stencil_ptr"), 4 * (nc + 1), for (int i = 1; i <= nc + 1; i++) I[i - 1] = c->st_ptr[i])
  EXP(!strcmp(name, "stencil_cell"), 4 * c->st_len, for (int i = 0; i < c->st_len; i++) I[i] = c->st_cell[i])
  EXP(!strcmp(name, "stencil_coef") && c->o.grad_method != FVS_GRAD_GGNB, 16 * c->st_len, memcpy(D, c->st_coef, 16 * (size_t)c->st_len))
  EXP(!strcmp(name, "stencil_coef") && c->o.grad_method == FVS_GRAD_GGNB, 8 * c->st_len, memcpy(D, c->st_coef, 8 * (size_t)c->st_len))
  EXP(!strcmp(name, "stencil_w") && c->o.grad_method == FVS_GRAD_LSQ, 8 * c->st_len, memcpy(D, c->st_w, 8 * (size_t)c->st_len))
  EXP(!strcmp(name, "coef0") && c->coef0, 16 * nc, for (int i = 1; i <= nc; i++) { D[2 * i - 2] = c->coef0[i][0]; D[2 * i - 1] = c->coef0[i][1]; })
  EXP(!strcmp(name, "coefedg") && c->coefedg, 64 * nc, for (int i = 1; i <= nc; i++) for (int k = 1; k <= 4; k++) { D[8 * (i - 1) + 2 * (k - 1)] = k <= c->nvrt[i] ? c->coefedg[i][k][0] : 0.0; D[8 * (i - 1) + 2 * (k - 1) + 1] = k <= c->nvrt[i] ? c->coefedg[i][k][1] : 0.0; })
  EXP(!strcmp(name, "eps2"), 8 * nc, for (int i = 1; i <= nc; i++) D[i - 1] = c->eps2[i])
#undef EXP
  return FVS_ERR_INVALID;
}
int orc_export_size(const orc* c, const char* name, int64_t* nbytes) { return export_impl(c, name, NULL, nbytes); }
int orc_export(const orc* c, const char* name, void* dst, int64_t nbytes) {
  if (!dst) return FVS_ERR_INVALID;
  return export_impl(c, name, dst, &nbytes);
}

/* initialize_solution, src/initialize.f90:19-90 (ntstart <= 1) */
int orc_init_state(orc* c) {
  int nc = c->ncells;
  double t_initial = (double)(c->o.ntstart - 1) * c->o.dt;
  for (int ic = 1; ic <= nc; ic++) {
    double pv[4];
    if (c->o.ntstart < 1) memcpy(pv, &c->mms_sol[4 * ic], sizeof(pv));
    else if (c->o.vortex) vortex_state(c, t_initial, c->xc[ic], c->yc[ic], pv);
    else memcpy(pv, c->pvar_inf, sizeof(pv));
    memcpy(&c->pvar[4 * ic], pv, sizeof(pv));
    prim2cnsr(c->o.gamma, pv, &c->cvar[4 * ic]);
  }
  return FVS_OK;
}

int orc_set_state(orc* c, const double* cvar) { memcpy(c->cvar + 4, cvar, sizeof(double) * 4 * (size_t)c->ncells); return FVS_OK; }
int orc_get_state(const orc* c, double* cvar) { memcpy(cvar, c->cvar + 4, sizeof(double) * 4 * (size_t)c->ncells); return FVS_OK; }

int orc_residual(orc* c, double time, double* resid, double* ws, int nthreads) {
  compute_residual(c, time, nthreads);
  if (resid) memcpy(resid, c->resid + 4, sizeof(double) * 4 * (size_t)c->ncells);
  if (ws) memcpy(ws, c->ws + 1, sizeof(double) * (size_t)c->ncells);
  return FVS_OK;
}

int orc_get_gradient(const orc* c, double* grad, double* phi) {
  int nc = c->ncells;
  if (grad)
    for (int d = 0; d < 2; d++)
      for (int ic = 1; ic <= nc; ic++)
        for (int v = 0; v < NV; v++) grad[(size_t)d * 4 * nc + 4 * (ic - 1) + v] = G(c, ic, v, d);
  if (phi) memcpy(phi, c->phi + 1, sizeof(double) * (size_t)nc);
  return FVS_OK;
}

/* write_inst_cp_un, src/io.f90:340-446: wall pressure coefficient and loads
 * of boundary ib (1-based, slip_wall).  The face values use the cell-centre
 * gradients of p, u, v from gradient_cellcntr_1var (src/gradient.f90:75-96),
 * the configured gradient without limiter, computed also for first-order
 * runs; the 1-variable routines (src/gradient_lsq.f90:425-441,
 * src/gradient_ggcb.f90:144-166, src/gradient_ggnb.f90:216-243) do the same
 * arithmetic per variable as gradient_cell.  edge_out [nedges][4] =
 * (xf, cp, cp_cell, un) in edge order (may be NULL); loads[11] = cl, cd, cl1,
 * cd1, |Vn|max, |Vn|_2, |Vn|_1, cn, ca, cn1, ca1. */
int orc_wall_loads(orc* c, int ib, double* edge_out, double* loads) {
  if (ib < 1 || ib > c->nb || c->b_type[ib] != FVS_BC_SLIP_WALL || !loads) return FVS_ERR_INVALID;
  for (int ic = 1; ic <= c->ncells; ic++) cvar2pvar_cell(c, ic);
  for (int ic = 1; ic <= c->ncells; ic++) gradient_cell(c, ic);
  const double m = c->o.mach_inf, p_inf = c->pvar_inf[3];
  const int n = c->b_nedges[ib];
  double un_max = 0.0, un_l2 = 0.0, un_l1 = 0.0, cn = 0.0, ca = 0.0, cn1 = 0.0, ca1 = 0.0;
  for (int i = 1; i <= n; i++) {
    int ie = c->b_edge[c->b_eptr[ib] + i];
    int ic = c->b_cell[c->b_cptr[ib] + i - 1];
    double xf = c->ex[ie], af = c->ea[ie], nx = c->enx[ie], ny = c->eny[ie];
    double dx = mix(c, c->ex[ie] - c->xc[ic]), dy = miy(c, c->ey[ie] - c->yc[ic]);
    double pw = P(c, ic, 3) + dx * G(c, ic, 3, 0) + dy * G(c, ic, 3, 1);
    double cp = 2.0 / (m * m) * (pw - p_inf);
    double cp1 = 2.0 / (m * m) * (P(c, ic, 3) - p_inf);
    cn = cn + cp * ny * af;
    ca = ca + cp * nx * af;
    cn1 = cn1 + cp1 * ny * af;
    ca1 = ca1 + cp1 * nx * af;
    double uw = P(c, ic, 1) + dx * G(c, ic, 1, 0) + dy * G(c, ic, 1, 1);
    double vw = P(c, ic, 2) + dx * G(c, ic, 2, 0) + dy * G(c, ic, 2, 1);
    double un = uw * nx + vw * ny;
    un_l2 = un_l2 + un * un;
    un_l1 = un_l1 + fabs(un);
    un_max = un_max > fabs(un) ? un_max : fabs(un);
    if (edge_out) {
      double* e = edge_out + 4 * (size_t)(i - 1);
      e[0] = xf; e[1] = cp; e[2] = cp1; e[3] = un;
    }
  }
  un_l2 = sqrt(un_l2 / (double)n);
  un_l1 = un_l1 / (double)n;
  /* cosd / sind of the angle of attack in degrees */
  const double a = c->o.aoa_inf_deg * PI / 180.0, ca_ = cos(a), sa = sin(a);
  loads[0] = cn * ca_ - ca * sa;
  loads[1] = cn * sa + ca * ca_;
  loads[2] = cn1 * ca_ - ca1 * sa;
  loads[3] = cn1 * sa + ca1 * ca_;
  loads[4] = un_max; loads[5] = un_l2; loads[6] = un_l1;
  loads[7] = cn; loads[8] = ca; loads[9] = cn1; loads[10] = ca1;
  return FVS_OK;
}

/* error_isentropic_vortex, src/mms.f90:271-365 */
int orc_vortex_error(orc* c, double time, double* e) {
  double g = c->o.gamma;
  double mx[4] = {0, 0, 0, 0}, l1[4] = {0, 0, 0, 0}, l2[4] = {0, 0, 0, 0}, L2 = 0.0;
  for (int i = 1; i <= c->ncells_intr; i++) {
    int ic = c->cell_intr[i];
    double pv[4];
    vortex_state(c, time, c->xc[ic], c->yc[ic], pv);
    double ex[4];
    ex[0] = pv[0];
    ex[1] = pv[0] * pv[1];
    ex[2] = pv[0] * pv[2];
    ex[3] = pv[3] / (g - 1.0) + 0.5 * ex[0] * (pv[1] * pv[1] + pv[2] * pv[2]);
    double d[4];
    for (int v = 0; v < 4; v++) {
      d[v] = fabs(U(c, ic, v) - ex[v]);
      if (d[v] > mx[v]) mx[v] = d[v];
      l1[v] = l1[v] + d[v];
      l2[v] = l2[v] + d[v] * d[v];
    }
    L2 = L2 + d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3];
  }
  double n = (double)c->ncells_intr;
  for (int v = 0; v < 4; v++) { e[3 * v] = mx[v]; e[3 * v + 1] = l1[v] / n; e[3 * v + 2] = sqrt(l2[v] / n); }
  e[12] = sqrt(L2 / n);
  return FVS_OK;
}

int orc_mms_source(const orc* c, double* src) {
  memcpy(src, c->mms_src + 4, sizeof(double) * 4 * (size_t)c->ncells);
  return FVS_OK;
}
