/*
 * g6_struct.c -- structure of a few-body system and whether its interaction
 * is over: the decision a multiples hand-off needs between increments of
 * the batched smallN integration (g6x_check_structure, include/g6.h).
 *
 * Restates smallN's check_structure (src/amuse_ph4/src/analyze.cc:866-1070)
 * for a flat system of leaves:
 *   - decompose (analyze.cc:304-348): repeatedly combine the two top-level
 *     nodes of lowest relative energy per unit reduced mass (exact leaf-leaf
 *     potential, analyze.cc:197-233), if negative and if the pair is lightly
 *     perturbed (largest m_k^2 / d_k^6 from the pair's centre of mass below
 *     1e-3 of (M/2)^2 / r^6, analyze.cc:278-302, hdyn.h:283); the centre-of-
 *     mass node takes the first node's place, components relative to it;
 *   - the relative energy of every binary node (analyze.cc:350-371);
 *   - escapers (analyze.cc:373-440): a top-level node is escaping when its
 *     energy relative to every other top-level node is positive, every other
 *     node recedes from it, it recedes from their centre of mass and is
 *     unbound from it (the other nodes' total mass summed in single
 *     precision, as there);
 *   - stability (analyze.cc:567-699): a leaf is stable when escaping, a pair
 *     of leaves when bound; a node with a multiple below it when both sides
 *     are stable, it is bound, and its outer orbit passes the hierarchy test;
 *   - over (analyze.cc:958-998): every top-level node escaping and every one
 *     stable.
 * Differences, by design:
 *   - the hierarchy test of a triple or higher multiple: smallN calls
 *     Mardling's nstab routine (nstab.c, an f2c translation of her code),
 *     which is not restated here.  This file applies the published
 *     Mardling & Aarseth criterion, r_p,out / a_in > 2.8 [(1 + q_out)
 *     (1 + e_out) / sqrt(1 - e_out)]^(2/5), with the linear inclination
 *     factor (23/3 + cos i) / (23/3 + 1) (the "aarseth_stable" form smallN
 *     also evaluates, analyze.cc:506-530), after the two rejections smallN
 *     applies first (outer pericentre inside the inner apocentre, period
 *     ratio below 1).  Decisions agree wherever no multiple above a binary
 *     is tested; the return value says when one was;
 *   - no history: smallN also ends an interaction whose top-level nodes
 *     all escape but are not all stable once the same top-level grouping
 *     has been seen at more than 15 consecutive checks (quasi-stable, a
 *     history kept in file statics, analyze.cc:909-956, 1031-1039).  A call
 *     here is stateless; it reports "every top-level node escaping" in bit
 *     2 and the grouping in the summary, and the caller keeps the history
 *     (amuse_gb300.multiples does, per encounter).
 * The arithmetic follows the reference's expression order (vec.h products
 * summed ((x x + y y) + z z), positions relative to an ancestor summed from
 * the leaf upwards), so energies and decisions are bit-identical for
 * systems of singles and binaries.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "g6.h"

#define ST_MAXN 64
#define ST_NODES (2 * ST_MAXN)

typedef struct {
  double m, x[3], v[3];            /* relative to the parent (absolute at top level) */
  int parent, od, ys, os, leaf;    /* -1: none; leaf: body index or -1 */
  double erel;                     /* relative energy per unit reduced mass */
  int stable, escaper;
} st_node;

typedef struct {
  st_node n[ST_NODES];
  int nn, root;
  int hier_tested; /* a multiple above a binary went through the hierarchy test */
} st_tree;

static double dot3(const double a[3], const double b[3]) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

/* Position / velocity of node k relative to ancestor a: the node's own
   value plus each parent's, from the node upwards (analyze.cc:171-195). */
static void rel_pos(const st_tree *T, int a, int k, double out[3]) {
  for (int c = 0; c < 3; c++) out[c] = T->n[k].x[c];
  while (k != a) {
    const int p = T->n[k].parent;
    for (int c = 0; c < 3; c++) out[c] += T->n[p].x[c];
    k = p;
  }
}
static void rel_vel(const st_tree *T, int a, int k, double out[3]) {
  for (int c = 0; c < 3; c++) out[c] = T->n[k].v[c];
  while (k != a) {
    const int p = T->n[k].parent;
    for (int c = 0; c < 3; c++) out[c] += T->n[p].v[c];
    k = p;
  }
}

/* Leaves of node k in depth-first order (oldest daughter first). */
static int leaves(const st_tree *T, int k, int *out) {
  if (T->n[k].od < 0) {
    out[0] = k;
    return 1;
  }
  int c = 0;
  for (int d = T->n[k].od; d >= 0; d = T->n[d].ys) c += leaves(T, d, out + c);
  return c;
}

/* Potential energy of node i with its sister j, summed over all leaf pairs
   (analyze.cc:197-215). */
static double potential(const st_tree *T, int i, int j) {
  const int p = T->n[i].parent;
  int li[ST_MAXN], lj[ST_MAXN];
  const int ni = leaves(T, i, li), nj = leaves(T, j, lj);
  double phi = 0;
  for (int a = 0; a < ni; a++) {
    double xi[3];
    rel_pos(T, p, li[a], xi);
    for (int b = 0; b < nj; b++) {
      double xj[3], d[3];
      rel_pos(T, p, lj[b], xj);
      for (int c = 0; c < 3; c++) d[c] = xi[c] - xj[c];
      phi -= T->n[li[a]].m * T->n[lj[b]].m / sqrt(dot3(d, d));
    }
  }
  return phi;
}

static double rel_energy(const st_tree *T, int i, int j) {
  const int p = T->n[i].parent;
  double vi[3], vj[3], d[3];
  rel_vel(T, p, i, vi);
  rel_vel(T, p, j, vj);
  const double mi = T->n[i].m, mj = T->n[j].m;
  const double mu_inv = (mi + mj) / (mi * mj);
  for (int c = 0; c < 3; c++) d[c] = vi[c] - vj[c];
  return 0.5 * dot3(d, d) + mu_inv * potential(T, i, j);
}

static int lightly_perturbed(const st_tree *T, int i, int j) {
  const st_node *a = &T->n[i], *b = &T->n[j];
  const double mt = a->m + b->m;
  double cm[3], d[3];
  for (int c = 0; c < 3; c++) cm[c] = (a->m * a->x[c] + b->m * b->x[c]) / mt;
  for (int c = 0; c < 3; c++) d[c] = a->x[c] - b->x[c];
  const double mr3 = 0.25 * mt * mt / pow(dot3(d, d), 3);
  double maxp = 0;
  for (int k = T->n[T->root].od; k >= 0; k = T->n[k].ys) {
    if (k == i || k == j) continue;
    double e[3];
    for (int c = 0; c < 3; c++) e[c] = T->n[k].x[c] - cm[c];
    const double p = pow(T->n[k].m, 2) / pow(dot3(e, e), 3);
    if (p > maxp) maxp = p;
  }
  return maxp < 0.001 * mr3;
}

/* The binary of top-level nodes i and j: a centre-of-mass node in i's place
   (hdyn.cc:108-124), components relative to it (analyze.cc:235-263). */
static void combine(st_tree *T, int i, int j) {
  st_node *a = &T->n[i], *b = &T->n[j];
  const int k = T->nn++;
  st_node *cmn = &T->n[k];
  memset(cmn, 0, sizeof(*cmn));
  cmn->leaf = -1;
  cmn->m = a->m + b->m;
  for (int c = 0; c < 3; c++) {
    cmn->x[c] = (a->m * a->x[c] + b->m * b->x[c]) / cmn->m;
    cmn->v[c] = (a->m * a->v[c] + b->m * b->v[c]) / cmn->m;
  }
  for (int c = 0; c < 3; c++) {
    a->x[c] += -cmn->x[c];
    b->x[c] += -cmn->x[c];
    a->v[c] += -cmn->v[c];
    b->v[c] += -cmn->v[c];
  }
  /* cm takes i's place among the top-level nodes; j leaves the list */
  const int r = T->root;
  cmn->parent = r;
  cmn->os = a->os;
  cmn->ys = a->ys;
  if (a->os >= 0) T->n[a->os].ys = k; else T->n[r].od = k;
  if (a->ys >= 0) T->n[a->ys].os = k;
  if (b->os >= 0) T->n[b->os].ys = b->ys; else T->n[r].od = b->ys;
  if (b->ys >= 0) T->n[b->ys].os = b->os;
  cmn->od = i;
  a->parent = k;
  b->parent = k;
  a->os = -1;
  a->ys = j;
  b->os = i;
  b->ys = -1;
}

static void decompose(st_tree *T) {
  for (;;) {
    double emin = 0;
    int bi = -1, bj = -1;
    for (int i = T->n[T->root].od; i >= 0; i = T->n[i].ys)
      for (int j = T->n[i].ys; j >= 0; j = T->n[j].ys) {
        const double e = rel_energy(T, i, j);
        if (e < emin && lightly_perturbed(T, i, j)) {
          emin = e;
          bi = i;
          bj = j;
        }
      }
    if (bi < 0) break;
    combine(T, bi, bj);
  }
}

/* Depth-first, node before daughters (for_all_nodes). */
static void relative_energies(st_tree *T, int k) {
  st_node *b = &T->n[k];
  if (b->parent >= 0 && b->od >= 0) {
    const int od = b->od, yd = T->n[od].ys;
    const double mu_inv = b->m / (T->n[od].m * T->n[yd].m);
    double d[3];
    for (int c = 0; c < 3; c++) d[c] = T->n[od].v[c] - T->n[yd].v[c];
    b->erel = 0.5 * dot3(d, d) + mu_inv * potential(T, od, yd);
  }
  for (int d = b->od; d >= 0; d = T->n[d].ys) relative_energies(T, d);
}

static int is_escaper(const st_tree *T, int i) {
  const st_node *a = &T->n[i];
  int esc1 = 1, receding = 1;
  const double mi = a->m;
  float mcm = 0; /* single precision, as analyze.cc:385 */
  double rcm[3] = {0, 0, 0}, vcm[3] = {0, 0, 0}, phicm = 0;
  for (int j = T->n[T->root].od; j >= 0; j = T->n[j].ys) {
    if (j == i) continue;
    const st_node *b = &T->n[j];
    const double mj = b->m;
    mcm += mj;
    for (int c = 0; c < 3; c++) {
      rcm[c] += mj * b->x[c];
      vcm[c] += mj * b->v[c];
    }
    const double mu_inv = (mi + mj) / (mi * mj);
    const double dphi = potential(T, i, j);
    phicm += dphi;
    double dv[3], dvji[3], dxji[3];
    for (int c = 0; c < 3; c++) {
      dv[c] = a->v[c] - b->v[c];
      dvji[c] = b->v[c] - a->v[c];
      dxji[c] = b->x[c] - a->x[c];
    }
    const double e = 0.5 * dot3(dv, dv) + mu_inv * dphi;
    esc1 &= e > 0;
    receding &= dot3(dvji, dxji) > 0;
  }
  int esc = esc1 && receding;
  if (esc && mcm > 0) {
    double dr[3], dv[3];
    for (int c = 0; c < 3; c++) {
      rcm[c] = rcm[c] / mcm;
      vcm[c] = vcm[c] / mcm;
    }
    for (int c = 0; c < 3; c++) {
      dr[c] = a->x[c] - rcm[c];
      dv[c] = a->v[c] - vcm[c];
    }
    const double r2 = dot3(dr, dr), v2 = dot3(dv, dv), vr = dot3(dv, dr);
    esc = esc && vr > -1.e-12 * sqrt(v2 * r2) &&
          0.5 * mi * mcm * dot3(dv, dv) / (mi + mcm) + phicm > 0;
  }
  return esc;
}

/* Semi-major axis of node k's binary from its relative energy; -1 unless
   bound (analyze.cc:453-478). */
static double semi(const st_tree *T, int k) {
  const st_node *b = &T->n[k];
  if (b->od < 0) return -1;
  double e = b->erel;
  if (e == 0) {
    const int od = b->od, yd = T->n[od].ys;
    double dv[3], dx[3];
    for (int c = 0; c < 3; c++) {
      dv[c] = T->n[od].v[c] - T->n[yd].v[c];
      dx[c] = T->n[od].x[c] - T->n[yd].x[c];
    }
    e = 0.5 * dot3(dv, dv) - b->m / sqrt(dot3(dx, dx));
  }
  return e < 0 ? -0.5 * b->m / e : -1;
}

/* Two-body elements of a relative orbit: eccentricity, periastron,
   apastron (inf unless bound), period (inf unless bound), unit normal. */
static void elements(double mu, const double r[3], const double v[3], double *e, double *peri,
                     double *apo, double *period, double nrm[3]) {
  const double rn = sqrt(dot3(r, r)), v2 = dot3(v, v);
  const double h[3] = {r[1] * v[2] - r[2] * v[1], r[2] * v[0] - r[0] * v[2],
                       r[0] * v[1] - r[1] * v[0]};
  const double hn = sqrt(dot3(h, h));
  for (int c = 0; c < 3; c++) nrm[c] = hn > 0 ? h[c] / hn : 0;
  const double en = 0.5 * v2 - mu / rn;
  const double p = hn * hn / mu;
  const double ee = sqrt(fmax(0.0, 1 + 2 * en * hn * hn / (mu * mu)));
  *e = ee;
  *peri = p / (1 + ee);
  if (en < 0) {
    const double a = -0.5 * mu / en;
    *apo = a * (1 + ee);
    *period = 6.283185307179586 * sqrt(a * a * a / mu);
  } else {
    *apo = INFINITY;
    *period = INFINITY;
  }
}

/* The hierarchy test of a bound node k with a multiple below it
   (analyze.cc:567-643, with the criterion stated in the file header). */
static int hier_stable(st_tree *T, int k) {
  T->hier_tested = 1;
  const st_node *b = &T->n[k];
  const int od = b->od, yd = T->n[od].ys;
  int bin = od;
  double a_in = semi(T, od);
  if (semi(T, yd) > a_in) {
    bin = yd;
    a_in = semi(T, yd);
  }
  if (a_in < 0) return 0;
  double ro[3], vo[3], ri[3], vi[3];
  for (int c = 0; c < 3; c++) {
    ro[c] = T->n[yd].x[c] - T->n[od].x[c];
    vo[c] = T->n[yd].v[c] - T->n[od].v[c];
  }
  const int iod = T->n[bin].od;
  if (iod < 0) return 0;
  const int iyd = T->n[iod].ys;
  for (int c = 0; c < 3; c++) {
    ri[c] = T->n[iod].x[c] - T->n[iyd].x[c];
    vi[c] = T->n[iod].v[c] - T->n[iyd].v[c];
  }
  double eo, po, ao, to, no[3], ei, pi_, ai, ti, ni_[3];
  elements(b->m, ro, vo, &eo, &po, &ao, &to, no);
  elements(T->n[bin].m, ri, vi, &ei, &pi_, &ai, &ti, ni_);
  const double peri_ratio = po / a_in;
  const double cos_i = dot3(ni_, no);
  if (po < ai) return 0;       /* outer pericentre inside the inner apocentre */
  if (to / ti < 1) return 0;   /* period ratio below 1 */
  const double m12 = T->n[od].m, m3 = T->n[yd].m;
  const double q = m3 / m12;
  const double ratio = (peri_ratio * pow((1 + q) * (1 + eo) / sqrt(1 - eo), -0.4)) /
                       (2.8 * (23.0 / 3 + cos_i) / (23.0 / 3 + 1));
  return ratio > 1;
}

static int check_stability(st_tree *T, int k) {
  st_node *b = &T->n[k];
  int stable = 0;
  b->stable = 0;
  if (b->od < 0) {
    stable = 1;
  } else {
    const int od = b->od, yd = T->n[od].ys;
    if (T->n[od].od < 0 && T->n[yd].od < 0) {
      stable = b->erel < 0;
    } else {
      const int s1 = check_stability(T, od);
      const int s2 = check_stability(T, yd);
      if (s1 && s2 && b->erel < 0) stable = hier_stable(T, k);
    }
  }
  if (stable) b->stable = 1;
  return stable;
}

/* Canonical text of node k's subtree: a leaf's body index, a binary as
   "(first,second)" in daughter order. */
static int describe(const st_tree *T, int k, char *s, int cap) {
  if (T->n[k].od < 0) return snprintf(s, cap > 0 ? cap : 0, "%d", T->n[k].leaf);
  int w = 0;
  w += snprintf(s + w, cap > w ? cap - w : 0, "(");
  w += describe(T, T->n[k].od, s + w, cap > w ? cap - w : 0);
  w += snprintf(s + w, cap > w ? cap - w : 0, ",");
  w += describe(T, T->n[T->n[k].od].ys, s + w, cap > w ? cap - w : 0);
  w += snprintf(s + w, cap > w ? cap - w : 0, ")");
  return w;
}

/* top_rank (optional): per body, the position of its top-level node in the
   tree's order; equal arrays mean the same top-level grouping in the same
   order, which is what smallN's state string records (analyze.cc:771-821). */
static int st_check(int n, const double *mass, const double *pos, const double *vel,
                    int *top_of, int *top_rank, char *summary, int summary_cap) {
  if (n < 1 || n > ST_MAXN || !mass || !pos || !vel) return G6_ERR_ARG;
  st_tree *T = (st_tree *)calloc(1, sizeof(st_tree));
  if (!T) return G6_ERR_NOMEM;
  T->root = 0;
  T->nn = 1;
  st_node *r = &T->n[0];
  r->parent = r->od = r->ys = r->os = r->leaf = -1;
  int prev = -1;
  for (int i = 0; i < n; i++) {
    const int k = T->nn++;
    st_node *b = &T->n[k];
    b->m = mass[i];
    r->m += mass[i];
    for (int c = 0; c < 3; c++) {
      b->x[c] = pos[3 * i + c];
      b->v[c] = vel[3 * i + c];
    }
    b->parent = 0;
    b->od = -1;
    b->ys = -1;
    b->os = prev;
    b->leaf = i;
    if (prev >= 0) T->n[prev].ys = k; else r->od = k;
    prev = k;
  }
  decompose(T);
  relative_energies(T, 0);
  for (int k = r->od; k >= 0; k = T->n[k].ys)
    if (is_escaper(T, k)) T->n[k].escaper = 1;
  for (int k = r->od; k >= 0; k = T->n[k].ys) {
    st_node *b = &T->n[k];
    b->stable = 0;
    if (b->od < 0) {
      if (is_escaper(T, k)) b->stable = 1;
    } else if (check_stability(T, k)) {
      b->stable = 1;
    }
  }
  int over = 1, stable = 1;
  for (int k = r->od; k >= 0; k = T->n[k].ys) {
    if (!is_escaper(T, k)) over = 0;
    if (!T->n[k].stable) stable = 0;
  }
  const int escaping = over;  /* every top-level node escaping */
  if (!stable) over = 0;
  if (top_of || top_rank) {
    int rank = 0;
    for (int k = r->od; k >= 0; k = T->n[k].ys, rank++) {
      int lv[ST_MAXN];
      const int c = leaves(T, k, lv);
      int first = n;
      for (int a = 0; a < c; a++)
        if (T->n[lv[a]].leaf < first) first = T->n[lv[a]].leaf;
      for (int a = 0; a < c; a++) {
        if (top_of) top_of[T->n[lv[a]].leaf] = first;
        if (top_rank) top_rank[T->n[lv[a]].leaf] = rank;
      }
    }
  }
  if (summary && summary_cap > 0) {
    int w = 0;
    summary[0] = 0;
    for (int k = r->od; k >= 0; k = T->n[k].ys) {
      if (w > 0) w += snprintf(summary + w, summary_cap > w ? summary_cap - w : 0, " ");
      w += describe(T, k, summary + w, summary_cap > w ? summary_cap - w : 0);
    }
  }
  const int tested = T->hier_tested;
  free(T);
  /* bit 0: over; bit 1: a multiple above a binary went through the
     hierarchy test (the decision smallN takes from nstab); bit 2: every
     top-level node escaping, stable or not (where smallN's quasi-stable
     ending applies, analyze.cc:958-990) */
  return over | (tested << 1) | (escaping << 2);
}

int g6x_check_structure(int n, const double *mass, const double *pos, const double *vel,
                        int *top_of, char *summary, int summary_cap) {
  return st_check(n, mass, pos, vel, top_of, NULL, summary, summary_cap);
}

/* Many systems at once: a pool of host threads takes systems from a shared
   counter (the checks of a hand-off increment are independent). */
typedef struct {
  int nsys, cap;
  const int *off;
  const double *mass, *pos, *vel;
  int *flags, *top_of, *top_rank;
  char *summary;
  atomic_int next;
} st_batch;

static void *st_worker(void *arg) {
  st_batch *B = (st_batch *)arg;
  for (;;) {
    const int s = atomic_fetch_add(&B->next, 1);
    if (s >= B->nsys) break;
    const int a = B->off[s], n = B->off[s + 1] - a;
    B->flags[s] = st_check(n, B->mass + a, B->pos + 3 * (size_t)a, B->vel + 3 * (size_t)a,
                           B->top_of ? B->top_of + a : NULL,
                           B->top_rank ? B->top_rank + a : NULL,
                           B->summary ? B->summary + (size_t)s * B->cap : NULL,
                           B->summary ? B->cap : 0);
  }
  return NULL;
}

int g6x_check_structure_batch(int nsys, const int *n_per_sys, const double *mass,
                              const double *pos, const double *vel, int *flags, int *top_of,
                              int *top_rank, char *summary, int summary_cap, int nthreads) {
  if (nsys < 0 || (nsys > 0 && (!n_per_sys || !mass || !pos || !vel || !flags)))
    return G6_ERR_ARG;
  if (summary && summary_cap < 1) return G6_ERR_ARG;
  if (nsys == 0) return 0;
  int *off = (int *)malloc(sizeof(int) * ((size_t)nsys + 1));
  if (!off) return G6_ERR_NOMEM;
  off[0] = 0;
  for (int s = 0; s < nsys; s++) {
    if (n_per_sys[s] < 1 || n_per_sys[s] > ST_MAXN) {
      free(off);
      return G6_ERR_ARG;
    }
    off[s + 1] = off[s] + n_per_sys[s];
  }
  st_batch B = {nsys, summary_cap, off, mass, pos, vel, flags, top_of, top_rank, summary, 0};
  atomic_init(&B.next, 0);
  if (nthreads <= 0) {
    const long c = sysconf(_SC_NPROCESSORS_ONLN);
    nthreads = c > 0 ? (int)c : 1;
  }
  if (nthreads > 64) nthreads = 64;
  if (nthreads > (nsys + 7) / 8) nthreads = (nsys + 7) / 8;  /* >= 8 systems a thread */
  pthread_t th[64];
  int started = 0;
  for (int t = 1; t < nthreads; t++) {
    if (pthread_create(&th[started], NULL, st_worker, &B) != 0) break;
    started++;
  }
  st_worker(&B);
  for (int t = 0; t < started; t++) pthread_join(th[t], NULL);
  free(off);
  for (int s = 0; s < nsys; s++)
    if (flags[s] < 0) return flags[s];
  return 0;
}
