/* milc_oracle.c -- CPU restatement of MILC's staggered operator, solvers
 * and link smearing.  TEST INFRASTRUCTURE ONLY (see milc_oracle.h).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "milc_oracle.h"

/* ---------------- geometry: generic/layout_hyper_prime.c:509-520 ---------------- */
size_t orc_index(const orc_lat *L, const int c[4]) {
  size_t i = (size_t)c[0] + (size_t)L->dims[0] * ((size_t)c[1] + (size_t)L->dims[1] *
             ((size_t)c[2] + (size_t)L->dims[2] * (size_t)c[3]));
  if (((c[0] + c[1] + c[2] + c[3]) & 1) == 0) return i / 2;
  return (i + L->V) / 2;
}

orc_lat *orc_lat_create(int nx, int ny, int nz, int nt) {
  orc_lat *L = (orc_lat *)calloc(1, sizeof(orc_lat));
  L->dims[0] = nx; L->dims[1] = ny; L->dims[2] = nz; L->dims[3] = nt;
  L->V = (size_t)nx * ny * nz * nt;
  L->Vh = L->V / 2;
  L->coord = (int *)malloc(L->V * 4 * sizeof(int));
  L->nb = (size_t *)malloc(L->V * 16 * sizeof(size_t));
  int c[4];
  for (c[3] = 0; c[3] < nt; c[3]++)
    for (c[2] = 0; c[2] < nz; c[2]++)
      for (c[1] = 0; c[1] < ny; c[1]++)
        for (c[0] = 0; c[0] < nx; c[0]++) {
          size_t i = orc_index(L, c);
          memcpy(L->coord + 4 * i, c, 4 * sizeof(int));
        }
  for (size_t i = 0; i < L->V; i++) {
    for (int d = 0; d < 8; d++) {
      int mu = d < 4 ? d : 7 - d, s = d < 4 ? 1 : -1;  /* OPP_DIR(d) = 7-d (include/dirs.h) */
      for (int hop = 1; hop <= 3; hop += 2) {
        int n[4];
        memcpy(n, L->coord + 4 * i, sizeof n);
        n[mu] = (n[mu] + s * hop + 4 * L->dims[mu]) % L->dims[mu];
        L->nb[16 * i + d + (hop == 3 ? 8 : 0)] = orc_index(L, n);
      }
    }
  }
  return L;
}

void orc_lat_free(orc_lat *L) {
  if (!L) return;
  free(L->coord); free(L->nb); free(L);
}

/* generic_ks/rephase.c:53-117: fold eta_mu(x) and the t = nt-1 sign into links */
void orc_rephase(const orc_lat *L, double *links) {
  for (size_t i = 0; i < L->V; i++) {
    const int *c = L->coord + 4 * i;
    double ph[4];
    ph[3] = 1.0;
    ph[0] = (c[3] % 2 == 1) ? -1.0 : 1.0;
    ph[1] = (c[0] % 2 == 1) ? -ph[0] : ph[0];
    ph[2] = (c[1] % 2 == 1) ? -ph[1] : ph[1];
    if (c[3] == L->dims[3] - 1) ph[3] = -ph[3];
    for (int d = 0; d < 4; d++)
      for (int k = 0; k < 18; k++) links[(4 * i + d) * 18 + k] *= ph[d];
  }
}

/* ---------------- SU(3) primitives (semantics of MILC's libraries/ directory) ---------------- */
#define RE(m, i, j) (m)[2 * (3 * (i) + (j))]
#define IM(m, i, j) (m)[2 * (3 * (i) + (j)) + 1]

static inline void mat_vec(const double *m, const double *v, double *o) { /* m_matvec.c */
  for (int i = 0; i < 3; i++) {
    double re = 0, im = 0;
    for (int j = 0; j < 3; j++) {
      re += RE(m, i, j) * v[2 * j] - IM(m, i, j) * v[2 * j + 1];
      im += RE(m, i, j) * v[2 * j + 1] + IM(m, i, j) * v[2 * j];
    }
    o[2 * i] = re; o[2 * i + 1] = im;
  }
}
static inline void adj_mat_vec(const double *m, const double *v, double *o) { /* m_amatvec.c */
  for (int i = 0; i < 3; i++) {
    double re = 0, im = 0;
    for (int j = 0; j < 3; j++) {
      re += RE(m, j, i) * v[2 * j] + IM(m, j, i) * v[2 * j + 1];
      im += RE(m, j, i) * v[2 * j + 1] - IM(m, j, i) * v[2 * j];
    }
    o[2 * i] = re; o[2 * i + 1] = im;
  }
}
static inline void mat_nn(const double *a, const double *b, double *c) { /* m_mat_nn.c */
  double r[18];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += RE(a, i, k) * RE(b, k, j) - IM(a, i, k) * IM(b, k, j);
        im += RE(a, i, k) * IM(b, k, j) + IM(a, i, k) * RE(b, k, j);
      }
      r[2 * (3 * i + j)] = re; r[2 * (3 * i + j) + 1] = im;
    }
  memcpy(c, r, sizeof r);
}
static inline void mat_na(const double *a, const double *b, double *c) { /* m_mat_na.c: a b^dag */
  double r[18];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += RE(a, i, k) * RE(b, j, k) + IM(a, i, k) * IM(b, j, k);
        im += IM(a, i, k) * RE(b, j, k) - RE(a, i, k) * IM(b, j, k);
      }
      r[2 * (3 * i + j)] = re; r[2 * (3 * i + j) + 1] = im;
    }
  memcpy(c, r, sizeof r);
}
static inline void mat_an(const double *a, const double *b, double *c) { /* m_mat_an.c: a^dag b */
  double r[18];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += RE(a, k, i) * RE(b, k, j) + IM(a, k, i) * IM(b, k, j);
        im += RE(a, k, i) * IM(b, k, j) - IM(a, k, i) * RE(b, k, j);
      }
      r[2 * (3 * i + j)] = re; r[2 * (3 * i + j) + 1] = im;
    }
  memcpy(c, r, sizeof r);
}

/* ---------------- D: generic_ks/dslash_fn.c:365-576 ---------------- */
void orc_dslash(const orc_lat *L, const double *fat, const double *lng,
                const double *src, double *dst, int parity) {
  size_t lo = 0, hi = L->V;
  if (parity == ORC_EVEN) hi = L->Vh;
  else if (parity == ORC_ODD) lo = L->Vh;
  double *out = (double *)malloc((hi - lo) * 6 * sizeof(double));
  long long n = (long long)(hi - lo);
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < n; k++) {
    size_t i = lo + (size_t)k;
    const size_t *nb = L->nb + 16 * i;
    double acc[6] = {0}, lacc[6] = {0}, t[6];
    /* forward one-link and three-link terms (mult_su3_mat_vec_sum_4dir) */
    for (int mu = 0; mu < 4; mu++) {
      mat_vec(fat + (4 * i + mu) * 18, src + 6 * nb[mu], t);
      for (int q = 0; q < 6; q++) acc[q] += t[q];
      mat_vec(lng + (4 * i + mu) * 18, src + 6 * nb[8 + mu], t);
      for (int q = 0; q < 6; q++) lacc[q] += t[q];
    }
    /* backward terms: F_mu(x-mu)^dag s(x-mu), L_mu(x-3mu)^dag s(x-3mu) */
    for (int mu = 0; mu < 4; mu++) {
      size_t b1 = nb[7 - mu], b3 = nb[8 + 7 - mu];
      adj_mat_vec(fat + (4 * b1 + mu) * 18, src + 6 * b1, t);
      for (int q = 0; q < 6; q++) acc[q] -= t[q];
      adj_mat_vec(lng + (4 * b3 + mu) * 18, src + 6 * b3, t);
      for (int q = 0; q < 6; q++) lacc[q] -= t[q];
    }
    for (int q = 0; q < 6; q++) out[6 * k + q] = acc[q] + lacc[q];
  }
  memcpy(dst + 6 * lo, out, (hi - lo) * 6 * sizeof(double));
  free(out);
}

/* ---------------- vector helpers ---------------- */
static void par_range(const orc_lat *L, int parity, size_t *lo, size_t *hi) {
  *lo = 0; *hi = L->V;
  if (parity == ORC_EVEN) *hi = L->Vh;
  else if (parity == ORC_ODD) *lo = L->Vh;
}

static double rel_residue(const orc_lat *L, const double *p, const double *q, int parity) {
  /* my_relative_residue, generic_ks/d_congrad5_fn_milc.c:38-56 */
  size_t lo, hi;
  par_range(L, parity, &lo, &hi);
  double residue = 0;
  for (size_t i = lo; i < hi; i++) {
    double num = 0, den = 0;
    for (int k = 0; k < 6; k++) { num += p[6 * i + k] * p[6 * i + k]; den += q[6 * i + k] * q[6 * i + k]; }
    residue += (den == 0) ? 1.0 : (num / den);
  }
  if (parity == ORC_EVENANDODD) return sqrt(residue / L->V);
  return sqrt(2 * residue / L->V);
}

/* D on nsrc fields at once (links read once per site for all of them); per
   field the arithmetic is orc_dslash's, statement for statement, so each
   output equals orc_dslash's bit for bit.  In place allowed (src == dst). */
static void orc_dslash_multi(const orc_lat *L, const double *fat, const double *lng, int nsrc,
                             double *const *src, double *const *dst, int parity) {
  size_t lo = 0, hi = L->V;
  if (parity == ORC_EVEN) hi = L->Vh;
  else if (parity == ORC_ODD) lo = L->Vh;
  const size_t n = hi - lo;
  double *out = (double *)malloc((size_t)nsrc * n * 6 * sizeof(double));
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < (long long)n; k++) {
    size_t i = lo + (size_t)k;
    const size_t *nb = L->nb + 16 * i;
    for (int s = 0; s < nsrc; s++) {
      const double *sv = src[s];
      double acc[6] = {0}, lacc[6] = {0}, t[6];
      for (int mu = 0; mu < 4; mu++) {
        mat_vec(fat + (4 * i + mu) * 18, sv + 6 * nb[mu], t);
        for (int q = 0; q < 6; q++) acc[q] += t[q];
        mat_vec(lng + (4 * i + mu) * 18, sv + 6 * nb[8 + mu], t);
        for (int q = 0; q < 6; q++) lacc[q] += t[q];
      }
      for (int mu = 0; mu < 4; mu++) {
        size_t b1 = nb[7 - mu], b3 = nb[8 + 7 - mu];
        adj_mat_vec(fat + (4 * b1 + mu) * 18, sv + 6 * b1, t);
        for (int q = 0; q < 6; q++) acc[q] -= t[q];
        adj_mat_vec(lng + (4 * b3 + mu) * 18, sv + 6 * b3, t);
        for (int q = 0; q < 6; q++) lacc[q] -= t[q];
      }
      for (int q = 0; q < 6; q++) out[((size_t)s * n + (size_t)k) * 6 + q] = acc[q] + lacc[q];
    }
  }
  for (int s = 0; s < nsrc; s++) memcpy(dst[s] + 6 * lo, out + (size_t)s * n * 6, n * 6 * sizeof(double));
  free(out);
}

/* ---------------- CG: generic_ks/d_congrad5_fn_milc.c:61-407 (FEWSUMS) ----------------
 * nsrc independent solves run in lockstep: each round applies M^dag M once
 * to every running source (to dest at a restart, to cg_p in an iteration)
 * with one multi-field D, then runs that source's part of MILC's loop.
 * Every source follows MILC's recurrences, restarts and stopping rule on
 * its own, in MILC's order of operations, so its result and iteration count
 * are those of a solve by itself; orc_congrad is the one-source case.  Sums
 * over sites are sequential, as in MILC's single-thread loop. */
typedef struct {
  const double *src;
  double *dest, *ttt, *cg_p, *res;
  double source_norm, size_r, size_relr, final_rsq, final_relrsq;
  double rsq, relrsq, actual_rsq, oldrsq;
  int iteration, nrestart, converged, mode, running;  /* mode 0: check, 1: restart, 2: iterate */
} orc_cg_state;

int orc_congrad_multi(const orc_lat *L, const double *fat, const double *lng, int nsrc,
                      const double *const *srcs, double *const *dests, double mass, int parity,
                      double resid, double relresid, int niter, int max_restarts, double *out7) {
  size_t lo, hi;
  par_range(L, parity, &lo, &hi);
  int otherparity = parity == ORC_EVEN ? ORC_ODD : ORC_EVEN;
  double rsqmin = resid * resid, relrsqmin = relresid * relresid;
  int max_cg = max_restarts * niter;
  double msq_x4 = 4.0 * mass * mass;
  size_t n6 = 6 * L->V;
  orc_cg_state *S = (orc_cg_state *)calloc((size_t)nsrc, sizeof(orc_cg_state));
  double **vin = (double **)malloc((size_t)nsrc * sizeof(double *));
  double **vout = (double **)malloc((size_t)nsrc * sizeof(double *));
  int nrun = 0;
  for (int s = 0; s < nsrc; s++) {
    orc_cg_state *q = &S[s];
    q->src = srcs[s];
    q->dest = dests[s];
    for (size_t i = 6 * lo; i < 6 * hi; i++) q->source_norm += q->src[i] * q->src[i];
    q->converged = 1;
    q->size_relr = 1.0;
    q->relrsq = 1.0;
    q->actual_rsq = 999.;
    if (q->source_norm == 0.0) {
      memset(q->dest + 6 * lo, 0, (hi - lo) * 6 * sizeof(double));
      continue;
    }
    q->ttt = (double *)calloc(n6, sizeof(double));
    q->cg_p = (double *)calloc(n6, sizeof(double));
    q->res = (double *)calloc(n6, sizeof(double));
    q->running = 1;
    nrun++;
  }
  while (nrun > 0) {
    int nd = 0;
    for (int s = 0; s < nsrc; s++) {
      orc_cg_state *q = &S[s];
      if (!q->running) continue;
      if (q->mode == 0)
        q->mode = ((q->iteration % niter == 0) ||
                   ((rsqmin <= 0 || rsqmin > q->size_r) && (relrsqmin <= 0 || relrsqmin > q->size_relr))) ? 1 : 2;
      vin[nd] = q->mode == 1 ? q->dest : q->cg_p;
      vout[nd] = q->ttt;
      nd++;
    }
    orc_dslash_multi(L, fat, lng, nd, vin, vout, otherparity);
    orc_dslash_multi(L, fat, lng, nd, vout, vout, parity);
#pragma omp parallel for schedule(dynamic, 1) reduction(- : nrun)
    for (int s = 0; s < nsrc; s++) {
      orc_cg_state *q = &S[s];
      if (!q->running) continue;
      double *ttt = q->ttt, *cg_p = q->cg_p, *res = q->res, *dest = q->dest;
      const double *src = q->src;
      if (q->mode == 1) {
        double rsq = 0;
        for (size_t i = 6 * lo; i < 6 * hi; i++) {
          ttt[i] = ttt[i] + (-msq_x4) * dest[i];
          res[i] = src[i] + ttt[i];
          cg_p[i] = res[i];
          rsq += res[i] * res[i];
        }
        q->rsq = rsq;
        q->actual_rsq = rsq;
        if (relrsqmin > 0) q->relrsq = rel_residue(L, res, dest, parity);
        q->final_rsq = rsq / q->source_norm;
        q->final_relrsq = q->relrsq;
        q->iteration++;
        if (q->iteration >= max_cg || q->nrestart >= max_restarts ||
            ((rsqmin <= 0 || rsqmin > q->final_rsq) && (relrsqmin <= 0 || relrsqmin > q->final_relrsq))) {
          q->running = 0;
          nrun--;
          continue;
        }
        q->nrestart++;
        q->mode = 2;  /* MILC's loop goes on to the iteration without a new check */
        continue;
      }
      q->oldrsq = q->actual_rsq;
      double pkp = 0, c_tr = 0, c_tt = 0;
      for (size_t st = lo; st < hi; st++) {
        double a = 0, b = 0, c = 0;
        for (int k = 0; k < 6; k++) {
          size_t i = 6 * st + k;
          ttt[i] = ttt[i] + (-msq_x4) * cg_p[i];
          a += cg_p[i] * ttt[i];
          b += ttt[i] * res[i];
          c += ttt[i] * ttt[i];
        }
        pkp += a; c_tr += b; c_tt += c;
      }
      q->iteration++;
      double a = -q->rsq / pkp;
      double actual_rsq = 0;
      for (size_t i = 6 * lo; i < 6 * hi; i++) {
        dest[i] = dest[i] + a * cg_p[i];
        res[i] = res[i] + a * ttt[i];
        actual_rsq += res[i] * res[i];
      }
      q->actual_rsq = actual_rsq;
      q->rsq = q->oldrsq + 2.0 * a * c_tr + a * a * c_tt;
      if (relrsqmin > 0) q->relrsq = rel_residue(L, res, dest, parity);
      q->size_r = q->rsq / q->source_norm;
      q->size_relr = q->relrsq;
      double b = q->rsq / q->oldrsq;
      for (size_t i = 6 * lo; i < 6 * hi; i++) cg_p[i] = res[i] + b * cg_p[i];
      q->mode = 0;
    }
  }
  for (int s = 0; s < nsrc; s++) {
    orc_cg_state *q = &S[s];
    if (q->source_norm != 0.0 && (q->nrestart == max_restarts || q->iteration == max_cg)) q->converged = 0;
    if (out7) {
      double *o = out7 + 7 * (size_t)s;
      if (q->source_norm == 0.0) {
        for (int k = 0; k < 7; k++) o[k] = 0;
        o[6] = 1;
      } else {
        o[0] = q->final_rsq; o[1] = q->final_relrsq; o[2] = q->size_r; o[3] = q->size_relr;
        o[4] = q->iteration; o[5] = q->nrestart; o[6] = q->converged;
      }
    }
    free(q->ttt); free(q->cg_p); free(q->res);
  }
  int maxit = 0;
  for (int s = 0; s < nsrc; s++) maxit = S[s].iteration > maxit ? S[s].iteration : maxit;
  free(S); free(vin); free(vout);
  return maxit;
}

int orc_congrad(const orc_lat *L, const double *fat, const double *lng,
                const double *src, double *dest, double mass, int parity,
                double resid, double relresid, int niter, int max_restarts, double out[7]) {
  return orc_congrad_multi(L, fat, lng, 1, &src, &dest, mass, parity, resid, relresid, niter, max_restarts, out);
}

/* ---------------- M^-1: generic_ks/mat_invert.c:18-44,328-407 ---------------- */
int orc_mat_invert_uml(const orc_lat *L, const double *fat, const double *lng,
                       const double *src, double *dst, double mass, double resid,
                       int max, int nrestart, double out[7]) {
  size_t n6 = 6 * L->V;
  double *tmp = (double *)malloc(n6 * sizeof(double));
  double *ttt = (double *)malloc(n6 * sizeof(double));
  /* tmp = M^dag src = 2m src - D src */
  orc_dslash(L, fat, lng, src, tmp, ORC_EVENANDODD);
  for (size_t i = 0; i < n6; i++) tmp[i] = -tmp[i] + 2.0 * mass * src[i];
  double o1[7], o2[7];
  int cgn = orc_congrad(L, fat, lng, tmp, dst, mass, ORC_EVEN, resid, 0, max, nrestart, o1);
  orc_dslash(L, fat, lng, dst, ttt, ORC_ODD);
  for (size_t i = 6 * L->Vh; i < n6; i++) dst[i] = (src[i] - ttt[i]) * (1.0 / (2.0 * mass));
  cgn += orc_congrad(L, fat, lng, tmp, dst, mass, ORC_ODD, resid, 0, max, nrestart, o2);
  if (out) { memcpy(out, o2, sizeof o2); out[4] += o1[4]; }
  free(tmp); free(ttt);
  return cgn;
}

/* ---------------- multi-shift CG: generic_ks/ks_multicg_offset.c:63-505 ---------------- */
int orc_multicg_offset(const orc_lat *L, const double *fat, const double *lng,
                       const double *src, double *psim, const double *offsets,
                       int num_offsets, int parity, double resid, int max, int nrestart,
                       double *final_rsq) {
  int niter = max * nrestart;
  double rsqmin = resid * resid;
  size_t lo, hi;
  par_range(L, parity, &lo, &hi);
  int otherparity = parity == ORC_EVEN ? ORC_ODD : ORC_EVEN;
  size_t n6 = 6 * L->V;
  if (num_offsets <= 0) return 0;
  double *shifts = (double *)malloc(num_offsets * sizeof(double));
  double *zeta_i = (double *)malloc(num_offsets * sizeof(double));
  double *zeta_im1 = (double *)malloc(num_offsets * sizeof(double));
  double *zeta_ip1 = (double *)malloc(num_offsets * sizeof(double));
  double *beta_i = (double *)malloc(num_offsets * sizeof(double));
  double *beta_im1 = (double *)malloc(num_offsets * sizeof(double));
  double *alpha = (double *)malloc(num_offsets * sizeof(double));
  double *pm = (double *)calloc((size_t)num_offsets * n6, sizeof(double));
  double *ttt = (double *)calloc(n6, sizeof(double));
  double *cg_p = (double *)calloc(n6, sizeof(double));
  double *res = (double *)calloc(n6, sizeof(double));
  double offset_low = 1.0e20;
  int j_low = -1, iteration = 0, num_now = num_offsets;
  for (int j = 0; j < num_offsets; j++) {
    shifts[j] = offsets[j];
    if (offsets[j] < offset_low) { offset_low = offsets[j]; j_low = j; }
  }
  if (j_low < 0) j_low = 0;  /* offsets >= 1e20: keep the first as the base */
  for (int j = 0; j < num_offsets; j++) if (j != j_low) shifts[j] -= shifts[j_low];
  double shift0 = -shifts[j_low];
  double source_norm = 0;
  for (size_t i = 6 * lo; i < 6 * hi; i++) {
    source_norm += src[i] * src[i];
    res[i] = src[i]; cg_p[i] = src[i];
    for (int j = 0; j < num_offsets; j++) { psim[(size_t)j * n6 + i] = 0; pm[(size_t)j * n6 + i] = src[i]; }
  }
  double rsq = source_norm, oldrsq, pkp, c1, c2;
  int done = 0;
  if (source_norm == 0.) {
    for (int j = 0; j < num_offsets; j++) if (final_rsq) final_rsq[j] = 0;
    done = 1;
  }
  if (!done) {
    iteration++;
    double rsqstop = rsqmin * source_norm;
    for (int j = 0; j < num_offsets; j++) { zeta_im1[j] = zeta_i[j] = 1.0; beta_im1[j] = -1.0; alpha[j] = 0.0; }
    do {
      oldrsq = rsq;
      orc_dslash(L, fat, lng, cg_p, ttt, otherparity);
      orc_dslash(L, fat, lng, ttt, ttt, parity);
      pkp = 0;
      for (size_t s = lo; s < hi; s++) {
        double a = 0;
        for (int k = 0; k < 6; k++) {
          size_t i = 6 * s + k;
          ttt[i] = ttt[i] + shift0 * cg_p[i];
          a += cg_p[i] * ttt[i];
        }
        pkp += a;
      }
      iteration++;
      beta_i[j_low] = -rsq / pkp;
      zeta_ip1[j_low] = 1.0;
      for (int j = 0; j < num_now; j++) if (j != j_low) {
        zeta_ip1[j] = zeta_i[j] * zeta_im1[j] * beta_im1[j_low];
        c1 = beta_i[j_low] * alpha[j_low] * (zeta_im1[j] - zeta_i[j]);
        c2 = zeta_im1[j] * beta_im1[j_low] * (1.0 + shifts[j] * beta_i[j_low]);
        if (c1 + c2 != 0.0) zeta_ip1[j] /= c1 + c2;
        else zeta_ip1[j] = 0.0;
        if (zeta_i[j] != 0.0) beta_i[j] = beta_i[j_low] * zeta_ip1[j] / zeta_i[j];
        else {
          zeta_ip1[j] = 0.0; beta_i[j] = 0.0;
          if (j == num_now - 1 && j > j_low) num_now--;
        }
      }
      rsq = 0;
      for (size_t s = lo; s < hi; s++) {
        double a = 0;
        for (int k = 0; k < 6; k++) {
          size_t i = 6 * s + k;
          for (int j = 0; j < num_now; j++)
            psim[(size_t)j * n6 + i] = psim[(size_t)j * n6 + i] + beta_i[j] * pm[(size_t)j * n6 + i];
          res[i] = res[i] + beta_i[j_low] * ttt[i];
          a += res[i] * res[i];
        }
        rsq += a;
      }
      if (rsqstop > 0 && rsq <= rsqstop) {
        for (int j = 0; j < num_offsets; j++) if (final_rsq) final_rsq[j] = rsq / source_norm;
        done = 1;
        break;
      }
      alpha[j_low] = rsq / oldrsq;
      for (int j = 0; j < num_now; j++) if (j != j_low) {
        if (zeta_i[j] * beta_i[j_low] != 0.0)
          alpha[j] = alpha[j_low] * zeta_ip1[j] * beta_i[j] / (zeta_i[j] * beta_i[j_low]);
        else alpha[j] = 0.0;
      }
      for (size_t i = 6 * lo; i < 6 * hi; i++) {
        for (int j = 0; j < num_now; j++) {
          double t = res[i] * zeta_ip1[j];
          pm[(size_t)j * n6 + i] = t + alpha[j] * pm[(size_t)j * n6 + i];
        }
        cg_p[i] = pm[(size_t)j_low * n6 + i];
      }
      for (int j = 0; j < num_now; j++) {
        beta_im1[j] = beta_i[j]; zeta_im1[j] = zeta_i[j]; zeta_i[j] = zeta_ip1[j];
      }
    } while (iteration < niter);
    if (!done) for (int j = 0; j < num_offsets; j++) if (final_rsq) final_rsq[j] = rsq / source_norm;
  }
  free(shifts); free(zeta_i); free(zeta_im1); free(zeta_ip1); free(beta_i); free(beta_im1);
  free(alpha); free(pm); free(ttt); free(cg_p); free(res);
  return iteration;
}

/* ---------------- link smearing ---------------- */
/* compute_gen_staple_field, generic/general_staple.c:42-140:
   S(x) = U_nu(x) A(x+nu) U_nu(x+mu)^dag + U_nu(x-nu)^dag A(x-nu) U_nu(x-nu+mu);
   fat_mu += coef*S; S saved when `staple` is non-NULL. */
static void gen_staple(const orc_lat *L, double *staple, int mu, int nu, const double *A,
                       int stride, double *fat, double coef, const double *U) {
  long long n = (long long)L->V;
  double *S = (double *)malloc(L->V * 18 * sizeof(double));
#pragma omp parallel for schedule(static)
  for (long long k = 0; k < n; k++) {
    size_t x = (size_t)k;
    const size_t *nb = L->nb + 16 * x;
    size_t xpnu = nb[nu], xpmu = nb[mu], xmnu = nb[7 - nu];
    size_t xmnupmu = L->nb[16 * xmnu + mu];
    double t1[18], t2[18], up[18], dn[18];
    /* upper: U_nu(x) [A(x+nu) U_nu(x+mu)^dag] */
    mat_na(A + stride * 18 * xpnu, U + (4 * xpmu + nu) * 18, t1);
    mat_nn(U + (4 * x + nu) * 18, t1, up);
    /* lower: [U_nu(x-nu)^dag A(x-nu)] U_nu(x-nu+mu) */
    mat_an(U + (4 * xmnu + nu) * 18, A + stride * 18 * xmnu, t2);
    mat_nn(t2, U + (4 * xmnupmu + nu) * 18, dn);
    for (int q = 0; q < 18; q++) S[18 * x + q] = up[q] + dn[q];
  }
#pragma omp parallel for schedule(static)
  for (size_t x = 0; x < L->V; x++)
    for (int q = 0; q < 18; q++) {
      fat[(4 * x + mu) * 18 + q] += coef * S[18 * x + q];
      if (staple) staple[18 * x + q] = S[18 * x + q];
    }
  free(S);
}

/* load_fatlinks_cpu with ASQ_OPTIMIZED_FATTENING,
   generic_ks/fermion_links_fn_load_milc.c:135-271 */
void orc_load_fatlinks(const orc_lat *L, const double *links, const orc_coeffs *c, double *fat) {
  double one_link = c->one_link - 6.0 * c->lepage;
  double *staple = (double *)malloc(L->V * 18 * sizeof(double));
  double *tmp1 = (double *)malloc(L->V * 18 * sizeof(double));
  for (int dir = 0; dir < 4; dir++) {
#pragma omp parallel for schedule(static)
    for (size_t x = 0; x < L->V; x++)
      for (int q = 0; q < 18; q++) fat[(4 * x + dir) * 18 + q] = one_link * links[(4 * x + dir) * 18 + q];
    if (c->three_staple == 0.0 && c->lepage == 0.0 && c->five_staple == 0.0) continue;
    for (int nu = 0; nu < 4; nu++) if (nu != dir) {
      gen_staple(L, staple, dir, nu, links + 18 * dir, 4, fat, c->three_staple, links);
      gen_staple(L, NULL, dir, nu, staple, 1, fat, c->lepage, links);
      for (int rho = 0; rho < 4; rho++) if (rho != dir && rho != nu) {
        gen_staple(L, tmp1, dir, rho, staple, 1, fat, c->five_staple, links);
        for (int sig = 0; sig < 4; sig++)
          if (sig != dir && sig != nu && sig != rho)
            gen_staple(L, NULL, dir, sig, tmp1, 1, fat, c->seven_staple, links);
      }
    }
  }
  free(staple); free(tmp1);
}

/* load_lnglinks, generic_ks/fermion_links_fn_load_milc.c:52-128: the only
   path with displacement 3 mu is the Naik path, giving
   L_mu(x) = naik * U_mu(x) U_mu(x+mu) U_mu(x+2mu). */
void orc_load_lnglinks(const orc_lat *L, const double *links, const orc_coeffs *c, double *lng) {
  for (size_t x = 0; x < L->V; x++)
    for (int mu = 0; mu < 4; mu++) {
      size_t x1 = L->nb[16 * x + mu], x2 = L->nb[16 * x1 + mu];
      double t[18], p[18];
      mat_nn(links + (4 * x1 + mu) * 18, links + (4 * x2 + mu) * 18, t);
      mat_nn(links + (4 * x + mu) * 18, t, p);
      for (int q = 0; q < 18; q++) lng[(4 * x + mu) * 18 + q] = c->naik * p[q];
    }
}

/* u3_unitarize_analytic, generic_ks/su3_mat_op.c:828-1200: W = V (V^dag V)^-1/2
   with the eigenvalues of Q = V^dag V from the trigonometric solution of its
   characteristic cubic (Hasenfratz, Hoffmann, Schaefer, JHEP05 (2007) 029).
   Returns 1 where MILC would fall back to an SVD (HISQ_REUNIT_SVD_* = 1e-8),
   0 otherwise.  The analytic result is written in either case. */
int orc_u3_unitarize(const double *V, double *W) {
  double Q[18], Q2[18], S2[18];
  mat_an(V, V, Q);
  mat_nn(Q, Q, Q2);
  double c0 = RE(Q, 0, 0) + RE(Q, 1, 1) + RE(Q, 2, 2);
  double c1 = (RE(Q2, 0, 0) + RE(Q2, 1, 1) + RE(Q2, 2, 2)) / 2;
  double q3d = 0;
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++)
      q3d += RE(Q2, i, k) * RE(Q, k, i) - IM(Q2, i, k) * IM(Q, k, i);
  double c2 = q3d / 3;
  double g0, g1, g2;
  double S = c1 / 3 - c0 * (c0 / 18);
  if (fabs(S) < 1.0e-14) {
    g0 = g1 = g2 = c0 / 3;
  } else {
    double R = c2 / 2 - c0 * (c1 / 3) + c0 * c0 * (c0 / 27);
    S = sqrt(S);
    double RoS = R / (S * S * S), theta;
    if (!(fabs(RoS) < 1.0)) theta = R > 0 ? 0.0 : 3.14159265358979323846264338328;
    else theta = acos(RoS);
    double th3 = theta / 3, pi23 = 6.28318530717958647692528676656 / 3;
    g0 = c0 / 3 + 2 * S * cos(th3);
    g1 = c0 / 3 + 2 * S * cos(th3 + pi23);
    g2 = c0 / 3 + 2 * S * cos(th3 + 2 * pi23);
  }
  /* determinant of V, for MILC's SVD trigger */
  double detre = 0, detim = 0;
  {
    double a1re = RE(V,1,1)*RE(V,2,2) - IM(V,1,1)*IM(V,2,2) - RE(V,1,2)*RE(V,2,1) + IM(V,1,2)*IM(V,2,1);
    double a1im = RE(V,1,1)*IM(V,2,2) + IM(V,1,1)*RE(V,2,2) - RE(V,1,2)*IM(V,2,1) - IM(V,1,2)*RE(V,2,1);
    double a2re = RE(V,1,0)*RE(V,2,2) - IM(V,1,0)*IM(V,2,2) - RE(V,1,2)*RE(V,2,0) + IM(V,1,2)*IM(V,2,0);
    double a2im = RE(V,1,0)*IM(V,2,2) + IM(V,1,0)*RE(V,2,2) - RE(V,1,2)*IM(V,2,0) - IM(V,1,2)*RE(V,2,0);
    double a3re = RE(V,1,0)*RE(V,2,1) - IM(V,1,0)*IM(V,2,1) - RE(V,1,1)*RE(V,2,0) + IM(V,1,1)*IM(V,2,0);
    double a3im = RE(V,1,0)*IM(V,2,1) + IM(V,1,0)*RE(V,2,1) - RE(V,1,1)*IM(V,2,0) - IM(V,1,1)*RE(V,2,0);
    detre = RE(V,0,0)*a1re - IM(V,0,0)*a1im - RE(V,0,1)*a2re + IM(V,0,1)*a2im + RE(V,0,2)*a3re - IM(V,0,2)*a3im;
    detim = IM(V,0,0)*a1re + RE(V,0,0)*a1im - IM(V,0,1)*a2re - RE(V,0,1)*a2im + IM(V,0,2)*a3re + RE(V,0,2)*a3im;
  }
  double det_check = detre * detre + detim * detim;
  int svd = 0;
  if (det_check != 0 && fabs(det_check - g0 * g1 * g2) / fabs(det_check) > 1e-8) svd = 1;
  if (det_check < 1e-8) svd = 1;
  double g0sq = sqrt(g0), g1sq = sqrt(g1), g2sq = sqrt(g2);
  double us = g1sq + g2sq, ws = g1sq * g2sq;
  double vs = g0sq * us + ws;
  us += g0sq;
  ws *= g0sq;
  double denom = ws * (us * vs - ws);
  double f0 = (us * vs * vs - ws * (us * us + vs)) / denom;
  double f1 = (2 * us * vs - ws - us * us * us) / denom;
  double f2 = us / denom;
  for (int k = 0; k < 18; k++) S2[k] = f1 * Q[k] + f2 * Q2[k];
  RE(S2, 0, 0) += f0; RE(S2, 1, 1) += f0; RE(S2, 2, 2) += f0;
  mat_nn(V, S2, W);
  return svd;
}

/* asqtad: generic_ks/imp_actions/asqtad_action.h:22-47 with the tadpole
   division of ks_action_paths.c (coefficient / u0^(length-1)) */
void orc_asqtad_coeffs(double u0, orc_coeffs *c) {
  c->one_link = (1.0 / 8.0) + (6.0 / 16.0) + (1.0 / 8.0);
  c->naik = (-1.0 / 24.0) / (u0 * u0);
  c->three_staple = (-1.0 / 8.0) * 0.5 / (u0 * u0);
  c->five_staple = (1.0 / 8.0) * 0.25 * 0.5 / (u0 * u0 * u0 * u0);
  c->seven_staple = (-1.0 / 8.0) * 0.125 * (1.0 / 6.0) / (u0 * u0 * u0 * u0 * u0 * u0);
  c->lepage = (-1.0 / 16) / (u0 * u0 * u0 * u0);
}

void orc_asqtad_links(const orc_lat *L, const double *U, double u0, double *fat, double *lng) {
  orc_coeffs c;
  orc_asqtad_coeffs(u0, &c);
  orc_load_fatlinks(L, U, &c, fat);
  orc_load_lnglinks(L, U, &c, lng);
}

/* HISQ: generic_ks/fermion_links_hisq_load_milc.c:547-640 with the
   coefficient tables of generic_ks/imp_actions/hisq/hisq_u3_action.h
   (no tadpole factors).  fat/lng hold n_naiks consecutive link fields.
   Returns the number of links where MILC would have used its SVD. */
int orc_hisq_links(const orc_lat *L, const double *U, int n_naiks, const double *eps_naik,
                   double *Vl, double *W, double *fat, double *lng) {
  orc_coeffs c1 = {1.0 / 8.0, 0.0, (-1.0 / 8.0) * 0.5, (1.0 / 8.0) * 0.25 * 0.5,
                   (-1.0 / 8.0) * 0.125 * (1.0 / 6.0), 0.0};
  orc_coeffs c2 = {(1.0 / 8.0) + (2.0 * 6.0 / 16.0) + (1.0 / 8.0), -1.0 / 24.0, (-1.0 / 8.0) * 0.5,
                   (1.0 / 8.0) * 0.25 * 0.5, (-1.0 / 8.0) * 0.125 * (1.0 / 6.0), -2.0 / 16};
  orc_coeffs c3 = {1.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0};
  size_t nl = L->V * 4 * 18;
  orc_load_fatlinks(L, U, &c1, Vl);
  int nsvd = 0;
  long long nl4 = (long long)(4 * L->V);
#pragma omp parallel for schedule(static) reduction(+ : nsvd)
  for (long long k = 0; k < nl4; k++) nsvd += orc_u3_unitarize(Vl + 18 * k, W + 18 * k);
  if (n_naiks > 1) {
    double *f3 = (double *)malloc(nl * sizeof(double));
    double *l3 = (double *)malloc(nl * sizeof(double));
    orc_load_fatlinks(L, W, &c3, f3);
    orc_load_lnglinks(L, W, &c3, l3);
    orc_load_fatlinks(L, W, &c2, fat);
    orc_load_lnglinks(L, W, &c2, lng);
    for (int in = 1; in < n_naiks; in++)
      for (size_t k = 0; k < nl; k++) {
        fat[in * nl + k] = eps_naik[in] * f3[k] + fat[k];
        lng[in * nl + k] = eps_naik[in] * l3[k] + lng[k];
      }
    free(f3); free(l3);
  } else {
    orc_load_fatlinks(L, W, &c2, fat);
    orc_load_lnglinks(L, W, &c2, lng);
  }
  return nsvd;
}
