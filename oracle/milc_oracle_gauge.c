/* milc_oracle_gauge.c -- CPU restatement of MILC's gauge-field side of the
 * RHMC molecular dynamics.  TEST INFRASTRUCTURE ONLY (see milc_oracle.h).
 *
 *   orc_loop_table      generic/gauge_stuff.c:87-197 (make_loop_table) with
 *                       generic/imp_actions/symanzik_1loop_hisq_action.h
 *   orc_gauge_action    (beta/3) * imp_gauge_action, gauge_stuff.c:277-330,
 *                       as d_action_rhmc.c:27-29 calls it (phases out)
 *   orc_gauge_force     imp_gauge_force_cpu, generic/gauge_force_imp.c:37-223
 *   orc_update_u        ks_imp_rhmc/update_u.c:49-108 (8th-order Taylor)
 *   orc_hmom_action     ks_imp_rhmc/d_action_rhmc.c:89-122
 *   orc_reunitarize     generic/reunitarize2.c:112-216 on every link
 *   orc_prn_*           generic/ranstuff.c:60-110 (64-bit congruence
 *                       variant), libraries/gaussrand.c:78-100,
 *                       libraries/rand_ahmat.c:36-52, generic/ranmom.c
 *   orc_plaquette       generic/d_plaq4.c
 *
 * Links are MILC's su3_matrix[4*i+dir] without staggered phases, momenta
 * anti_hermitmat[4*i+dir] (10 doubles), i the MILC site index.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "milc_oracle.h"

#define RE(m, i, j) (m)[2 * (3 * (i) + (j))]
#define IM(m, i, j) (m)[2 * (3 * (i) + (j)) + 1]

static void mnn(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += RE(a, i, k) * RE(b, k, j) - IM(a, i, k) * IM(b, k, j);
        im += RE(a, i, k) * IM(b, k, j) + IM(a, i, k) * RE(b, k, j);
      }
      RE(c, i, j) = re;
      IM(c, i, j) = im;
    }
}
static void mna(const double *a, const double *b, double *c) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += RE(a, i, k) * RE(b, j, k) + IM(a, i, k) * IM(b, j, k);
        im += IM(a, i, k) * RE(b, j, k) - RE(a, i, k) * IM(b, j, k);
      }
      RE(c, i, j) = re;
      IM(c, i, j) = im;
    }
}
static void unit(double *m) {
  memset(m, 0, 18 * sizeof(double));
  RE(m, 0, 0) = RE(m, 1, 1) = RE(m, 2, 2) = 1.0;
}

/* ---------------------------------------------------------------- loops */

/* smallest integer label over cyclic shifts and the reversed path: two
   paths with the same label are the same loop (gauge_stuff.c:237-275) */
static int loop_label(const int *dig, int length) {
  int tenl = 1, chr, old, newv, bdig[8] = {0};
  for (int j = 0; j < length - 1; j++) tenl *= 10;
  chr = dig[length - 1];
  for (int j = length - 2; j >= 0; j--) chr = chr * 10 + dig[j];
  old = chr;
  for (int j = length - 1; j >= 1; j--) {
    newv = (old - tenl * dig[j]) * 10 + dig[j];
    if (newv < chr) chr = newv;
    old = newv;
  }
  for (int j = 0; j < length; j++) bdig[j] = 7 - dig[length - j - 1];
  old = bdig[length - 1];
  for (int j = length - 2; j >= 0; j--) old = old * 10 + bdig[j];
  if (old < chr) chr = old;
  for (int j = length - 1; j >= 1; j--) {
    newv = (old - tenl * bdig[j]) * 10 + bdig[j];
    if (newv < chr) chr = newv;
    old = newv;
  }
  return chr;
}

void orc_loop_table(int nflavors, double u0, orc_loops *T) {
  static const int base[3][6] = {{0, 1, 7, 6, -1, -1}, {0, 0, 1, 7, 7, 6}, {0, 1, 2, 7, 6, 5}};
  static const int blen[3] = {4, 6, 6};
  memset(T, 0, sizeof *T);
  T->nloop = 3;
  const double lu = log(u0);
  T->coeff[0] = 1.0;
  T->coeff[1] = -1.0 / (20.0 * u0 * u0) * (1.0 - (0.6264 - 1.1746 * nflavors) * lu);
  T->coeff[2] = 1.0 / (u0 * u0) * (0.0433 - 0.0156 * nflavors) * lu;
  for (int il = 0; il < 3; il++) {
    int count = 0, labels[ORC_MAX_LOOPS];
    T->length[il] = blen[il];
    int perm[4], ir[4], pp[8], vec[6];
    for (perm[0] = 0; perm[0] < 4; perm[0]++)
      for (perm[1] = 0; perm[1] < 4; perm[1]++)
        for (perm[2] = 0; perm[2] < 4; perm[2]++)
          for (perm[3] = 0; perm[3] < 4; perm[3]++) {
            if (perm[0] == perm[1] || perm[0] == perm[2] || perm[0] == perm[3] || perm[1] == perm[2] ||
                perm[1] == perm[3] || perm[2] == perm[3])
              continue;
            for (ir[0] = 0; ir[0] < 2; ir[0]++)
              for (ir[1] = 0; ir[1] < 2; ir[1]++)
                for (ir[2] = 0; ir[2] < 2; ir[2]++)
                  for (ir[3] = 0; ir[3] < 2; ir[3]++) {
                    for (int j = 0; j < 4; j++) {
                      pp[j] = ir[j] ? 7 - perm[j] : perm[j];
                      pp[7 - j] = 7 - pp[j];
                    }
                    for (int j = 0; j < blen[il]; j++) vec[j] = pp[base[il][j]];
                    int chr = loop_label(vec, blen[il]), seen = 0;
                    for (int j = 0; j < count; j++)
                      if (labels[j] == chr) seen = 1;
                    if (!seen) {
                      labels[count] = chr;
                      for (int j = 0; j < blen[il]; j++) T->dirs[il][count][j] = vec[j];
                      count++;
                    }
                  }
          }
    T->num[il] = count;
  }
}

/* product of links along `path` (MILC directions, 0-3 forward, 7-d
   backward along d) starting at site x */
static void path_from(const orc_lat *L, const double *U, size_t x, const int *path, int len, double *P) {
  double t[18];
  unit(P);
  size_t y = x;
  for (int k = 0; k < len; k++) {
    int d = path[k];
    if (d < 4) {
      mnn(P, U + (4 * y + d) * 18, t);
      y = L->nb[16 * y + d];
    } else {
      y = L->nb[16 * y + d];
      mna(P, U + (4 * y + (7 - d)) * 18, t);
    }
    memcpy(P, t, sizeof t);
  }
}

double orc_gauge_action(const orc_lat *L, const double *U, double beta, double u0, int nflavors) {
  orc_loops T;
  orc_loop_table(nflavors, u0, &T);
  double total = 0;
  for (int il = 0; il < T.nloop; il++)
    for (int ln = 0; ln < T.num[il]; ln++) {
      double part = 0;
#pragma omp parallel for reduction(+ : part)
      for (size_t x = 0; x < L->V; x++) {
        double P[18];
        path_from(L, U, x, T.dirs[il][ln], T.length[il], P);
        part += T.coeff[il] * (3.0 - (RE(P, 0, 0) + RE(P, 1, 1) + RE(P, 2, 2)));
      }
      total += part;
    }
  return beta / 3.0 * total;
}

/* mom_mu(x) <- TA(mom_mu(x) - eps beta/3 U_mu(x) sum_loops c Q), Q the rest
   of each loop through the link, traversed from x+mu back to x */
void orc_gauge_force(const orc_lat *L, const double *U, double eps, double beta, double u0, int nflavors,
                     double *mom) {
  orc_loops T;
  orc_loop_table(nflavors, u0, &T);
  const double eb3 = eps * beta / 3.0;
  for (int dir = 0; dir < 4; dir++) {
    /* staple paths for links in direction dir (gauge_force_imp.c:121-155) */
    int npath = 0, plen[ORC_MAX_STAPLES], paths[ORC_MAX_STAPLES][6];
    double pc[ORC_MAX_STAPLES];
    for (int il = 0; il < T.nloop; il++)
      for (int ln = 0; ln < T.num[il]; ln++) {
        int len = T.length[il], dirs[6];
        for (int k = 0; k < len; k++) {
          int d = T.dirs[il][ln][k];
          dirs[k] = d < 4 ? (dir + d) % 4 : 7 - ((dir + 7 - d) % 4);
        }
        for (int k = 0; k < len; k++) {
          if (dirs[k] != dir && dirs[k] != 7 - dir) continue;
          if (dirs[k] < 4)
            for (int j = 0; j < len - 1; j++) paths[npath][j] = dirs[(k + j + 1) % len];
          else
            for (int j = 0; j < len - 1; j++) paths[npath][len - 2 - j] = 7 - dirs[(k + j + 1) % len];
          plen[npath] = len - 1;
          pc[npath] = T.coeff[il];
          npath++;
        }
      }
#pragma omp parallel for
    for (size_t x = 0; x < L->V; x++) {
      double S[18], P[18], G[18];
      memset(S, 0, sizeof S);
      const size_t xp = L->nb[16 * x + dir];
      for (int p = 0; p < npath; p++) {
        path_from(L, U, xp, paths[p], plen[p], P);
        for (int k = 0; k < 18; k++) S[k] += pc[p] * P[k];
      }
      mnn(U + (4 * x + dir) * 18, S, G);
      double *m = mom + (4 * x + dir) * 10;
      double A[18];
      memset(A, 0, sizeof A);
      RE(A, 0, 1) = m[0]; IM(A, 0, 1) = m[1];
      RE(A, 0, 2) = m[2]; IM(A, 0, 2) = m[3];
      RE(A, 1, 2) = m[4]; IM(A, 1, 2) = m[5];
      RE(A, 1, 0) = -m[0]; IM(A, 1, 0) = m[1];
      RE(A, 2, 0) = -m[2]; IM(A, 2, 0) = m[3];
      RE(A, 2, 1) = -m[4]; IM(A, 2, 1) = m[5];
      IM(A, 0, 0) = m[6]; IM(A, 1, 1) = m[7]; IM(A, 2, 2) = m[8];
      for (int k = 0; k < 18; k++) A[k] -= eb3 * G[k];
      double tr = (IM(A, 0, 0) + IM(A, 1, 1) + IM(A, 2, 2)) * 0.33333333333333333;
      m[6] = IM(A, 0, 0) - tr; m[7] = IM(A, 1, 1) - tr; m[8] = IM(A, 2, 2) - tr;
      m[0] = (RE(A, 0, 1) - RE(A, 1, 0)) * 0.5; m[1] = (IM(A, 0, 1) + IM(A, 1, 0)) * 0.5;
      m[2] = (RE(A, 0, 2) - RE(A, 2, 0)) * 0.5; m[3] = (IM(A, 0, 2) + IM(A, 2, 0)) * 0.5;
      m[4] = (RE(A, 1, 2) - RE(A, 2, 1)) * 0.5; m[5] = (IM(A, 1, 2) + IM(A, 2, 1)) * 0.5;
    }
  }
}

static void uncompress(const double *m, double *A) {
  memset(A, 0, 18 * sizeof(double));
  RE(A, 0, 1) = m[0]; IM(A, 0, 1) = m[1];
  RE(A, 0, 2) = m[2]; IM(A, 0, 2) = m[3];
  RE(A, 1, 2) = m[4]; IM(A, 1, 2) = m[5];
  RE(A, 1, 0) = -m[0]; IM(A, 1, 0) = m[1];
  RE(A, 2, 0) = -m[2]; IM(A, 2, 0) = m[3];
  RE(A, 2, 1) = -m[4]; IM(A, 2, 1) = m[5];
  IM(A, 0, 0) = m[6]; IM(A, 1, 1) = m[7]; IM(A, 2, 2) = m[8];
}

/* U <- exp(eps H) U to eighth order, Horner form (update_u.c:74-96) */
void orc_update_u(const orc_lat *L, double *U, const double *mom, double eps) {
  const double t[9] = {0, eps, eps / 2.0, eps / 3.0, eps / 4.0, eps / 5.0, eps / 6.0, eps / 7.0, eps / 8.0};
#pragma omp parallel for
  for (size_t x = 0; x < L->V; x++)
    for (int dir = 0; dir < 4; dir++) {
      double H[18], T1[18], T2[18], *link = U + (4 * x + dir) * 18;
      uncompress(mom + (4 * x + dir) * 10, H);
      mnn(H, link, T1);
      for (int k = 0; k < 18; k++) T2[k] = link[k] + t[8] * T1[k];
      for (int o = 7; o >= 1; o--) {
        mnn(H, T2, T1);
        for (int k = 0; k < 18; k++) T2[k] = link[k] + t[o] * T1[k];
      }
      memcpy(link, T2, sizeof T2);
    }
}

double orc_hmom_action(const orc_lat *L, const double *mom) {
  double sum = 0;
  for (size_t x = 0; x < L->V; x++)
    for (int dir = 0; dir < 4; dir++) {
      const double *m = mom + (4 * x + dir) * 10;
      double s = 0.5 * (m[6] * m[6] + m[7] * m[7] + m[8] * m[8]);
      for (int k = 0; k < 6; k++) s += m[k] * m[k];
      sum += s - 4.0;
    }
  return sum;
}

/* reunit_su3 on every link (generic/reunitarize2.c:112-216): normalise
   row 0, orthogonalise and normalise row 1, row 2 = (row0 x row1)^* */
void orc_reunitarize(const orc_lat *L, double *U) {
#pragma omp parallel for
  for (size_t k = 0; k < 4 * L->V; k++) {
    double *c = U + 18 * k;
    double n0 = 0;
    for (int j = 0; j < 6; j++) n0 += c[j] * c[j];
    n0 = 1.0 / sqrt(n0);
    for (int j = 0; j < 6; j++) c[j] *= n0;
    double ar = 0, ai = 0;
    for (int j = 0; j < 3; j++) {
      ar += RE(c, 0, j) * RE(c, 1, j) + IM(c, 0, j) * IM(c, 1, j);
      ai += RE(c, 0, j) * IM(c, 1, j) - IM(c, 0, j) * RE(c, 1, j);
    }
    for (int j = 0; j < 3; j++) {
      double r0 = RE(c, 0, j), i0 = IM(c, 0, j);
      RE(c, 1, j) -= ar * r0 - ai * i0;
      IM(c, 1, j) -= ar * i0 + ai * r0;
    }
    double n1 = 0;
    for (int j = 6; j < 12; j++) n1 += c[j] * c[j];
    n1 = 1.0 / sqrt(n1);
    for (int j = 6; j < 12; j++) c[j] *= n1;
    /* row 2 = conj(row0 x row1) */
    for (int j = 0; j < 3; j++) {
      int a = (j + 1) % 3, b = (j + 2) % 3;
      double re = RE(c, 0, a) * RE(c, 1, b) - IM(c, 0, a) * IM(c, 1, b) - (RE(c, 0, b) * RE(c, 1, a) - IM(c, 0, b) * IM(c, 1, a));
      double im = RE(c, 0, a) * IM(c, 1, b) + IM(c, 0, a) * RE(c, 1, b) - (RE(c, 0, b) * IM(c, 1, a) + IM(c, 0, b) * RE(c, 1, a));
      RE(c, 2, j) = re;
      IM(c, 2, j) = -im;
    }
  }
}

void orc_plaquette(const orc_lat *L, const double *U, double *ss, double *st) {
  double s1 = 0, s2 = 0;
  for (size_t x = 0; x < L->V; x++)
    for (int mu = 0; mu < 4; mu++)
      for (int nu = mu + 1; nu < 4; nu++) {
        const int path[4] = {mu, nu, 7 - mu, 7 - nu};
        double P[18];
        path_from(L, U, x, path, 4, P);
        double tr = RE(P, 0, 0) + RE(P, 1, 1) + RE(P, 2, 2);
        if (nu == 3) s2 += tr; else s1 += tr;
      }
  *ss = s1 / (3.0 * L->V);
  *st = s2 / (3.0 * L->V);
}

/* ---------------------------------------------------------------- RNG */

void orc_prn_init(orc_prn *p, int seed, int index) {
  /* 32-bit wrap-around arithmetic of the int seed (ranstuff.c:67-90) */
  uint32_t s = (uint32_t)seed;
  const uint32_t a = (uint32_t)(69607 + 8 * index);
  uint32_t r[7];
  for (int k = 0; k < 7; k++) {
    s = a * s + 12345u;
    r[k] = ((uint32_t)((int32_t)s >> 8)) & 0xffffffu;
  }
  s = a * s + 12345u;
  for (int k = 0; k < 7; k++) p->r[k] = r[k];
  p->ic_state = (uint64_t)(int64_t)(int32_t)s;
  p->multiplier = 100000005ull + 8ull * (uint64_t)index;
  p->addend = 12345ull;
}

double orc_myrand(orc_prn *p) {
  uint32_t t = (((p->r[5] >> 7) | (p->r[6] << 17)) ^ ((p->r[4] >> 1) | (p->r[5] << 23))) & 0xffffffu;
  for (int k = 6; k > 0; k--) p->r[k] = p->r[k - 1];
  p->r[0] = t;
  uint64_t s = p->ic_state * p->multiplier + p->addend;
  p->ic_state = s;
  return (double)(1.0f / (float)0x1000000) * (double)(t ^ ((s >> 40) & 0xffffffu));
}

double orc_gaussian(orc_prn *p) {
  double v1, v2, r;
  do {
    v1 = 2.0 * orc_myrand(p) - 1.0;
    v2 = 2.0 * orc_myrand(p) - 1.0;
    r = v1 * v1 + v2 * v2;
  } while (r >= 1.0);
  return v2 * sqrt(-log(r) / r);
}

void orc_complex_gaussian(orc_prn *p, double *re, double *im) {
  double v1, v2, r;
  do {
    v1 = 2.0 * orc_myrand(p) - 1.0;
    v2 = 2.0 * orc_myrand(p) - 1.0;
    r = v1 * v1 + v2 * v2;
  } while (r >= 1.0);
  double fac = sqrt(-log(r) / r);
  *re = v2 * fac;
  *im = v1 * fac;
}

void orc_site_prn_init(const orc_lat *L, int seed, orc_prn *prn) {
  for (size_t i = 0; i < L->V; i++) {
    const int *c = L->coord + 4 * i;
    int index = c[0] + L->dims[0] * (c[1] + L->dims[1] * (c[2] + L->dims[2] * c[3]));
    orc_prn_init(prn + i, seed, index);
  }
}

/* ranmom: random_anti_hermitian per site and direction, site generators */
void orc_ranmom(const orc_lat *L, orc_prn *prn, double *mom) {
  const double sqrt_third = sqrt(1.0 / 3.0);
  for (size_t i = 0; i < L->V; i++)
    for (int dir = 0; dir < 4; dir++) {
      double *m = mom + (4 * i + dir) * 10, r, s;
      orc_complex_gaussian(prn + i, &r, &s);
      m[6] = r + sqrt_third * s;
      m[7] = -r + sqrt_third * s;
      m[8] = -2.0 * sqrt_third * s;
      orc_complex_gaussian(prn + i, &m[0], &m[1]);
      orc_complex_gaussian(prn + i, &m[2], &m[3]);
      orc_complex_gaussian(prn + i, &m[4], &m[5]);
      m[9] = 0.0;
    }
}

/* three complex Gaussians per site of `parity` (grsource_rhmc.c:31-41) */
void orc_gaussian_vector(const orc_lat *L, orc_prn *prn, int parity, double *v) {
  for (size_t i = 0; i < L->V; i++) {
    int even = i < L->Vh;
    if (!((parity & ORC_EVEN) && even) && !((parity & ORC_ODD) && !even)) continue;
    for (int c = 0; c < 3; c++) orc_complex_gaussian(prn + i, v + 6 * i + 2 * c, v + 6 * i + 2 * c + 1);
  }
}
