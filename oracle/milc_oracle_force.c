/* milc_oracle_force.c -- CPU restatement of the HISQ fermion force.
 * TEST INFRASTRUCTURE ONLY (see milc_oracle.h).
 *
 * MILC's eo_fermion_force_multi (generic_ks/fermion_force_hisq_multi.c:
 * 170-219, wrapper_mx_cpu :1182-1475) differentiates
 *   S = sum_j res_j phi^dag (sigma_j - D_eo D_oe)^-1 phi
 * through the Naik/fat smearing of W, the U(3) projection W(V) and the
 * fat7 smearing V(U).  Its own implementation walks the sorted path
 * tables; this restatement differentiates the same link construction by
 * reverse mode through the optimised staple recursion used to build the
 * links (load_fatlinks_cpu, generic_ks/fermion_links_fn_load_milc.c:
 * 207-253), written with serial scatter loops.  The two agree because the
 * derivative is only ever contracted with tangent directions of U(3)
 * (dW = A W, A anti-Hermitian), along which the retraced paths that
 * distinguish the recursion from the path sum have zero derivative.
 *
 * Conventions.  For a link-like field Z, K_Z denotes the matrix with
 * dS = 2 Re sum tr(K_Z dZ).  The fermion bilinear gives
 * dS = 2 Re sum_j res_j X_j^dag dD_eo Y_j, Y_j = D_oe X_j, so a fat link
 * F_mu(z) receives K = s(z) res_j xxx_j(z+mu) xxx_j(z)^dag with s = +1 on
 * even z and -1 on odd z, where xxx_j holds X_j on even and Y_j on odd
 * sites (ks_imp_rhmc/update_h_rhmc.c:82-87); the Naik link uses z+3mu.
 * The momentum update is mom_mu(x) <- TA(mom_mu(x) + 2 eps U_mu(x) K_U(x))
 * up to the overall sign fixed against MILC (ORC_FORCE_SIGN below).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "milc_oracle.h"

#define RE(m, i, j) (m)[2 * (3 * (i) + (j))]
#define IM(m, i, j) (m)[2 * (3 * (i) + (j)) + 1]

/* overall sign and factor of the momentum update relative to
   TA(U K_U); fixed by comparison with MILC's own force */
#define ORC_FORCE_FACTOR (2.0)

static void mnn(const double *a, const double *b, double *c) {
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
static void adj(const double *a, double *c) {
  double r[18];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) { RE(r, i, j) = RE(a, j, i); IM(r, i, j) = -IM(a, j, i); }
  memcpy(c, r, sizeof r);
}
static void mna(const double *a, const double *b, double *c) { double t[18]; adj(b, t); mnn(a, t, c); }
static void man(const double *a, const double *b, double *c) { double t[18]; adj(a, t); mnn(t, b, c); }
static void acc(double *d, const double *s, double f) { for (int k = 0; k < 18; k++) d[k] += f * s[k]; }
static void acc_adj(double *d, const double *s, double f) { double t[18]; adj(s, t); acc(d, t, f); }

/* forward staple S(x) (generic/general_staple.c:42-140) */
static void staple_fwd(const orc_lat *L, int mu, int nu, const double *A, int stride, const double *U, double *S) {
  for (size_t x = 0; x < L->V; x++) {
    const size_t *nb = L->nb + 16 * x;
    size_t xpnu = nb[nu], xpmu = nb[mu], xmnu = nb[7 - nu], xmnupmu = L->nb[16 * xmnu + mu];
    double t[18], up[18], dn[18];
    mna(A + stride * 18 * xpnu, U + (4 * xpmu + nu) * 18, t);
    mnn(U + (4 * x + nu) * 18, t, up);
    man(U + (4 * xmnu + nu) * 18, A + stride * 18 * xmnu, t);
    mnn(t, U + (4 * xmnupmu + nu) * 18, dn);
    for (int q = 0; q < 18; q++) S[18 * x + q] = up[q] + dn[q];
  }
}

/* reverse of staple_fwd: given K (adjoint of S, one matrix per site, scaled
   by f), accumulate K_A (stride like A) and K_U for the links U_nu. */
static void staple_adj(const orc_lat *L, int mu, int nu, const double *A, int stride, const double *U,
                       const double *K, double f, double *KA, double *KU) {
  for (size_t x = 0; x < L->V; x++) {
    const size_t *nb = L->nb + 16 * x;
    size_t xpnu = nb[nu], xpmu = nb[mu], xmnu = nb[7 - nu], xmnupmu = L->nb[16 * xmnu + mu];
    const double *Kx = K + 18 * x;
    const double *Ux = U + (4 * x + nu) * 18, *Upmu = U + (4 * xpmu + nu) * 18;
    const double *Umnu = U + (4 * xmnu + nu) * 18, *Umnupmu = U + (4 * xmnupmu + nu) * 18;
    const double *Ap = A + stride * 18 * xpnu, *Am = A + stride * 18 * xmnu;
    double t[18], t2[18];
    /* upper  U_nu(x) A(x+nu) U_nu(x+mu)^dag */
    mna(Ap, Upmu, t); mnn(t, Kx, t2); acc(KU + (4 * x + nu) * 18, t2, f);              /* C K */
    man(Upmu, Kx, t); mnn(t, Ux, t2); acc(KA + stride * 18 * xpnu, t2, f);             /* R K L */
    mnn(Kx, Ux, t); mnn(t, Ap, t2); acc_adj(KU + (4 * xpmu + nu) * 18, t2, f);         /* (K L)^dag */
    /* lower  U_nu(x-nu)^dag A(x-nu) U_nu(x-nu+mu) */
    mnn(Am, Umnupmu, t); mnn(t, Kx, t2); acc_adj(KU + (4 * xmnu + nu) * 18, t2, f);    /* (R K)^dag */
    mnn(Umnupmu, Kx, t); mna(t, Umnu, t2); acc(KA + stride * 18 * xmnu, t2, f);        /* R K L */
    mna(Kx, Umnu, t); mnn(t, Am, t2); acc(KU + (4 * xmnupmu + nu) * 18, t2, f);        /* K L */
  }
}

/* reverse of orc_load_fatlinks (same recursion, intermediates recomputed) */
static void fat_adj(const orc_lat *L, const double *links, const orc_coeffs *c, const double *Kfat, double *KU) {
  size_t n = L->V * 18;
  double one_link = c->one_link - 6.0 * c->lepage;
  double *S1 = malloc(n * sizeof(double)), *S2 = malloc(n * sizeof(double));
  double *K1 = malloc(n * sizeof(double)), *K2 = malloc(n * sizeof(double));
  double *Kd = malloc(n * sizeof(double));
  for (int dir = 0; dir < 4; dir++) {
    for (size_t x = 0; x < L->V; x++) {
      acc(KU + (4 * x + dir) * 18, Kfat + (4 * x + dir) * 18, one_link);
      memcpy(Kd + 18 * x, Kfat + (4 * x + dir) * 18, 18 * sizeof(double));
    }
    if (c->three_staple == 0.0 && c->lepage == 0.0 && c->five_staple == 0.0) continue;
    for (int nu = 0; nu < 4; nu++) {
      if (nu == dir) continue;
      staple_fwd(L, dir, nu, links + 18 * dir, 4, links, S1);
      for (size_t k = 0; k < n; k++) K1[k] = c->three_staple * Kd[k];
      if (c->lepage != 0.0) staple_adj(L, dir, nu, S1, 1, links, Kd, c->lepage, K1, KU);
      for (int rho = 0; rho < 4; rho++) {
        if (rho == dir || rho == nu) continue;
        staple_fwd(L, dir, rho, S1, 1, links, S2);
        for (size_t k = 0; k < n; k++) K2[k] = c->five_staple * Kd[k];
        for (int sig = 0; sig < 4; sig++) {
          if (sig == dir || sig == nu || sig == rho) continue;
          staple_adj(L, dir, sig, S2, 1, links, Kd, c->seven_staple, K2, KU);
        }
        staple_adj(L, dir, rho, S1, 1, links, K2, 1.0, K1, KU);
      }
      staple_adj(L, dir, nu, links + 18 * dir, 4, links, K1, 1.0, KU + 18 * dir, KU);
    }
  }
  free(S1); free(S2); free(K1); free(K2); free(Kd);
}

/* reverse of the Naik product L_mu(x) = c W_mu(x) W_mu(x+mu) W_mu(x+2mu) */
static void naik_adj(const orc_lat *L, const double *W, double c, const double *Klng, double *KW) {
  for (size_t x = 0; x < L->V; x++)
    for (int mu = 0; mu < 4; mu++) {
      size_t x1 = L->nb[16 * x + mu], x2 = L->nb[16 * x1 + mu];
      const double *K = Klng + (4 * x + mu) * 18;
      const double *W0 = W + (4 * x + mu) * 18, *W1 = W + (4 * x1 + mu) * 18, *W2 = W + (4 * x2 + mu) * 18;
      double t[18], t2[18];
      mnn(W1, W2, t); mnn(t, K, t2); acc(KW + (4 * x + mu) * 18, t2, c);
      mnn(W2, K, t); mnn(t, W0, t2); acc(KW + (4 * x1 + mu) * 18, t2, c);
      mnn(K, W0, t); mnn(t, W1, t2); acc(KW + (4 * x2 + mu) * 18, t2, c);
    }
}

/* reverse of W = V (V^dag V)^-1/2 for one link.  With Q = V^dag V,
   R = Q^-1/2 = f0 + f1 Q + f2 Q^2 (f_i rational in u = sum s_a,
   v = sum_{a<b} s_a s_b, w = s0 s1 s2, s_a = sqrt of the eigenvalues of Q,
   as in u3_unitarize_analytic), and du = tr(R dQ)/2,
   dv = tr((u R - 1) dQ)/2, dw = (w/2) tr(R^2 dQ):
     K_V = R K_W + (N + N^dag) V^dag,
     N = sum_i tr(M Q^i) Psi_i + f1 M + f2 (Q M + M Q),  M = K_W V,
     Psi_i = df_i/du R/2 + df_i/dv (u R - 1)/2 + df_i/dw (w/2) R^2.
   The eigenvalue filter of generic_ks/su3_mat_op.c:1680-1734
   (HISQ_FORCE_FILTER = 5e-5) is applied the same way: below it, Q and
   the eigenvalues are shifted by the filter before differentiating. */
static int unit_adj(const double *V, const double *KW, double *KV) {
  double Q[18], Q2[18], R[18], R2[18], M[18], N[18], t[18], Vd[18];
  man(V, V, Q);
  double c0 = RE(Q, 0, 0) + RE(Q, 1, 1) + RE(Q, 2, 2);
  mnn(Q, Q, Q2);
  double c1 = (RE(Q2, 0, 0) + RE(Q2, 1, 1) + RE(Q2, 2, 2)) / 2;
  double q3 = 0;
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) q3 += RE(Q2, i, k) * RE(Q, k, i) - IM(Q2, i, k) * IM(Q, k, i);
  double c2 = q3 / 3, g[3];
  double S = c1 / 3 - c0 * (c0 / 18);
  if (fabs(S) < 1.0e-14) {
    g[0] = g[1] = g[2] = c0 / 3;
  } else {
    double Rr = c2 / 2 - c0 * (c1 / 3) + c0 * c0 * (c0 / 27);
    S = sqrt(S);
    double RoS = Rr / (S * S * S), theta;
    if (!(fabs(RoS) < 1.0)) theta = Rr > 0 ? 0.0 : 3.14159265358979323846264338328;
    else theta = acos(RoS);
    double th3 = theta / 3, pi23 = 6.28318530717958647692528676656 / 3;
    g[0] = c0 / 3 + 2 * S * cos(th3);
    g[1] = c0 / 3 + 2 * S * cos(th3 + pi23);
    g[2] = c0 / 3 + 2 * S * cos(th3 + 2 * pi23);
  }
  int filtered = 0;
  double gmin = g[0] < g[1] ? g[0] : g[1];
  gmin = gmin < g[2] ? gmin : g[2];
  if (gmin < 5.0e-5) {
    filtered = 1;
    for (int a = 0; a < 3; a++) g[a] += 5.0e-5;
    for (int i = 0; i < 3; i++) RE(Q, i, i) += 5.0e-5;
    mnn(Q, Q, Q2);
  }
  double s0 = sqrt(g[0]), s1 = sqrt(g[1]), s2 = sqrt(g[2]);
  double u = s0 + s1 + s2, v = s0 * s1 + s0 * s2 + s1 * s2, w = s0 * s1 * s2;
  double D = w * (u * v - w);
  double f0 = (u * v * v - w * (u * u + v)) / D;
  double f1 = (2 * u * v - w - u * u * u) / D;
  double f2 = u / D;
  double Du = v * w, Dv = u * w, Dw = u * v - 2 * w;
  double fu[3], fv[3], fw[3];
  fu[0] = (v * v - 2 * u * w) / D - f0 * Du / D;
  fv[0] = (2 * u * v - w) / D - f0 * Dv / D;
  fw[0] = (-u * u - v) / D - f0 * Dw / D;
  fu[1] = (2 * v - 3 * u * u) / D - f1 * Du / D;
  fv[1] = (2 * u) / D - f1 * Dv / D;
  fw[1] = -1.0 / D - f1 * Dw / D;
  fu[2] = 1.0 / D - f2 * Du / D;
  fv[2] = -f2 * Dv / D;
  fw[2] = -f2 * Dw / D;
  for (int k = 0; k < 18; k++) R[k] = f1 * Q[k] + f2 * Q2[k];
  for (int i = 0; i < 3; i++) RE(R, i, i) += f0;
  mnn(R, R, R2);
  mnn(KW, V, M);
  /* tr(M Q^i) */
  double trMQ[3][2];
  const double *Qp[3] = {NULL, Q, Q2};
  for (int i = 0; i < 3; i++) {
    double re = 0, im = 0;
    if (i == 0) {
      for (int a = 0; a < 3; a++) { re += RE(M, a, a); im += IM(M, a, a); }
    } else {
      mnn(M, Qp[i], t);
      for (int a = 0; a < 3; a++) { re += RE(t, a, a); im += IM(t, a, a); }
    }
    trMQ[i][0] = re; trMQ[i][1] = im;
  }
  /* N */
  double QM[18], MQ[18];
  mnn(Q, M, QM); mnn(M, Q, MQ);
  for (int k = 0; k < 18; k++) N[k] = f1 * M[k] + f2 * (QM[k] + MQ[k]);
  for (int i = 0; i < 3; i++) {
    /* Psi_i = fu R/2 + fv (u R - 1)/2 + fw (w/2) R^2 (Hermitian) times tr(M Q^i) (complex) */
    double P[18];
    for (int k = 0; k < 18; k++) P[k] = 0.5 * fu[i] * R[k] + 0.5 * fv[i] * u * R[k] + 0.5 * fw[i] * w * R2[k];
    for (int a = 0; a < 3; a++) RE(P, a, a) -= 0.5 * fv[i];
    double tr = trMQ[i][0], ti = trMQ[i][1];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++) {
        double pr = RE(P, a, b), pi = IM(P, a, b);
        RE(N, a, b) += tr * pr - ti * pi;
        IM(N, a, b) += tr * pi + ti * pr;
      }
  }
  /* K_V = R K_W + (N + N^dag) V^dag */
  double Nh[18], t2[18];
  adj(N, t);
  for (int k = 0; k < 18; k++) Nh[k] = N[k] + t[k];
  adj(V, Vd);
  mnn(Nh, Vd, t2);
  mnn(R, KW, t);
  for (int k = 0; k < 18; k++) KV[k] = t[k] + t2[k];
  return filtered;
}

/* level-0 outer products: K(z) += s(z) res xxx(z+hop*mu) xxx(z)^dag */
static void outer(const orc_lat *L, const double *xxx, double res, int hop, double *K) {
  for (size_t z = 0; z < L->V; z++) {
    double s = z < L->Vh ? res : -res;
    for (int mu = 0; mu < 4; mu++) {
      size_t y = L->nb[16 * z + mu + (hop == 3 ? 8 : 0)];
      const double *a = xxx + 6 * y, *b = xxx + 6 * z;
      double *k = K + (4 * z + mu) * 18;
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
          k[2 * (3 * i + j)] += s * (a[2 * i] * b[2 * j] + a[2 * i + 1] * b[2 * j + 1]);
          k[2 * (3 * i + j) + 1] += s * (a[2 * i + 1] * b[2 * j] - a[2 * i] * b[2 * j + 1]);
        }
    }
  }
}

/* K_U for the thin links (phases in) */
static int force_KU(const orc_lat *L, const double *U, int n_naiks, const double *eps_naik,
                    const double *residues, const double *xxx, int nterms, const int *n_orders_naik,
                    double *KU) {
  size_t nl = L->V * 4 * 18;
  orc_coeffs c1 = {1.0 / 8.0, 0.0, -1.0 / 16.0, 1.0 / 64.0, -1.0 / 384.0, 0.0};
  orc_coeffs c2 = {1.0 / 8.0 + 2.0 * 6.0 / 16.0 + 1.0 / 8.0, -1.0 / 24.0, -1.0 / 16.0, 1.0 / 64.0,
                   -1.0 / 384.0, -2.0 / 16.0};
  orc_coeffs c3 = {1.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0};
  double *Vl = calloc(nl, sizeof(double)), *W = calloc(nl, sizeof(double));
  double *Kf = calloc(nl, sizeof(double)), *Kl = calloc(nl, sizeof(double));
  double *KW = calloc(nl, sizeof(double)), *KV = calloc(nl, sizeof(double));
  orc_load_fatlinks(L, U, &c1, Vl);
  for (size_t k = 0; k < 4 * L->V; k++) orc_u3_unitarize(Vl + 18 * k, W + 18 * k);
  /* level 2 with every term (Naik group 0 table covers all terms) */
  for (int j = 0; j < nterms; j++) {
    outer(L, xxx + (size_t)j * 6 * L->V, residues[j], 1, Kf);
    outer(L, xxx + (size_t)j * 6 * L->V, residues[j], 3, Kl);
  }
  fat_adj(L, W, &c2, Kf, KW);
  naik_adj(L, W, c2.naik, Kl, KW);
  /* the epsilon-corrected groups: eps_i (1-link + Naik)(W) for their own terms */
  int off = n_orders_naik[0];
  for (int g = 1; g < n_naiks; g++) {
    memset(Kf, 0, nl * sizeof(double));
    memset(Kl, 0, nl * sizeof(double));
    for (int j = off; j < off + n_orders_naik[g]; j++) {
      outer(L, xxx + (size_t)j * 6 * L->V, residues[j], 1, Kf);
      outer(L, xxx + (size_t)j * 6 * L->V, residues[j], 3, Kl);
    }
    for (size_t k = 0; k < nl; k++) { Kf[k] *= eps_naik[g]; Kl[k] *= eps_naik[g]; }
    fat_adj(L, W, &c3, Kf, KW);
    naik_adj(L, W, c3.naik, Kl, KW);
    off += n_orders_naik[g];
  }
  int nfilt = 0;
  for (size_t k = 0; k < 4 * L->V; k++) nfilt += unit_adj(Vl + 18 * k, KW + 18 * k, KV + 18 * k);
  memset(KU, 0, nl * sizeof(double));
  fat_adj(L, U, &c1, KV, KU);
  free(Vl); free(W); free(Kf); free(Kl); free(KW); free(KV);
  return nfilt;
}

/* mom <- TA(mom + FACTOR eps U K_U) in MILC's anti_hermitmat layout
   (libraries/make_ahmat.c, uncmp_ahmat.c) */
static void mom_update(const orc_lat *L, const double *U, const double *KU, double eps, double *mom) {
  for (size_t x = 0; x < L->V; x++)
    for (int mu = 0; mu < 4; mu++) {
      double G[18];
      mnn(U + (4 * x + mu) * 18, KU + (4 * x + mu) * 18, G);
      double *m = mom + (4 * x + mu) * 10;
      /* uncompress mom, add, take the traceless anti-Hermitian part */
      double A[18];
      memset(A, 0, sizeof A);
      RE(A, 0, 1) = m[0]; IM(A, 0, 1) = m[1];
      RE(A, 0, 2) = m[2]; IM(A, 0, 2) = m[3];
      RE(A, 1, 2) = m[4]; IM(A, 1, 2) = m[5];
      RE(A, 1, 0) = -m[0]; IM(A, 1, 0) = m[1];
      RE(A, 2, 0) = -m[2]; IM(A, 2, 0) = m[3];
      RE(A, 2, 1) = -m[4]; IM(A, 2, 1) = m[5];
      IM(A, 0, 0) = m[6]; IM(A, 1, 1) = m[7]; IM(A, 2, 2) = m[8];
      acc(A, G, ORC_FORCE_FACTOR * eps);
      double tr = (IM(A, 0, 0) + IM(A, 1, 1) + IM(A, 2, 2)) * 0.33333333333333333;
      m[6] = IM(A, 0, 0) - tr; m[7] = IM(A, 1, 1) - tr; m[8] = IM(A, 2, 2) - tr;
      m[0] = (RE(A, 0, 1) - RE(A, 1, 0)) * 0.5; m[1] = (IM(A, 0, 1) + IM(A, 1, 0)) * 0.5;
      m[2] = (RE(A, 0, 2) - RE(A, 2, 0)) * 0.5; m[3] = (IM(A, 0, 2) + IM(A, 2, 0)) * 0.5;
      m[4] = (RE(A, 1, 2) - RE(A, 2, 1)) * 0.5; m[5] = (IM(A, 1, 2) + IM(A, 2, 1)) * 0.5;
    }
}

void orc_fermion_force_hisq(const orc_lat *L, const double *U, int n_naiks, const double *eps_naik,
                            double eps, const double *residues, const double *xxx, int nterms,
                            const int *n_orders_naik, double *mom) {
  size_t nl = L->V * 4 * 18;
  double *KU = malloc(nl * sizeof(double));
  force_KU(L, U, n_naiks, eps_naik, residues, xxx, nterms, n_orders_naik, KU);
  mom_update(L, U, KU, eps, mom);
  free(KU);
}

/* asqtad: one smearing level, fat + Naik links built directly from U with
   the tadpole-improved coefficients and no unitarization, so K_U is the
   fat-link adjoint plus the Naik adjoint of the level-0 outer products.
   MILC walks its sorted path table (fermion_force_fn_multi.c:145-297,
   forward paths doubled); the derivative is the same. */
void orc_fermion_force_asqtad(const orc_lat *L, const double *U, double u0, double eps,
                              const double *residues, const double *xxx, int nterms, double *mom) {
  size_t nl = L->V * 4 * 18;
  orc_coeffs c;
  orc_asqtad_coeffs(u0, &c);
  double *Kf = calloc(nl, sizeof(double)), *Kl = calloc(nl, sizeof(double)), *KU = calloc(nl, sizeof(double));
  for (int j = 0; j < nterms; j++) {
    outer(L, xxx + (size_t)j * 6 * L->V, residues[j], 1, Kf);
    outer(L, xxx + (size_t)j * 6 * L->V, residues[j], 3, Kl);
  }
  fat_adj(L, U, &c, Kf, KU);
  naik_adj(L, U, c.naik, Kl, KU);
  mom_update(L, U, KU, eps, mom);
  free(Kf); free(Kl); free(KU);
}

/* S_lin(U) = 2 Re sum_j res_j X_j^dag D_eo[links(U)] Y_j with X_j, Y_j the
   even / odd parts of xxx_j held fixed: its derivative at fixed X, Y is the
   force above, so central differences of S_lin check the adjoint chain
   without any solve. */
double orc_force_action(const orc_lat *L, const double *U, int n_naiks, const double *eps_naik,
                        const double *residues, const double *xxx, int nterms, const int *n_orders_naik) {
  size_t nl = L->V * 4 * 18;
  double *Vl = malloc(nl * sizeof(double)), *W = malloc(nl * sizeof(double));
  double *fat = malloc((size_t)n_naiks * nl * sizeof(double)), *lng = malloc((size_t)n_naiks * nl * sizeof(double));
  double *Yv = malloc(L->V * 6 * sizeof(double)), *DY = malloc(L->V * 6 * sizeof(double));
  orc_hisq_links(L, U, n_naiks, eps_naik, Vl, W, fat, lng);
  double S = 0;
  int g = 0, left = n_orders_naik[0];
  for (int j = 0; j < nterms; j++) {
    while (left == 0 && g + 1 < n_naiks) left = n_orders_naik[++g];
    left--;
    const double *x = xxx + (size_t)j * 6 * L->V;
    memset(Yv, 0, L->V * 6 * sizeof(double));
    memcpy(Yv + 6 * L->Vh, x + 6 * L->Vh, L->Vh * 6 * sizeof(double));
    orc_dslash(L, fat + (size_t)g * nl, lng + (size_t)g * nl, Yv, DY, ORC_EVEN);
    double s = 0;
    for (size_t k = 0; k < 6 * L->Vh; k++) s += x[k] * DY[k];
    S += 2.0 * residues[j] * s;
  }
  free(Vl); free(W); free(fat); free(lng); free(Yv); free(DY);
  return S;
}
