/* milc_ref_driver.c -- test-infrastructure driver that links MILC's own
 * CPU sources (compiled straight from the reference tree by
 * oracle/ref/Makefile) into oracle/_ref/libmilc_ref_<action>.so.
 *
 * It is the "control.c" of a tiny application: it owns MILC's globals
 * (CONTROL is defined before lattice.h, exactly as an application's
 * control.c does), sets up a single-node lattice, accepts thin links and
 * vectors in MILC's field order through plain pointers, and calls MILC's
 * functions unmodified:
 *   dslash_fn_field             generic_ks/dslash_fn_dblstore.c:285
 *   ks_congrad_parity_cpu       generic_ks/d_congrad5_fn_milc.c:61
 *   ks_multicg_offset_field_cpu generic_ks/ks_multicg_offset.c:63
 *   mat_invert_uml_field        generic_ks/mat_invert.c:328
 *   eo_fermion_force_multi      generic_ks/fermion_force_hisq_multi.c:170
 *   create_fermion_links_from_site generic_ks/fermion_links_from_site.c:14
 * The precedent for a custom driver in place of control.c is
 * ks_imp_rhmc/Make_template:361-398 (control_test_su3_mat_op).
 *
 * This library is a checker only: tests and the golden-fixture script load
 * it to pin the C restatement in oracle/; nothing in the product links it.
 *
 * Field formats (all FP64, MILC_PRECISION=2):
 *   thin links  double[V][4][18]  = lattice[i].link[dir] for MILC index i
 *   fn links    double[V][4][18]  = fat[4*i+dir], lng[4*i+dir]
 *   vectors     double[V][6]      = su3_vector[i]
 *   momenta     double[V][4][10]  = anti_hermitmat mom[dir]
 * i is MILC's node index (even sites first, layout_hyper_prime.c:509-520).
 */
#define CONTROL
#include "ks_imp_includes.h"
#include "quark_action.h"
#include "../include/fermion_links.h"
#include <string.h>

/* Globals normally defined by other application files */
#ifndef DBLSTORE_FN
#error "expected -DDBLSTORE_FN (default MILC CPU build)"
#endif

#if FERM_ACTION == HISQ
#define REF_DESTROY_LINKS(fl) destroy_fermion_links_hisq(fl)
#else
#define REF_DESTROY_LINKS(fl) destroy_fermion_links(fl)
#endif

static int ref_ready = 0;
static int ref_n_naiks = 1;
static double ref_eps_naik[MAX_NAIK];

/* third-neighbour gather, the same geometry as ks_imp_rhmc/setup.c:640 */
static void third_neighbor_ref(int x, int y, int z, int t, int *dirpt, int FB,
                               int *xp, int *yp, int *zp, int *tp) {
  int dir = (FB == FORWARDS) ? *dirpt : OPP_DIR(*dirpt);
  *xp = x; *yp = y; *zp = z; *tp = t;
  switch (dir) {
  case XUP: *xp = (x + 3) % nx; break;
  case XDOWN: *xp = (x + 4 * nx - 3) % nx; break;
  case YUP: *yp = (y + 3) % ny; break;
  case YDOWN: *yp = (y + 4 * ny - 3) % ny; break;
  case ZUP: *zp = (z + 3) % nz; break;
  case ZDOWN: *zp = (z + 4 * nz - 3) % nz; break;
  case TUP: *tp = (t + 3) % nt; break;
  case TDOWN: *tp = (t + 4 * nt - 3) % nt; break;
  default: exit(1);
  }
}

int ref_is_hisq(void) { return FERM_ACTION == HISQ; }

int ref_init(int lx, int ly, int lz, int lt, int n_naiks, const double *eps_naik) {
  int argc = 1, i;
  char *argv0[] = {"milc_ref", NULL};
  char **argv = argv0;
  if (ref_ready) return 1; /* one lattice per process */
  initialize_machine(&argc, &argv);
  this_node = mynode();
  number_of_nodes = numnodes();
  nx = lx; ny = ly; nz = lz; nt = lt;
  volume = (size_t)nx * ny * nz * nt;
  iseed = 1234;
  u0 = 1.0;
  setup_layout();
  make_lattice();
  make_nn_gathers();
  for (i = XUP; i <= TUP; i++)
    make_gather(third_neighbor_ref, &i, WANT_INVERSE, ALLOW_EVEN_ODD, SWITCH_PARITY);
  sort_eight_gathers(X3UP);
  phaseset();
  phases_in = OFF;
  ref_n_naiks = n_naiks < 1 ? 1 : n_naiks;
  for (i = 0; i < MAX_NAIK; i++) ref_eps_naik[i] = 0.0;
  for (i = 0; i < ref_n_naiks; i++) ref_eps_naik[i] = eps_naik ? eps_naik[i] : 0.0;
  /* Naik-epsilon bookkeeping read by the HISQ force (fermion_force_hisq_multi.c:1188-1200) */
  n_order_naik_total = 0;
  for (i = 0; i < MAX_N_PSEUDO; i++) { n_orders_naik[i] = 0; n_pseudo_naik[i] = 0; }
  fn_links = NULL;
  ref_ready = 1;
  return 0;
}

size_t ref_sites(void) { return sites_on_node; }
size_t ref_even_sites(void) { return even_sites_on_node; }

/* Coordinates of MILC index i (so callers can check their own layout). */
void ref_coords(int *xyzt) {
  size_t i;
  for (i = 0; i < sites_on_node; i++) {
    xyzt[4 * i + 0] = lattice[i].x; xyzt[4 * i + 1] = lattice[i].y;
    xyzt[4 * i + 2] = lattice[i].z; xyzt[4 * i + 3] = lattice[i].t;
  }
}

/* Load thin links WITHOUT phases; MILC's rephase(ON) folds in the
   staggered phases and the antiperiodic time boundary (rephase.c:99). */
void ref_set_thin_links(const double *U) {
  size_t i; int dir;
  if (phases_in == ON) rephase(OFF);
  for (i = 0; i < sites_on_node; i++)
    for (dir = 0; dir < 4; dir++)
      memcpy(&lattice[i].link[dir], U + (4 * i + dir) * 18, 18 * sizeof(double));
  rephase(ON);
  if (fn_links != NULL) { REF_DESTROY_LINKS(fn_links); fn_links = NULL; }
}

/* Thin links as MILC holds them (phases in). */
void ref_get_thin_links_phased(double *U) {
  size_t i; int dir;
  for (i = 0; i < sites_on_node; i++)
    for (dir = 0; dir < 4; dir++)
      memcpy(U + (4 * i + dir) * 18, &lattice[i].link[dir], 18 * sizeof(double));
}

/* Tadpole factor of the asqtad path coefficients (ks_action_paths.c divides
   each coefficient by u0^(length-1)); set it before the first
   ref_build_links / ref_fermion_force of the process, as MILC's force
   caches its sorted path table on first use. */
void ref_set_u0(double v) { u0 = v; }

void ref_build_links(void) {
  if (fn_links != NULL) { REF_DESTROY_LINKS(fn_links); fn_links = NULL; }
  /* the DBLSTORE_FN dslash needs back links (ks_imp_rhmc/setup.c:581-584) */
  fermion_links_want_back(1);
  fn_links = create_fermion_links_from_site(MILC_PRECISION, ref_n_naiks, ref_eps_naik);
}

static imp_ferm_links_t *ref_fn(int inaik) { return get_fm_links(fn_links)[inaik]; }

void ref_get_fn_links(int inaik, double *fat, double *lng) {
  imp_ferm_links_t *fn = ref_fn(inaik);
  memcpy(fat, get_fatlinks(fn), 4 * sites_on_node * sizeof(su3_matrix));
  memcpy(lng, get_lnglinks(fn), 4 * sites_on_node * sizeof(su3_matrix));
}

#if FERM_ACTION == HISQ
/* HISQ auxiliary smearing stages U (phased copy), V (fat7), W (U(3) projected) */
void ref_get_hisq_aux(double *U, double *Vl, double *W) {
  hisq_auxiliary_t *aux = get_hisq_auxiliary(fn_links);
  size_t n = 4 * sites_on_node * sizeof(su3_matrix);
  if (U) memcpy(U, aux->U_link, n);
  if (Vl) memcpy(Vl, aux->V_link, n);
  if (W) memcpy(W, aux->W_unitlink, n);
}
#endif

void ref_dslash(const double *src, double *dst, int parity, int inaik) {
  su3_vector *s = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  su3_vector *d = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  memcpy(s, src, sites_on_node * sizeof(su3_vector));
  memcpy(d, dst, sites_on_node * sizeof(su3_vector));
  dslash_fn_field(s, d, parity, ref_fn(inaik));
  memcpy(dst, d, sites_on_node * sizeof(su3_vector));
  free(s); free(d);
}

/* out[0..6] = final_rsq, final_relrsq, size_r, size_relr, final_iters, final_restart, converged */
int ref_congrad(const double *src, double *dst, double mass, int parity,
                double resid, double relresid, int max, int nrestart, int inaik,
                double *out) {
  quark_invert_control qic;
  int iters;
  su3_vector *s = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  su3_vector *d = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  memcpy(s, src, sites_on_node * sizeof(su3_vector));
  memcpy(d, dst, sites_on_node * sizeof(su3_vector));
  memset(&qic, 0, sizeof(qic));
  qic.prec = 2; qic.max = max; qic.nrestart = nrestart; qic.parity = parity;
  qic.resid = resid; qic.relresid = relresid; qic.start_flag = 1;
  iters = ks_congrad_parity_cpu(s, d, &qic, mass, ref_fn(inaik));
  memcpy(dst, d, sites_on_node * sizeof(su3_vector));
  if (out) {
    out[0] = qic.final_rsq; out[1] = qic.final_relrsq; out[2] = qic.size_r;
    out[3] = qic.size_relr; out[4] = qic.final_iters; out[5] = qic.final_restart;
    out[6] = qic.converged;
  }
  free(s); free(d);
  return iters;
}

/* M^-1 on both parities (mat_invert.c:328); out as in ref_congrad for the
   last (odd) solve. */
int ref_mat_invert_uml(const double *src, double *dst, double mass, double resid,
                       int max, int nrestart, int inaik, double *out) {
  quark_invert_control qic;
  int iters;
  su3_vector *s = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  su3_vector *d = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  memcpy(s, src, sites_on_node * sizeof(su3_vector));
  memcpy(d, dst, sites_on_node * sizeof(su3_vector));
  memset(&qic, 0, sizeof(qic));
  qic.prec = 2; qic.max = max; qic.nrestart = nrestart; qic.parity = EVENANDODD;
  qic.resid = resid; qic.relresid = 0; qic.start_flag = 0;
  iters = mat_invert_uml_field(s, d, &qic, mass, ref_fn(inaik));
  memcpy(dst, d, sites_on_node * sizeof(su3_vector));
  if (out) {
    out[0] = qic.final_rsq; out[1] = qic.final_relrsq; out[2] = qic.size_r;
    out[3] = qic.size_relr; out[4] = qic.final_iters; out[5] = qic.final_restart;
    out[6] = qic.converged;
  }
  free(s); free(d);
  return iters;
}

/* psim: num_offsets consecutive vectors of V sites each */
int ref_multicg_offset(const double *src, double *psim, const double *offsets,
                       int num_offsets, int parity, double resid, int max,
                       int nrestart, int inaik, double *final_rsq) {
  int j, iters;
  ks_param *ksp = (ks_param *)malloc(num_offsets * sizeof(ks_param));
  quark_invert_control *qic = (quark_invert_control *)malloc(num_offsets * sizeof(quark_invert_control));
  su3_vector **ps = (su3_vector **)malloc(num_offsets * sizeof(su3_vector *));
  su3_vector *s = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
  memcpy(s, src, sites_on_node * sizeof(su3_vector));
  for (j = 0; j < num_offsets; j++) {
    memset(&ksp[j], 0, sizeof(ks_param));
    ksp[j].offset = offsets[j];
    memset(&qic[j], 0, sizeof(quark_invert_control));
    qic[j].prec = 2; qic[j].max = max; qic[j].nrestart = nrestart;
    qic[j].parity = parity; qic[j].resid = resid; qic[j].relresid = 0;
    ps[j] = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
    memset(ps[j], 0, sites_on_node * sizeof(su3_vector));
  }
  iters = ks_multicg_offset_field_cpu(s, ps, ksp, num_offsets, qic, ref_fn(inaik));
  for (j = 0; j < num_offsets; j++) {
    memcpy(psim + (size_t)j * sites_on_node * 6, ps[j], sites_on_node * sizeof(su3_vector));
    if (final_rsq) final_rsq[j] = qic[j].final_rsq;
    free(ps[j]);
  }
  free(ps); free(s); free(ksp); free(qic);
  return iters;
}

/* Fermion force (HISQ: fermion_force_hisq_multi.c; asqtad:
   fermion_force_multi.c -> fermion_force_fn_multi.c).  xxx holds nterms
   vectors (X on even sites, D_oe X on odd sites, as update_h_rhmc.c:82-87
   prepares them); mom is read and updated in place.  For HISQ
   n_orders_naik[] gives the number of terms per Naik epsilon group (first
   group includes every term with eps=0); asqtad ignores it. */
void ref_fermion_force(double eps, const double *residues, const double *xxx,
                       int nterms, const int *orders_naik, double *mom) {
  int j;
  size_t i;
  Real *res = (Real *)malloc(nterms * sizeof(Real));
  su3_vector **xv = (su3_vector **)malloc(nterms * sizeof(su3_vector *));
#if FERM_ACTION == HISQ
  n_order_naik_total = 0;
  for (j = 0; j < ref_n_naiks; j++) {
    n_orders_naik[j] = orders_naik ? orders_naik[j] : (j == 0 ? nterms : 0);
    n_order_naik_total += n_orders_naik[j];
  }
#else
  (void)orders_naik;
#endif
  for (j = 0; j < nterms; j++) {
    res[j] = residues[j];
    xv[j] = (su3_vector *)malloc(sites_on_node * sizeof(su3_vector));
    memcpy(xv[j], xxx + (size_t)j * sites_on_node * 6, sites_on_node * sizeof(su3_vector));
  }
  for (i = 0; i < sites_on_node; i++)
    memcpy(&lattice[i].mom[0], mom + i * 40, 4 * sizeof(anti_hermitmat));
  eo_fermion_force_multi(eps, res, xv, nterms, 2, fn_links);
  for (i = 0; i < sites_on_node; i++)
    memcpy(mom + i * 40, &lattice[i].mom[0], 4 * sizeof(anti_hermitmat));
  for (j = 0; j < nterms; j++) free(xv[j]);
  free(xv); free(res);
}

int ref_sizeof_anti_hermitmat(void) { return (int)sizeof(anti_hermitmat); }

/* ---------------- gauge side of the RHMC ----------------
 * MILC's own routines, called as ks_imp_rhmc's update() calls them:
 *   make_loop_table / imp_gauge_action   generic/gauge_stuff.c:87,277
 *   imp_gauge_force_ks                   generic_ks/gauge_force_imp_ks.c:8
 *   update_u                             ks_imp_rhmc/update_u.c:49
 *   hmom_action                          ks_imp_rhmc/d_action_rhmc.c:89
 *   ranmom / site generators             generic/ranmom.c, generic/ranstuff.c:117
 *   reunitarize_ks                       generic_ks/reunitarize_ks.c:9
 *   d_plaquette                          generic/d_plaq4.c
 * Links pass through ref_set_thin_links / ref_get_thin_links_phased;
 * momenta are anti_hermitmat[4*i+dir]. */
static int ref_loops_made = 0;

void ref_set_gauge_params(double b, double u0v, int nmasses, const int *flavors) {
  int i;
  beta = b;
  u0 = u0v;
  n_dyn_masses = nmasses;
  for (i = 0; i < nmasses; i++) dyn_flavors[i] = flavors[i];
  if (!ref_loops_made) { make_loop_table(); ref_loops_made = 1; }
}

static void ref_put_mom(const double *mom) {
  size_t i;
  for (i = 0; i < sites_on_node; i++) memcpy(&lattice[i].mom[0], mom + i * 40, 4 * sizeof(anti_hermitmat));
}
static void ref_take_mom(double *mom) {
  size_t i;
  for (i = 0; i < sites_on_node; i++) memcpy(mom + i * 40, &lattice[i].mom[0], 4 * sizeof(anti_hermitmat));
}

double ref_gauge_action(void) {
  double g;
  rephase(OFF);
  g = (beta / 3.0) * imp_gauge_action();
  rephase(ON);
  return g;
}

void ref_gauge_force(double eps, double *mom) {
  ref_put_mom(mom);
  imp_gauge_force_ks(eps, F_OFFSET(mom));
  ref_take_mom(mom);
}

void ref_update_u(double eps, const double *mom) {
  ref_put_mom(mom);
  update_u(eps);
}

double ref_hmom_action(const double *mom) {
  ref_put_mom(mom);
  return hmom_action();
}

void ref_seed(int seed) {
  iseed = seed;
  initialize_site_prn_from_seed(seed);
}

void ref_ranmom(double *mom) {
  ranmom();
  ref_take_mom(mom);
}

/* three complex Gaussians per site of `parity`, as grsource_rhmc.c:31-41 */
void ref_gaussian_vector(int parity, double *v) {
  int i, j;
  site *s;
  FORSOMEPARITY(i, s, parity) {
    for (j = 0; j < 3; j++) {
      complex z = complex_gaussian_rand_no(&(s->site_prn));
      v[6 * i + 2 * j] = z.real;
      v[6 * i + 2 * j + 1] = z.imag;
    }
  }
}

void ref_reunitarize(void) { reunitarize_ks(); }

void ref_plaquette(double *ss, double *st) { d_plaquette(ss, st); }
