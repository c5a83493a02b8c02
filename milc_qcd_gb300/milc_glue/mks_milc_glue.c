/* mks_milc_glue.c -- MILC-side binding of libmilc_ks_gb300.so.
 *
 * Compiled inside a MILC build (it includes MILC's headers) in place of the
 * QUDA shims, it defines the `_gpu` functions that MILC's compile-time
 * macro swap selects (include/imp_ferm_links.h:73-101,211-246,
 * include/fermion_links_milc.h:107-126) plus the HISQ force entry, and
 * forwards each to the C ABI of include/milc_ks_gb300.h:
 *
 *   ks_congrad_parity_gpu        -> mks_ks_congrad_parity
 *   ks_congrad_block_parity_gpu  -> mks_ks_congrad_block_parity
 *   ks_multicg_offset_field_gpu  -> mks_ks_multicg_offset_field
 *   load_fatlinks_gpu            -> mks_fatlong_links (fat only)
 *   load_fatlonglinks_gpu        -> mks_fatlong_links
 *   load_hisq_aux_links_gpu      -> mks_hisq_aux_links
 *   eo_fermion_force_multi       -> mks_fermion_force_multi_hisq
 *   eo_fermion_force_oneterm / _twoterms (the same, one or two terms)
 *
 * Fields are passed straight through: with MILC_PRECISION=2 an su3_vector
 * array is double[V][6] and an su3_matrix array double[V][4][18] in MILC's
 * site order, which is the ABI's layout.  Fermion links are cached on the
 * device per fn_links_t pointer (the role of QUDA's fn_last cache,
 * generic_ks/ks_multicg_offset_gpu.c:27-35) and re-uploaded when MILC
 * raises notify_quda_new_links (fresh_fn_links, include/fn_links.h:15).
 *
 * Inner precision: qic->prec = 2 gives the plain FP64 CG; qic->prec = 1
 * the FP32 inner solve with FP64 reliable updates; the environment
 * variable MKS_HALF=1 turns qic->prec = 1 into the FP16 inner solve.
 */
#include "generic_ks_includes.h"
#include "../include/fermion_links.h"
#include "../include/fermion_links_milc.h"
#include "../include/fn_links.h"
#include "milc_ks_gb300.h"
#include <stdlib.h>
#include <string.h>

#if MILC_PRECISION != 2
#error "mks_milc_glue.c passes MILC fields through unchanged: build MILC with PRECISION=2"
#endif

static int mks_ready = 0;
static imp_ferm_links_t *mks_slot_fn[MKS_MAX_SLOTS];
static int mks_next_slot = 0;

static void mks_die(const char *who, int st) {
  node0_printf("%s: %s\n", who, mks_error_string(st));
  terminate(1);
}

static void mks_setup(void) {
  int dims[4], st;
  if (mks_ready) return;
  if (numnodes() != 1) {
    node0_printf("mks_milc_glue: one process per GPU, whole lattice per process\n");
    terminate(1);
  }
  dims[0] = nx; dims[1] = ny; dims[2] = nz; dims[3] = nt;
  if ((st = mks_init(0)) < 0) mks_die("mks_init", st);
  if ((st = mks_set_lattice(dims)) < 0) mks_die("mks_set_lattice", st);
  mks_ready = 1;
}

/* device slot holding fn's links, uploading them when new or refreshed */
static int mks_slot_for(imp_ferm_links_t *fn) {
  int s, st;
  for (s = 0; s < MKS_MAX_SLOTS; s++)
    if (mks_slot_fn[s] == fn && !fresh_fn_links(fn)) return s;
  for (s = 0; s < MKS_MAX_SLOTS; s++)
    if (mks_slot_fn[s] == fn) break;
  if (s == MKS_MAX_SLOTS) {
    s = mks_next_slot;
    mks_next_slot = (mks_next_slot + 1) % MKS_MAX_SLOTS;
  }
  st = mks_load_fn_links(s, (const double *)get_fatlinks(fn), (const double *)get_lnglinks(fn), fn->eps_naik);
  if (st < 0) mks_die("mks_load_fn_links", st);
  mks_slot_fn[s] = fn;
  cancel_quda_notification(fn);
  return s;
}

static void mks_fill_arg(mks_invert_arg *a, const quark_invert_control *qic) {
  const char *h = getenv("MKS_HALF");
  a->max = qic->max;
  a->nrestart = qic->nrestart;
  a->parity = qic->parity;
  a->prec = qic->prec == 2 ? MKS_PREC_DOUBLE : ((h && atoi(h)) ? MKS_PREC_HALF : MKS_PREC_SINGLE);
  a->resid = qic->resid;
  a->relresid = qic->relresid;
  a->delta = 0.1;
}

static void mks_take(quark_invert_control *qic, const mks_invert_result *r) {
  qic->final_rsq = r->final_rsq;
  qic->final_relrsq = r->final_relrsq;
  qic->size_r = r->size_r;
  qic->size_relr = r->size_relr;
  qic->final_iters = r->final_iters;
  qic->final_restart = r->final_restart;
  qic->converged = r->converged;
}

/* include/imp_ferm_links.h:95-97 */
int ks_congrad_parity_gpu(su3_vector *src, su3_vector *dest, quark_invert_control *qic, Real mass,
                          imp_ferm_links_t *fn) {
  mks_invert_arg a;
  mks_invert_result r;
  int it;
  mks_setup();
  mks_fill_arg(&a, qic);
  it = mks_ks_congrad_parity((const double *)src, (double *)dest, mass, mks_slot_for(fn), &a, &r);
  if (it < 0) mks_die("ks_congrad_parity_gpu", it);
  mks_take(qic, &r);
  return it;
}

/* include/imp_ferm_links.h:99-101 */
int ks_congrad_block_parity_gpu(int nsrc, su3_vector **src, su3_vector **dest, quark_invert_control *qic,
                                Real mass, imp_ferm_links_t *fn) {
  mks_invert_arg a;
  mks_invert_result *r = (mks_invert_result *)malloc(nsrc * sizeof(mks_invert_result));
  int it, k;
  mks_setup();
  mks_fill_arg(&a, qic);
  it = mks_ks_congrad_block_parity(nsrc, (const double *const *)src, (double *const *)dest, mass,
                                   mks_slot_for(fn), &a, r);
  if (it < 0) mks_die("ks_congrad_block_parity_gpu", it);
  mks_take(qic, &r[0]);
  for (k = 1; k < nsrc; k++)
    if (r[k].final_rsq > qic->final_rsq) mks_take(qic, &r[k]);
  free(r);
  return it;
}

/* include/imp_ferm_links.h:211-218 */
int ks_multicg_offset_field_gpu(su3_vector *src, su3_vector **psim, ks_param *ksp, int num_offsets,
                                quark_invert_control qic[], imp_ferm_links_t *fn) {
  mks_invert_arg a;
  mks_invert_result *r;
  double *off;
  int it, j;
  if (num_offsets == 0) return 0;
  mks_setup();
  r = (mks_invert_result *)malloc(num_offsets * sizeof(mks_invert_result));
  off = (double *)malloc(num_offsets * sizeof(double));
  for (j = 0; j < num_offsets; j++) off[j] = ksp[j].offset;
  mks_fill_arg(&a, &qic[0]);
  it = mks_ks_multicg_offset_field((const double *)src, (double *const *)psim, off, num_offsets,
                                   mks_slot_for(fn), &a, r);
  if (it < 0) mks_die("ks_multicg_offset_field_gpu", it);
  for (j = 0; j < num_offsets; j++) mks_take(&qic[j], &r[j]);
  free(r);
  free(off);
  return it;
}

static void mks_coeffs(const ks_component_paths *p, double c[6]) {
  c[0] = p->act_path_coeff.one_link;
  c[1] = p->act_path_coeff.naik;
  c[2] = p->act_path_coeff.three_staple;
  c[3] = p->act_path_coeff.five_staple;
  c[4] = p->act_path_coeff.seven_staple;
  c[5] = p->act_path_coeff.lepage;
}

/* include/fermion_links_milc.h:107-109 */
void load_fatlinks_gpu(info_t *info, su3_matrix *fat, ks_component_paths *p, su3_matrix *links) {
  double c[6];
  int st;
  mks_setup();
  mks_coeffs(p, c);
  if ((st = mks_fatlong_links(c, (const double *)links, (double *)fat, NULL)) < 0) mks_die("load_fatlinks_gpu", st);
  info->final_flop = 61632. * volume / numnodes();
}

/* include/fermion_links_milc.h:111-113 */
void load_fatlonglinks_gpu(info_t *info, su3_matrix *fatlinks, su3_matrix *longlinks, ks_component_paths *p,
                           su3_matrix *links) {
  double c[6];
  int st;
  mks_setup();
  mks_coeffs(p, c);
  if ((st = mks_fatlong_links(c, (const double *)links, (double *)fatlinks, (double *)longlinks)) < 0)
    mks_die("load_fatlonglinks_gpu", st);
  info->final_flop = (61632. + 1728.) * volume / numnodes();
}

/* include/fermion_links_milc.h:115-116 */
void load_hisq_aux_links_gpu(info_t *info, ks_action_paths_hisq *ap, hisq_auxiliary_t *aux, su3_matrix *links) {
  double c[6];
  int st;
  mks_setup();
  memcpy(aux->U_link, links, 4 * sizeof(su3_matrix) * sites_on_node);
  mks_coeffs(&ap->p1, c);
  if ((st = mks_hisq_aux_links(c, (const double *)links, (double *)aux->V_link, (double *)aux->W_unitlink)) < 0)
    mks_die("load_hisq_aux_links_gpu", st);
  info->final_flop = 61632. * volume / numnodes();
}

#if FERM_ACTION == HISQ
/* generic_ks/fermion_force_hisq_multi.c:170-219: mom[dir] += TA(+-2 eps U dS/dU) */
void eo_fermion_force_multi(Real eps, Real *residues, su3_vector **xxx, int nterms, int prec,
                            fermion_links_t *fl) {
  hisq_auxiliary_t *aux = get_hisq_auxiliary(fl);
  int n_naiks = fermion_links_get_n_naiks(fl);
  double *mom = (double *)malloc(sites_on_node * 4 * sizeof(anti_hermitmat));
  double *res = (double *)malloc(nterms * sizeof(double));
  int *orders = (int *)malloc((n_naiks > 0 ? n_naiks : 1) * sizeof(int));
  int i, g, st, tot = 0;
  site *s;
  (void)prec;
  mks_setup();
  for (g = 0; g < n_naiks; g++) { orders[g] = n_orders_naik[g]; tot += orders[g]; }
  if (tot != nterms) { orders[0] = nterms; for (g = 1; g < n_naiks; g++) orders[g] = 0; }
  for (i = 0; i < nterms; i++) res[i] = residues[i];
  FORALLSITES(i, s) { memcpy(mom + 40 * i, s->mom, 4 * sizeof(anti_hermitmat)); }
  if ((st = mks_load_hisq_aux((const double *)aux->U_link, (const double *)aux->V_link,
                              (const double *)aux->W_unitlink)) < 0)
    mks_die("eo_fermion_force_multi", st);
  st = mks_fermion_force_multi_hisq(eps, res, (const double *const *)xxx, nterms, orders, n_naiks, mom);
  if (st < 0) mks_die("eo_fermion_force_multi", st);
  FORALLSITES(i, s) { memcpy(s->mom, mom + 40 * i, 4 * sizeof(anti_hermitmat)); }
  free(mom); free(res); free(orders);
}
#else
/* asqtad: generic_ks/fermion_force_multi.c:29-44 (FNMAT,
   fermion_force_fn_multi.c:80-316); the links are rebuilt on the device from
   the thin links (phases in) with MILC's tadpole factor u0 */
void eo_fermion_force_multi(Real eps, Real *residues, su3_vector **xxx, int nterms, int prec,
                            fermion_links_t *fl) {
  double *mom = (double *)malloc(sites_on_node * 4 * sizeof(anti_hermitmat));
  double *thin = (double *)malloc(sites_on_node * 72 * sizeof(double));
  double *res = (double *)malloc(nterms * sizeof(double));
  double eps0 = 0.0;
  int i, dir, st;
  site *s;
  (void)prec; (void)fl;
  mks_setup();
  for (i = 0; i < nterms; i++) res[i] = residues[i];
  FORALLSITES(i, s) {
    memcpy(mom + 40 * i, s->mom, 4 * sizeof(anti_hermitmat));
    for (dir = XUP; dir <= TUP; dir++) memcpy(thin + (4 * i + dir) * 18, &s->link[dir], 18 * sizeof(double));
  }
  if ((st = mks_load_links_from_thin(MKS_ACTION_ASQTAD, thin, 1, &eps0, u0)) < 0)
    mks_die("eo_fermion_force_multi", st);
  st = mks_fermion_force_multi_asqtad(eps, res, (const double *const *)xxx, nterms, mom);
  if (st < 0) mks_die("eo_fermion_force_multi", st);
  FORALLSITES(i, s) { memcpy(s->mom, mom + 40 * i, 4 * sizeof(anti_hermitmat)); }
  free(mom); free(thin); free(res);
}
#endif

void eo_fermion_force_oneterm(Real eps, Real weight, su3_vector *temp_x, int prec, fermion_links_t *fl) {
  su3_vector *xxx[1] = {temp_x};
  Real residues[1] = {weight};
  eo_fermion_force_multi(eps, residues, xxx, 1, prec, fl);
}

void eo_fermion_force_twoterms(Real eps, Real weight1, Real weight2, su3_vector *x1_off, su3_vector *x2_off,
                               int prec, fermion_links_t *fl) {
  su3_vector *xxx[2] = {x1_off, x2_off};
  Real residues[2] = {weight1, weight2};
  eo_fermion_force_multi(eps, residues, xxx, 2, prec, fl);
}

/* Host allocators named by MILC's -DUSE_FL_GPU code paths (see
   mks_milc_alloc.h).  Plain malloc: the library copies from pageable memory
   correctly, pinning only changes the copy speed. */
#ifdef USE_GF_GPU
/* ---- gauge side of the molecular dynamics (-DUSE_GF_GPU) ----
 * Replaces imp_gauge_force_gpu (generic/gauge_force_imp_gpu.c:15),
 * reunitarize_gpu (generic/reunitarize2.c:210) and the QUDA variant of
 * update_u (ks_imp_rhmc/update_u.c:23-45; drop update_u.o, this file
 * defines update_u).  MILC keeps links and momenta in its site structure,
 * so each call uploads them (links without phases), runs the kernel and
 * copies back what changed; a trajectory that stays on the GPU from start
 * to end is mks_rhmc_trajectory. */
static double *mks_links_buf = NULL, *mks_mom_buf = NULL;

static void mks_put_links(void) {
  int i, dir, k, st;
  site *s;
  if (!mks_links_buf) mks_links_buf = (double *)malloc(sizeof(double) * 72 * sites_on_node);
  FORALLSITES(i, s) for (dir = XUP; dir <= TUP; dir++) {
    const double *m = (const double *)&s->link[dir];
    double ph = (phases_in == ON) ? s->phase[dir] : 1.0;   /* phases are +-1 */
    for (k = 0; k < 18; k++) mks_links_buf[(4 * i + dir) * 18 + k] = ph * m[k];
  }
  if ((st = mks_gauge_load(mks_links_buf)) < 0) mks_die("mks_gauge_load", st);
}

static void mks_take_links(void) {
  int i, dir, k, st;
  site *s;
  if ((st = mks_gauge_get(mks_links_buf)) < 0) mks_die("mks_gauge_get", st);
  FORALLSITES(i, s) for (dir = XUP; dir <= TUP; dir++) {
    double *m = (double *)&s->link[dir];
    double ph = (phases_in == ON) ? s->phase[dir] : 1.0;
    for (k = 0; k < 18; k++) m[k] = ph * mks_links_buf[(4 * i + dir) * 18 + k];
  }
}

static void mks_put_mom(field_offset mom_off) {
  int i, st;
  site *s;
  if (!mks_mom_buf) mks_mom_buf = (double *)malloc(sizeof(double) * 40 * sites_on_node);
  FORALLSITES(i, s) memcpy(mks_mom_buf + 40 * i, F_PT(s, mom_off), 4 * sizeof(anti_hermitmat));
  if ((st = mks_mom_load(mks_mom_buf)) < 0) mks_die("mks_mom_load", st);
}

static void mks_take_mom(field_offset mom_off) {
  int i, st;
  site *s;
  if ((st = mks_mom_get(mks_mom_buf)) < 0) mks_die("mks_mom_get", st);
  FORALLSITES(i, s) memcpy(F_PT(s, mom_off), mks_mom_buf + 40 * i, 4 * sizeof(anti_hermitmat));
}

static int mks_total_flavors(void) {
  int i, n = 0;
  for (i = 0; i < n_dyn_masses; i++) n += dyn_flavors[i];
  return n;
}

void imp_gauge_force_gpu(Real eps, field_offset mom_off) {
  int st;
  mks_setup();
  mks_put_links();
  mks_put_mom(mom_off);
  if ((st = mks_gauge_force(eps, beta, u0, mks_total_flavors())) < 0) mks_die("imp_gauge_force_gpu", st);
  mks_take_mom(mom_off);
}

void update_u(Real eps) {
  int st;
#ifdef FN
  invalidate_fermion_links(fn_links);
#endif
  mks_setup();
  mks_put_links();
  mks_put_mom(F_OFFSET(mom));
  if ((st = mks_update_u(eps)) < 0) mks_die("update_u", st);
  mks_take_links();
}

void reunitarize_gpu(void) {
  int st;
  mks_setup();
  mks_put_links();
  if ((st = mks_reunitarize()) < 0) mks_die("reunitarize_gpu", st);
  mks_take_links();
}
#endif /* USE_GF_GPU */

void *qudaAllocatePinned(size_t bytes) { return malloc(bytes); }
void qudaFreePinned(void *ptr) { free(ptr); }

/* The site links as one su3_matrix[4*sites_on_node] array: what
 * fermion_links_from_site.c:14-58 asks for under -DUSE_FL_GPU (the QUDA
 * build takes it from include/generic_quda.h, which needs QUDA). */
void *create_G_from_site_quda(void) {
  int i;
  site *s;
  su3_matrix *links = (su3_matrix *)qudaAllocatePinned((size_t)sites_on_node * 4 * sizeof(su3_matrix));
  if (!links) mks_die("create_G_from_site_quda", MKS_ERR_NOMEM);
  FORALLSITES(i, s) { memcpy(links + 4 * i, s->link, 4 * sizeof(su3_matrix)); }
  return links;
}
void destroy_G_quda(void *links) { qudaFreePinned(links); }

/* The option string MILC prints at start-up (show_generic_ks_md_opts.c:12);
 * its definition lives in fermion_force_hisq_multi.c, which this binding
 * replaces (generic_ks/fermion_force_hisq_multi.c:277-293). */
const char *ks_multiff_opt_chr(void) {
  switch (KS_MULTIFF) {
  case ASVEC: return "ASVEC";
  case FNMATREV: return "FNMATREV";
  default: return "FNMAT";
  }
}
