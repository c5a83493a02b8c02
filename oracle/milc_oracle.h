/* milc_oracle.h -- CPU restatement of MILC's improved-staggered hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA path is compared
 * against (tests, the smoke check and the CPU-baseline leg of the
 * benchmark); the product library never links or calls it.
 *
 * Every function restates the reference function named beside it, in
 * plain C99 + OpenMP, FP64, on MILC's field layouts (su3_vector[V],
 * su3_matrix[4*i+dir], anti_hermitmat[4*i+dir], even sites first).  The
 * restatement is pinned against MILC itself (oracle/_ref, built from the
 * reference sources by oracle/ref/Makefile) and against the committed
 * fixtures in tests/golden/.
 */
#ifndef MILC_ORACLE_H
#define MILC_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#define ORC_ODD 0x01
#define ORC_EVEN 0x02
#define ORC_EVENANDODD 0x03

typedef struct {
  int dims[4];
  size_t V, Vh;
  int *coord;      /* [V][4] */
  size_t *nb;      /* [V][16]: MILC directions XUP..XDOWN then X3UP..X3DOWN */
} orc_lat;

/* path coefficients in MILC's asqtad-style naming (ks_action_paths_hisq.c:123-205) */
typedef struct {
  double one_link, naik, three_staple, five_staple, seven_staple, lepage;
} orc_coeffs;

orc_lat *orc_lat_create(int nx, int ny, int nz, int nt);
void orc_lat_free(orc_lat *L);
size_t orc_index(const orc_lat *L, const int c[4]);
void orc_rephase(const orc_lat *L, double *links);

void orc_dslash(const orc_lat *L, const double *fat, const double *lng,
                const double *src, double *dst, int parity);
/* nsrc independent solves in lockstep (one multi-field D per round); each
   source's result, iteration count and out7[7*s..] equal orc_congrad's */
int orc_congrad_multi(const orc_lat *L, const double *fat, const double *lng, int nsrc,
                      const double *const *srcs, double *const *dests, double mass, int parity,
                      double resid, double relresid, int niter, int max_restarts, double *out7);
int orc_congrad(const orc_lat *L, const double *fat, const double *lng,
                const double *src, double *dst, double mass, int parity,
                double resid, double relresid, int max, int nrestart, double out[7]);
int orc_mat_invert_uml(const orc_lat *L, const double *fat, const double *lng,
                       const double *src, double *dst, double mass, double resid,
                       int max, int nrestart, double out[7]);
int orc_multicg_offset(const orc_lat *L, const double *fat, const double *lng,
                       const double *src, double *psim, const double *offsets,
                       int num_offsets, int parity, double resid, int max, int nrestart,
                       double *final_rsq);

void orc_load_fatlinks(const orc_lat *L, const double *links, const orc_coeffs *c, double *fat);
void orc_load_lnglinks(const orc_lat *L, const double *links, const orc_coeffs *c, double *lng);
int orc_u3_unitarize(const double *V, double *W);
void orc_asqtad_coeffs(double u0, orc_coeffs *c);
void orc_asqtad_links(const orc_lat *L, const double *U, double u0, double *fat, double *lng);
int orc_hisq_links(const orc_lat *L, const double *U, int n_naiks, const double *eps_naik,
                   double *Vl, double *W, double *fat, double *lng);

/* asqtad force, generic_ks/fermion_force_fn_multi.c:80-316 (FNMAT):
   mom <- TA(mom + 2 eps U K_U) through the asqtad fat + Naik links of U */
void orc_fermion_force_asqtad(const orc_lat *L, const double *U, double u0, double eps,
                              const double *residues, const double *xxx, int nterms, double *mom);
void orc_fermion_force_hisq(const orc_lat *L, const double *U, int n_naiks,
                            const double *eps_naik, double eps, const double *residues,
                            const double *xxx, int nterms, const int *n_orders_naik,
                            double *mom);
/* S = sum_j res_j <X_j| (M^dag M + sigma_j)^-1 ... helper: the bilinear
   sum_j res_j Re <xxx_j| D |xxx_j>-type action used by finite-difference
   checks; see the definition in milc_oracle_force.c */
double orc_force_action(const orc_lat *L, const double *U, int n_naiks, const double *eps_naik,
                        const double *residues, const double *xxx, int nterms,
                        const int *n_orders_naik);

/* ---- gauge side of the RHMC (milc_oracle_gauge.c) ---- */
#define ORC_MAX_LOOPS 16     /* orientations per loop kind (gauge_stuff.c MAX_NUM) */
#define ORC_MAX_STAPLES 64   /* staple paths per link direction */
typedef struct {
  int nloop;
  int length[3];
  int num[3];
  int dirs[3][ORC_MAX_LOOPS][6];
  double coeff[3];
} orc_loops;

typedef struct {
  uint32_t r[7];
  uint64_t multiplier, addend, ic_state;
} orc_prn;

void orc_loop_table(int nflavors, double u0, orc_loops *T);
double orc_gauge_action(const orc_lat *L, const double *U, double beta, double u0, int nflavors);
void orc_gauge_force(const orc_lat *L, const double *U, double eps, double beta, double u0, int nflavors,
                     double *mom);
void orc_update_u(const orc_lat *L, double *U, const double *mom, double eps);
double orc_hmom_action(const orc_lat *L, const double *mom);
void orc_reunitarize(const orc_lat *L, double *U);
void orc_plaquette(const orc_lat *L, const double *U, double *ss, double *st);
void orc_prn_init(orc_prn *p, int seed, int index);
double orc_myrand(orc_prn *p);
double orc_gaussian(orc_prn *p);
void orc_complex_gaussian(orc_prn *p, double *re, double *im);
void orc_site_prn_init(const orc_lat *L, int seed, orc_prn *prn);
void orc_ranmom(const orc_lat *L, orc_prn *prn, double *mom);
void orc_gaussian_vector(const orc_lat *L, orc_prn *prn, int parity, double *v);

#endif
