/* milc_ks_gb300.h -- C ABI of the GB300-native improved-staggered hot path.
 *
 * One process drives one GPU.  Every entry point returns an int status
 * (MKS_OK = 0, negative on error; mks_error_string() describes it) unless
 * it is documented otherwise.  Arrays are plain C arrays in MILC's own
 * memory layout for MILC_PRECISION=2, so a MILC build can pass its fields
 * through unchanged:
 *
 *   colour vector field   double[V][6]       su3_vector[i]      (3 complex)
 *   link field            double[V][4][18]   su3_matrix[4*i+dir] (3x3 complex, row major)
 *   momentum field        double[V][4][10]   anti_hermitmat mom[dir] (m01,m02,m12,
 *                                              m00im,m11im,m22im,space)
 *
 * where i is MILC's single-node site index: lexicographic
 * x + nx*(y + ny*(z + nz*t)), even sites first (generic/layout_hyper_prime.c:
 * 509-520).  Link fields carry the staggered phases and the antiperiodic
 * time boundary folded in (generic_ks/rephase.c:99-117), as MILC's fermion
 * links do.
 *
 * Operator conventions are MILC's (generic_ks/dslash_fn.c:365-576,
 * generic_ks/mat_invert.c:18-44): D is anti-Hermitian without a factor 1/2,
 *   (D s)(x) = sum_mu F_mu(x) s(x+mu) - F_mu(x-mu)^dag s(x-mu)
 *            +       L_mu(x) s(x+3mu) - L_mu(x-3mu)^dag s(x-3mu),
 * M = 2m + D, and the parity solves work with M^dag M = 4m^2 - D_eo D_oe.
 *
 * Host arrays stay owned by the caller; the library never frees them.
 * Functions named *_dev take device pointers with the same layout and do
 * no host<->device copies of field data.
 */
#ifndef MILC_KS_GB300_H
#define MILC_KS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define MKS_OK              0
#define MKS_ERR_ARG        -1   /* bad argument (size, parity, null pointer) */
#define MKS_ERR_CUDA       -2   /* a CUDA runtime call failed */
#define MKS_ERR_NOMEM      -3   /* device allocation failed */
#define MKS_ERR_STATE      -4   /* library not initialised / lattice or links not loaded */
#define MKS_ERR_TIMEOUT    -5   /* a bounded device-side wait gave up */
#define MKS_ERR_NUMERIC    -6   /* NaN/Inf met in a solver recurrence */
#define MKS_ERR_UNSUPPORTED -7  /* option not provided by the library */

/* ---- parities: same values as MILC include/macros.h:17-19 ---- */
#define MKS_ODD        0x01
#define MKS_EVEN       0x02
#define MKS_EVENANDODD 0x03

/* ---- arithmetic precisions of the inner (sloppy) solve ----
   MILC's qic->prec uses 1 = single, 2 = double (include/generic_quark_types.h:168) */
#define MKS_PREC_HALF   0
#define MKS_PREC_SINGLE 1
#define MKS_PREC_DOUBLE 2

/* Solver controls: the fields of MILC's quark_invert_control
   (include/generic_quark_types.h:167-190) that the hot path reads. */
typedef struct {
  int    max;        /* iterations per restart (qic->max) */
  int    nrestart;   /* maximum restarts (qic->nrestart); cap = max*nrestart */
  int    parity;     /* MKS_EVEN, MKS_ODD (MKS_EVENANDODD where noted) */
  int    prec;       /* inner precision: MKS_PREC_DOUBLE (plain FP64 CG),
                        MKS_PREC_SINGLE or MKS_PREC_HALF (FP64 reliable updates) */
  double resid;      /* target |r|/|b|, NOT squared (qic->resid) */
  double relresid;   /* target Fermilab relative residual, 0 = unused (qic->relresid) */
  double delta;      /* reliable-update trigger for mixed precision (0 -> 0.1) */
} mks_invert_arg;

/* Solver results: the fields MILC fills on return
   (generic_ks/d_congrad5_fn_milc.c:370-395). */
typedef struct {
  double final_rsq;      /* true |r|^2/|b|^2 (squared, normalised) */
  double final_relrsq;   /* relative residual, squared */
  double size_r;         /* iterated residual, same normalisation */
  double size_relr;
  int    final_iters;
  int    final_restart;
  int    converged;      /* 1 converged, 0 not */
  int    reliable_updates; /* FP64 true-residual recomputations (mixed precision) */
} mks_invert_result;

/* ------------------------------------------------------------------ */
/* Library lifetime.  Replaces the QUDA set-up MILC performs in
   initialize_quda() (generic/milc_to_quda_utilities.c:11-41). */
int mks_init(int device);
int mks_finalize(void);
const char *mks_error_string(int status);
/* Lattice extents (all even and at least 4: the Naik term reaches 3 sites).
 * Frees every cached field of another size. */
int mks_set_lattice(const int dims[4]);

/* ------------------------------------------------------------------ */
/* Fermion links.
 * Replaces load_fatlinks_gpu / load_fatlonglinks_gpu
 * (generic_ks/fermion_links_fn_load_gpu.c:19,49) and the QUDA link cache
 * keyed on fn_links_t (include/fn_links.h:9-17, fresh_fn_links /
 * cancel_quda_notification, generic_ks/d_congrad5_fn_gpu.c:121-126):
 * fat and long links of one Naik-epsilon group are uploaded once into
 * slot `slot` (0 .. MKS_MAX_SLOTS-1) and stay resident until reloaded or
 * invalidated.  eps_naik is stored with the slot (fn->eps_naik). */
#define MKS_MAX_SLOTS 12
int mks_load_fn_links(int slot, const double *fat, const double *lng, double eps_naik);
int mks_load_fn_links_dev(int slot, const double *fat_dev, const double *lng_dev, double eps_naik);
int mks_invalidate_fn_links(int slot);
int mks_get_fn_links(int slot, double *fat, double *lng);

/* ------------------------------------------------------------------ */
/* D_eo / D_oe.  Replaces dslash_fn_field (generic_ks/dslash_fn.c:302-358,
 * generic_ks/dslash_fn_dblstore.c:285): dst on `parity` sites receives
 * D src, src read on the other parity.  parity may be MKS_EVENANDODD. */
int mks_dslash_fn_field(const double *src, double *dst, int parity, int slot);
int mks_dslash_fn_field_dev(const double *src_dev, double *dst_dev, int parity, int slot);
/* The same D_eo for callers that cannot allocate device memory (no
 * counterpart in the reference; MILC's own paths allocate freely).
 * mks_dslash_fn_field_dev allocates its staging buffers with cudaMalloc on
 * first use; an application that gives nearly all device memory to its own
 * pool allocator, or code that must not run a device-wide synchronising
 * call such as cudaMalloc at that moment, calls this variant instead.  It
 * allocates nothing: its staging lives in a fixed 32 MiB device array that
 * every GPU loading the library keeps until exit, which limits it to
 * lattices of at most 349,525 sites (MKS_ERR_ARG beyond).  All calls share
 * that array; calls that overlap on the GPU race on it.  mks_init looks up
 * the array's device address (cudaGetSymbolAddress, with the library's
 * device current) and loads the kernels this entry point launches, so the
 * array is resident from mks_init on and no call of this entry point loads
 * code or takes device memory; call mks_init before handing the device
 * memory to a pool.  Links must already be loaded in `slot`. */
int mks_dslash_fn_field_dev_noalloc(const double *src_dev, double *dst_dev, int parity, int slot);

/* ------------------------------------------------------------------ */
/* Single-source CG on (4m^2 - D_eo D_oe) for one parity.
 * Replaces ks_congrad_parity_gpu (include/imp_ferm_links.h:95-97,
 * generic_ks/d_congrad5_fn_gpu.c:35-165; CPU semantics
 * generic_ks/d_congrad5_fn_milc.c:61-407).  dst holds the initial guess on
 * entry and the solution on return; sites of the other parity are not
 * touched.  A zero source gives a zero solution and 0 iterations.
 * Returns the number of iterations (>= 0) or a negative status. */
int mks_ks_congrad_parity(const double *src, double *dst, double mass, int slot,
                          const mks_invert_arg *arg, mks_invert_result *res);
int mks_ks_congrad_parity_dev(const double *src_dev, double *dst_dev, double mass, int slot,
                              const mks_invert_arg *arg, mks_invert_result *res);

/* Multi-source CG: nsrc right-hand sides solved together, every link read
 * once per operator application for all sources.  Replaces
 * ks_congrad_block_parity_gpu (include/imp_ferm_links.h:99-101,
 * generic_ks/d_congrad5_fn_gpu.c:167-305).  res has nsrc entries.
 * Host arrays that are page-locked and mapped (cudaHostAlloc,
 * cudaHostRegister) are read and written in place by the solver's kernels;
 * pageable arrays are staged through device copies.  Either way only the
 * solved parity's half of each array moves.
 * Returns the largest iteration count or a negative status. */
int mks_ks_congrad_block_parity(int nsrc, const double *const *src, double *const *dst,
                                double mass, int slot, const mks_invert_arg *arg,
                                mks_invert_result *res);
int mks_ks_congrad_block_parity_dev(int nsrc, const double *const *src_dev, double *const *dst_dev,
                                    double mass, int slot, const mks_invert_arg *arg,
                                    mks_invert_result *res);

/* M^{-1} on both parities: precondition with M^dag, even CG, odd
 * reconstruction, odd polish (generic_ks/mat_invert.c:328-407).  dst
 * holds the initial guess.  arg->parity is ignored. */
int mks_mat_invert_uml_field(const double *src, double *dst, double mass, int slot,
                             const mks_invert_arg *arg, mks_invert_result *res);
/* Same for nsrc sources (generic_ks/mat_invert.c:409-483); res[nsrc]. */
int mks_mat_invert_block_uml(int nsrc, const double *const *src, double *const *dst,
                             double mass, int slot, const mks_invert_arg *arg,
                             mks_invert_result *res);

/* Multi-shift CG: psim[j] = (sigma_j - D_eo D_oe)^{-1} src on arg->parity
 * for offsets sigma_j > 0 (MILC's ksp[j].offset, sigma = 4 m^2 for a
 * plain mass).  Replaces ks_multicg_offset_field_gpu
 * (include/imp_ferm_links.h:211-218, generic_ks/ks_multicg_offset_gpu.c:
 * 38-250; CPU semantics generic_ks/ks_multicg_offset.c:63-505).  Stops
 * when the smallest shift meets arg->resid, like the CPU code (:381).
 * psim is overwritten on arg->parity (zero initial guess); its other sites
 * are not touched.  res has num_offsets entries.  Page-locked, mapped
 * arrays are read and written in place by the solver's kernels; pageable
 * ones are staged through device copies.
 * arg->prec selects FP64, or FP32/FP16 shifted updates with FP64 reliable
 * updates of the lowest shift (every shift's solution accumulated in FP64;
 * for arg->resid below 1e-7 the shifts' search directions and solutions
 * are FP64 vectors), an FP64 true-residual check of every shift, and a
 * mixed-precision refinement of the shifts that miss arg->resid
 * (generic_ks/ks_multicg.c:170-228; its inner solve is FP32 when arg->prec
 * is FP16). */
int mks_ks_multicg_offset_field(const double *src, double *const *psim,
                                const double *offsets, int num_offsets, int slot,
                                const mks_invert_arg *arg, mks_invert_result *res);
int mks_ks_multicg_offset_field_dev(const double *src_dev, double *const *psim_dev,
                                    const double *offsets, int num_offsets, int slot,
                                    const mks_invert_arg *arg, mks_invert_result *res);
/* Multi-shift CG for nf <= 4 fields (pseudofermion sources) on the same
 * links, each with its own offsets: the same result as one
 * mks_ks_multicg_offset_field_dev call per field (MILC calls
 * ks_multicg_offset_field once per field, ks_imp_rhmc/ks_ratinv.c:108),
 * with the fields' iterations batched: in FP32 (arg->prec MKS_PREC_SINGLE)
 * one multi-source D_eo pair per iteration reads the links once for every
 * running field.  offsets, psim_dev and res hold the fields' lists one after
 * the other (num_offsets[f] entries each); device pointers.  Other
 * precisions solve field by field.  Returns the largest iteration count. */
int mks_ks_multicg_offset_multi_dev(int nf, const double *const *src_dev, const int *num_offsets,
                                    const double *offsets, double *const *psim_dev, int slot,
                                    const mks_invert_arg *arg, mks_invert_result *res);

/* ------------------------------------------------------------------ */
/* HISQ link construction.  Replaces load_hisq_aux_links_gpu and the fat /
 * long smearing of load_hisq_fn_links (generic_ks/fermion_links_fn_load_gpu.c:
 * 80-110, generic_ks/fermion_links_hisq_load_milc.c:547-640): from thin
 * links U (phases in) build V = fat7(U), W = U(3) projection of V
 * (analytic, generic_ks/su3_mat_op.c:828), and for each Naik group i the fat
 * and long links X_i = asqtad+2xLepage(W) + eps_i (1-link + Naik)(W),
 * stored in slots 0..n_naiks-1.  The aux links stay resident for the force.
 * action: MKS_ACTION_HISQ; MKS_ACTION_ASQTAD builds asqtad fat/long links
 * directly from U into slot 0 (tadpole factor u0). */
#define MKS_ACTION_HISQ   1
#define MKS_ACTION_ASQTAD 2
int mks_load_links_from_thin(int action, const double *thin, int n_naiks,
                             const double *eps_naik, double u0);
int mks_get_hisq_aux(double *V, double *W);
/* Number of links in the last HISQ construction for which MILC's
   HISQ_REUNIT_ALLOW_SVD criteria (relative 1e-8 / absolute 1e-8 on det V^dag V,
   generic_ks/su3_mat_op.c:1037-1080) would have switched to its SVD branch;
   the analytic projection was used for them.  Returns a count >= 0; 0 after
   a construction in the FP32 molecular-dynamics precision, where the test
   is below the arithmetic's resolution and is not made. */
int mks_hisq_reunit_svd_count(void);
/* Rebuild the fat/long links of slots 0..n_naiks-1 from the thin links
 * already resident on the device (after mks_update_u / mks_reunitarize or
 * mks_gauge_load): restore_fermion_links_from_site after
 * invalidate_fermion_links (generic_ks/fermion_links_hisq_milc.c,
 * ks_imp_rhmc/update_u.c:66).  Same arguments as mks_load_links_from_thin. */
int mks_rebuild_links(int action, int n_naiks, const double *eps_naik, double u0);

/* Generic-coefficient loaders, one per MILC GPU loader:
 * coeffs = {one_link, naik, three_staple, five_staple, seven_staple, lepage}
 * as in MILC's asqtad_coeffs_t (include/ks_action_paths.h:23-30).
 *  - mks_fatlong_links replaces load_fatlinks_gpu / load_fatlonglinks_gpu
 *    (generic_ks/fermion_links_fn_load_gpu.c:19-78): fat (and, when lng is
 *    not NULL, long) links of `links` by the optimised staple recursion
 *    (fermion_links_fn_load_milc.c:207-253) and the Naik path.
 *  - mks_hisq_aux_links replaces load_hisq_aux_links_gpu (:80-110): V =
 *    fat(U; coeffs1), W = U(3) projection of V; U, V, W stay resident for
 *    the force and are copied back when V / W are not NULL.
 *  - mks_load_hisq_aux uploads U, V, W built elsewhere for the force. */
int mks_fatlong_links(const double coeffs[6], const double *links, double *fat, double *lng);
int mks_hisq_aux_links(const double coeffs1[6], const double *U, double *V, double *W);
int mks_load_hisq_aux(const double *U, const double *V, const double *W);

/* ------------------------------------------------------------------ */
/* HISQ fermion force.  Replaces eo_fermion_force_multi with the GPU
 * wrapper fn_fermion_force_multi_hisq_wrapper_mx_gpu
 * (generic_ks/fermion_force_hisq_multi.c:155-219,2168-2290; CPU semantics
 * :1182-1475): mom[dir](x) += TA( +-2 eps U_mu(x) dS/dU_mu(x) ) for the
 * rational-function terms sum_j residues[j] |xxx_j><xxx_j| with xxx_j = X_j
 * on even sites and D_oe X_j on odd sites.  n_orders_naik[g] gives how many
 * consecutive terms belong to Naik group g (MILC's n_orders_naik[],
 * ks_imp_rhmc/setup.c:295-339; the counts add up to nterms): every term
 * goes through the level-2 smearing, and the terms of group g >= 1 also
 * through eps_naik[g] (1-link + Naik) of that group's links.  Uses the aux
 * links U, V, W of the last mks_load_links_from_thin (HISQ action). */
int mks_fermion_force_multi_hisq(double eps, const double *residues,
                                 const double *const *xxx, int nterms,
                                 const int *n_orders_naik, int n_naiks, double *mom);
/* asqtad fermion force.  Replaces eo_fermion_force_multi of an asqtad
 * build (generic_ks/fermion_force_multi.c:29-44 -> fermion_force_fn_multi,
 * generic_ks/fermion_force_fn_multi.c:80-316; GPU wrapper
 * generic_ks/fermion_force_asqtad_gpu.c): mom[dir](x) <- TA(mom + 2 eps
 * U_mu(x) dS/dU_mu(x)) through the asqtad fat + Naik links (tadpole factor
 * u0 of the last mks_load_links_from_thin with MKS_ACTION_ASQTAD; no
 * unitarization), xxx_j and residues as for the HISQ force.  Returns
 * MKS_ERR_STATE unless asqtad links were loaded from thin links. */
int mks_fermion_force_multi_asqtad(double eps, const double *residues,
                                   const double *const *xxx, int nterms, double *mom);
/* The backward half of the force as a forward/backward pair (no reference
 * counterpart; MILC only ever applies the projected update): writes
 * ku[4*i+dir] (su3_matrix layout, thin links of the last load with phases
 * in) with dS = 2 Re sum_{x,mu} tr(K_U,mu(x) dU_mu(x)) for
 * S = 2 Re sum_j residues[j] X_j^dag D_eo[links(U)] Y_j at fixed X_j (even
 * part of xxx_j) and Y_j (odd part).  The forward half is D_eo itself on the
 * links built from U.  Uses the action of the last mks_load_links_from_thin
 * (or mks_load_hisq_aux: HISQ); n_orders_naik may be NULL when n_naiks is 1.
 * The force entry points apply mom <- TA(mom + 2 eps U K_U). */
int mks_fermion_force_adjoint(const double *residues, const double *const *xxx, int nterms,
                              const int *n_orders_naik, int n_naiks, double *ku);
/* FP64 flops of the adjoint kernels in the last force call (our count:
   198 per 3x3 complex matrix product), and the number of links where the
   eigenvalue filter (generic_ks/su3_mat_op.c:1680-1734) was applied. */
double mks_force_flops_last(void);
int mks_force_filter_count(void);

/* ------------------------------------------------------------------ */
/* Kernel timing.  When enabled, the library brackets every launch of its
 * kernels with CUDA events on its own stream; totals are per kernel family. */
#define MKS_K_DSLASH_F64   0
#define MKS_K_DSLASH_F32   1
#define MKS_K_DSLASH_F16   2
#define MKS_K_DSLASH_MRHS  3
#define MKS_K_BLAS         4
#define MKS_K_SHIFT        5
#define MKS_K_LINKS        6
#define MKS_K_FORCE        7
#define MKS_K_TUNE         8   /* autotuner trial launches */
#define MKS_K_GAUGE        9   /* gauge force/action, link update, momenta, RNG */
#define MKS_K_COUNT        10
int mks_timing_enable(int on);
int mks_timing_reset(void);
int mks_timing_get(int family, double *total_ms, long long *launches);
/* Total kernel launches issued by the library since the last reset
   (counted whether or not timing is enabled). */
long long mks_launch_count(void);
/* The library's CUDA stream, as a cudaStream_t cast to void*. */
void *mks_stream(void);

/* Run the D_eo kernel `iters` times at the given precision on resident
 * copies of the slot's links and a resident random source, timing each
 * launch with CUDA events (optionally writing a 256 MB buffer between
 * launches to flush L2).  Returns the mean launch time in ms in *ms.
 * nsrc > 1 times the multi-source kernel. */
int mks_bench_dslash(int prec, int nsrc, int parity, int slot, int iters, int flush_l2,
                     double *ms);

/* D_eo launch shape chosen by the autotuner for (prec, nsrc): G threads per
 * site, nb sources per thread, block threads per CTA.  The tuner times its
 * candidates on the live links the first time a precision and a class of
 * source counts (1, 2, 3-4, 5-8, 9-16) is launched, for the class's widest
 * count, and every count of the class takes that shape (environment
 * MKS_TUNE=0 keeps a fixed table).  Returns MKS_ERR_STATE when no shape
 * has been chosen for nsrc yet (a class's widest count has its shape as
 * soon as any count of the class was launched). */
int mks_tuned_shape(int prec, int nsrc, int *G, int *nb, int *block);

/* The same for the launches with the fused CG epilogue (D_eo, axpy and
 * three dot products in one kernel), tuned separately; *tma = 1 when the
 * TMA-staged kernel won (then *block = threads per CTA). */
int mks_tuned_shape_epi(int prec, int nsrc, int *G, int *nb, int *block, int *tma);

/* Counts of the last multi-shift call's iteration phase (no counterpart in
 * the reference; used to state the bytes the multi-shift update kernel
 * moves): the iterations and the shift updates, i.e. the shifts the update
 * kernel advanced summed over the iterations (a shift that has converged is
 * no longer advanced).  Per shift update the kernel moves 4 colour vectors
 * (psim and pm read and written), per iteration 4 more (r read and written,
 * ttt read, p written). */
int mks_multishift_counts(long long *iters, long long *shift_updates);

/* Which D_eo kernel the tuner chose for (prec, nsrc), plain D (epi = 0) or
 * fused-epilogue launches (epi = 1): 0 direct loads, 1 TMA-staged links,
 * 2 direct loads software-pipelined one term deep; plus 4 when the launch
 * uses a persistent grid (the CTAs that fit at once loop over the sites).
 * MKS_ERR_STATE when the pair has not been launched yet. */
int mks_tuned_variant(int prec, int nsrc, int epi);

/* ------------------------------------------------------------------ */
/* Gauge side of the RHMC molecular dynamics (mks_gauge.cu).  The library
 * keeps one resident thin-link field (the one the fermion links are built
 * from; phases in on the device) and one momentum field, and updates them
 * in place, as MILC's lattice[].link / lattice[].mom.  Changing the thin
 * links invalidates every fermion-link slot (mks_rebuild_links rebuilds).
 *  - mks_gauge_load / mks_gauge_get: thin links WITHOUT phases, host
 *    double[V][4][18] (MILC's rephase(OFF) state).
 *  - mks_mom_load / mks_mom_get: anti_hermitmat[V][4].
 *  - mks_rng_seed: MILC's site generators (SITERAND), seeded like
 *    initialize_site_prn_from_seed (generic/ranstuff.c:117-130) from iseed
 *    and each site's lexicographic index; mks_ranmom replaces ranmom
 *    (generic/ranmom.c); mks_gaussian_vector draws three complex Gaussians
 *    per site of `parity` into v (other sites untouched), as grsource_rhmc.c:
 *    31-41 does.  The streams continue from call to call.
 *  - mks_gauge_force replaces imp_gauge_force_ks / imp_gauge_force_gpu
 *    (generic_ks/gauge_force_imp_ks.c, generic/gauge_force_imp.c:37-223):
 *    mom <- TA(mom - eps beta/3 U sum c staples) for MILC's HISQ-improved
 *    Symanzik action (plaquette, rectangle, bent loop;
 *    generic/imp_actions/symanzik_1loop_hisq_action.h; nflavors = the
 *    total_dyn_flavors of make_loop_table).
 *  - mks_gauge_action: (beta/3) imp_gauge_action (generic/gauge_stuff.c:277),
 *    the g term of d_action_rhmc.c:27-29.
 *  - mks_update_u replaces update_u (ks_imp_rhmc/update_u.c:49-108):
 *    U <- exp(eps mom) U to eighth order.
 *  - mks_mom_action: hmom_action (ks_imp_rhmc/d_action_rhmc.c:89-122).
 *  - mks_reunitarize: reunitarize_ks (generic_ks/reunitarize_ks.c).
 *  - mks_plaquette: d_plaquette (generic/d_plaq4.c) without phases. */
int mks_gauge_load(const double *thin);
int mks_gauge_get(double *thin);
int mks_mom_load(const double *mom);
int mks_mom_get(double *mom);
int mks_rng_seed(int iseed);
int mks_ranmom(void);
int mks_gaussian_vector(int parity, double *v);
int mks_gauge_force(double eps, double beta, double u0, int nflavors);
/* the same with the staple sums in `prec` (MKS_PREC_DOUBLE as above, or
   MKS_PREC_SINGLE: FP32 staples and products, FP64 momentum update) */
int mks_gauge_force_prec(double eps, double beta, double u0, int nflavors, int prec);
int mks_gauge_action(double beta, double u0, int nflavors, double *action);
int mks_update_u(double eps);
int mks_mom_action(double *h);
int mks_reunitarize(void);
int mks_plaquette(double *ss, double *st);
/* Precision of later link constructions (mks_load_links_from_thin,
 * mks_rebuild_links) and fermion forces: MKS_PREC_DOUBLE (the default,
 * MILC's double build) or MKS_PREC_SINGLE (for molecular-dynamics forces,
 * like MILC's single-precision build: the smearing stages, the U(3)
 * projection, staples and force adjoints stored and computed in FP32; the
 * resident links, the slots' fat / long links and the momentum update stay
 * FP64 fields).  No reference counterpart in MILC's double build. */
int mks_md_precision(int prec);

/* ------------------------------------------------------------------ */
/* One RHMC molecular-dynamics trajectory (mks_rhmc.cu): MILC's update()
 * (ks_imp_rhmc/update_rhmc.c:182-473) for the HISQ action on the resident
 * thin links and momenta.  With refresh = 1 it draws the momenta (ranmom)
 * and one heat-bath source per pseudofermion field (grsource_rhmc.c:
 * phi = R_GR(M^dag M) g, g Gaussian on even sites) from the site
 * generators (mks_rng_seed first); with refresh = 0 it reuses the momenta
 * and the fields of the previous call.  It computes the action
 * (d_action_rhmc.c: g, h, f), integrates `steps` steps of size `epsilon`
 * with the chosen integrator, and the action again; the links and momenta
 * are left at the trajectory's end (the caller accepts or restores them;
 * MILC draws its Metropolis number from node_prn).  Multi-shift solves use
 * the offsets pole[1..order] and the residues res[0..order] of each
 * rational function (MILC's rationals file, ks_imp_rhmc/
 * load_rhmc_params.c), with resid_* NOT squared (cgresid_md_fa_gr) and
 * prec_* the inner precision (FP64 reproduces MILC's double build). */
#define MKS_INT_LEAPFROG 0
#define MKS_INT_OMELYAN  1
#define MKS_INT_2G1F     2
#define MKS_INT_3G1F     3
#define MKS_RHMC_MAX_PSEUDO 16
typedef struct {
  int order;            /* number of poles */
  const double *res;    /* order+1 residues, res[0] the constant term */
  const double *pole;   /* order+1 poles, pole[0] unused */
} mks_ratfunc;
typedef struct {
  double naik_eps;      /* naik_term_epsilon of the field (first field: 0) */
  mks_ratfunc md, gr, fa;
  double resid_md, resid_fa, resid_gr;
  int max_cg;           /* max_multicg_md_fa_gr */
} mks_pseudofermion;
typedef struct {
  double beta, u0;      /* gauge coupling and tadpole factor of the gauge action */
  int nflavors;         /* total_dyn_flavors (gauge action coefficients) */
  double epsilon;       /* microcanonical_time_step */
  int steps;            /* steps_per_trajectory */
  int int_alg;          /* MKS_INT_* */
  int n_pseudo;
  const mks_pseudofermion *pf;
  int prec_md, prec_fa, prec_gr;  /* MKS_PREC_* */
  int nrestart;         /* CG restarts (MILC's nrestart, 0 -> 5) */
  int refresh;
  int prec_force;       /* arithmetic of the gauge force, the fermion force and the
                           link rebuilds inside the integration: MKS_PREC_SINGLE, or
                           FP64 (any other value); the action is always FP64 */
} mks_rhmc_params;
typedef struct {
  double g0, h0, f0;    /* action terms at the start */
  double g1, h1, f1;    /* and at the end of the trajectory */
  double delta_s;       /* (g1+h1+f1) - (g0+h0+f0) */
  double plaq_ss, plaq_st;  /* plaquettes at the end (no phases) */
  double grsource_sum[MKS_RHMC_MAX_PSEUDO];  /* |g|^2 of each heat-bath Gaussian */
  long long cg_iters;   /* summed multi-shift iterations */
  int n_solves, unconverged, n_gauge_force, n_fermion_force;
  double t_total, t_solve, t_fermion_force, t_gauge_force, t_links;  /* seconds */
} mks_rhmc_result;
int mks_rhmc_trajectory(const mks_rhmc_params *p, mks_rhmc_result *r);

/* ------------------------------------------------------------------ */
/* Host-side synthetic inputs (no device work).  See mks_fields.c. */
void   mks_site_coords(const int dims[4], size_t index, int xyzt[4]);
size_t mks_site_index(const int dims[4], const int xyzt[4]);
double mks_staggered_phase(const int dims[4], const int xyzt[4], int dir);
int mks_gen_thin_links(const int dims[4], uint64_t seed, double a, double *links);
int mks_apply_phases(const int dims[4], double *links, int sign);
int mks_gen_vector(const int dims[4], uint64_t seed, int parity, double *vec);
int mks_gen_momenta(const int dims[4], uint64_t seed, double *mom);

#ifdef __cplusplus
}
#endif
#endif /* MILC_KS_GB300_H */
