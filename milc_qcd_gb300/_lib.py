"""ctypes binding of libmilc_ks_gb300.so (the C ABI in include/milc_ks_gb300.h).

Loading fails loudly when the shared library is missing: there is no CPU
fallback for any entry point.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmilc_ks_gb300.so")

MKS_OK = 0
MKS_ODD, MKS_EVEN, MKS_EVENANDODD = 0x01, 0x02, 0x03
MKS_PREC_HALF, MKS_PREC_SINGLE, MKS_PREC_DOUBLE = 0, 1, 2
MKS_ACTION_HISQ, MKS_ACTION_ASQTAD = 1, 2
MKS_MAX_SLOTS = 12
KERNEL_FAMILIES = {"dslash_f64": 0, "dslash_f32": 1, "dslash_f16": 2, "dslash_mrhs": 3, "blas": 4,
                   "shift": 5, "links": 6, "force": 7, "tune": 8, "gauge": 9}


class InvertArg(ctypes.Structure):
    _fields_ = [("max", ctypes.c_int), ("nrestart", ctypes.c_int), ("parity", ctypes.c_int),
                ("prec", ctypes.c_int), ("resid", ctypes.c_double), ("relresid", ctypes.c_double),
                ("delta", ctypes.c_double)]


class InvertResult(ctypes.Structure):
    _fields_ = [("final_rsq", ctypes.c_double), ("final_relrsq", ctypes.c_double),
                ("size_r", ctypes.c_double), ("size_relr", ctypes.c_double),
                ("final_iters", ctypes.c_int), ("final_restart", ctypes.c_int),
                ("converged", ctypes.c_int), ("reliable_updates", ctypes.c_int)]


DP = ctypes.POINTER(ctypes.c_double)
DPP = ctypes.POINTER(DP)
IP = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); every symbol declared in the public header
SIGNATURES = {
    "mks_init": (ctypes.c_int, [ctypes.c_int]),
    "mks_finalize": (ctypes.c_int, []),
    "mks_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "mks_set_lattice": (ctypes.c_int, [IP]),
    "mks_load_fn_links": (ctypes.c_int, [ctypes.c_int, DP, DP, ctypes.c_double]),
    "mks_load_fn_links_dev": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]),
    "mks_invalidate_fn_links": (ctypes.c_int, [ctypes.c_int]),
    "mks_get_fn_links": (ctypes.c_int, [ctypes.c_int, DP, DP]),
    "mks_dslash_fn_field": (ctypes.c_int, [DP, DP, ctypes.c_int, ctypes.c_int]),
    "mks_dslash_fn_field_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "mks_dslash_fn_field_dev_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                                       ctypes.c_int]),
    "mks_ks_congrad_parity": (ctypes.c_int, [DP, DP, ctypes.c_double, ctypes.c_int,
                                             ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_ks_congrad_parity_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                                 ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_ks_congrad_block_parity": (ctypes.c_int, [ctypes.c_int, DPP, DPP, ctypes.c_double, ctypes.c_int,
                                                   ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_ks_congrad_block_parity_dev": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_double,
                                                       ctypes.c_int, ctypes.POINTER(InvertArg),
                                                       ctypes.POINTER(InvertResult)]),
    "mks_mat_invert_uml_field": (ctypes.c_int, [DP, DP, ctypes.c_double, ctypes.c_int,
                                                ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_mat_invert_block_uml": (ctypes.c_int, [ctypes.c_int, DPP, DPP, ctypes.c_double, ctypes.c_int,
                                                ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_ks_multicg_offset_field": (ctypes.c_int, [DP, DPP, DP, ctypes.c_int, ctypes.c_int,
                                                   ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_ks_multicg_offset_field_dev": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), DP,
                                                       ctypes.c_int, ctypes.c_int, ctypes.POINTER(InvertArg),
                                                       ctypes.POINTER(InvertResult)]),
    "mks_ks_multicg_offset_multi_dev": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                                       ctypes.POINTER(ctypes.c_int), DP,
                                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                                       ctypes.POINTER(InvertArg), ctypes.POINTER(InvertResult)]),
    "mks_load_links_from_thin": (ctypes.c_int, [ctypes.c_int, DP, ctypes.c_int, DP, ctypes.c_double]),
    "mks_get_hisq_aux": (ctypes.c_int, [DP, DP]),
    "mks_hisq_reunit_svd_count": (ctypes.c_int, []),
    "mks_fatlong_links": (ctypes.c_int, [DP, DP, DP, DP]),
    "mks_hisq_aux_links": (ctypes.c_int, [DP, DP, DP, DP]),
    "mks_load_hisq_aux": (ctypes.c_int, [DP, DP, DP]),
    "mks_fermion_force_multi_hisq": (ctypes.c_int, [ctypes.c_double, DP, DPP, ctypes.c_int, IP, ctypes.c_int, DP]),
    "mks_fermion_force_multi_asqtad": (ctypes.c_int, [ctypes.c_double, DP, DPP, ctypes.c_int, DP]),
    "mks_fermion_force_adjoint": (ctypes.c_int, [DP, DPP, ctypes.c_int, IP, ctypes.c_int, DP]),
    "mks_force_flops_last": (ctypes.c_double, []),
    "mks_rebuild_links": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, DP, ctypes.c_double]),
    "mks_rhmc_trajectory": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "mks_md_precision": (ctypes.c_int, [ctypes.c_int]),
    "mks_gauge_load": (ctypes.c_int, [DP]),
    "mks_gauge_get": (ctypes.c_int, [DP]),
    "mks_mom_load": (ctypes.c_int, [DP]),
    "mks_mom_get": (ctypes.c_int, [DP]),
    "mks_rng_seed": (ctypes.c_int, [ctypes.c_int]),
    "mks_ranmom": (ctypes.c_int, []),
    "mks_gaussian_vector": (ctypes.c_int, [ctypes.c_int, DP]),
    "mks_gauge_force": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]),
    "mks_gauge_action": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_int, DP]),
    "mks_gauge_force_prec": (ctypes.c_int, [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                            ctypes.c_int]),
    "mks_update_u": (ctypes.c_int, [ctypes.c_double]),
    "mks_mom_action": (ctypes.c_int, [DP]),
    "mks_reunitarize": (ctypes.c_int, []),
    "mks_plaquette": (ctypes.c_int, [DP, DP]),
    "mks_force_filter_count": (ctypes.c_int, []),
    "mks_timing_enable": (ctypes.c_int, [ctypes.c_int]),
    "mks_timing_reset": (ctypes.c_int, []),
    "mks_timing_get": (ctypes.c_int, [ctypes.c_int, DP, ctypes.POINTER(ctypes.c_longlong)]),
    "mks_launch_count": (ctypes.c_longlong, []),
    "mks_stream": (ctypes.c_void_p, []),
    "mks_bench_dslash": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, DP]),
    "mks_tuned_shape": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, IP, IP, IP]),
    "mks_tuned_shape_epi": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, IP, IP, IP, IP]),
    "mks_tuned_variant": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "mks_multishift_counts": (ctypes.c_int, [ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
    "mks_site_coords": (None, [IP, ctypes.c_size_t, IP]),
    "mks_site_index": (ctypes.c_size_t, [IP, IP]),
    "mks_staggered_phase": (ctypes.c_double, [IP, IP, ctypes.c_int]),
    "mks_gen_thin_links": (ctypes.c_int, [IP, ctypes.c_uint64, ctypes.c_double, DP]),
    "mks_apply_phases": (ctypes.c_int, [IP, DP, ctypes.c_int]),
    "mks_gen_vector": (ctypes.c_int, [IP, ctypes.c_uint64, ctypes.c_int, DP]),
    "mks_gen_momenta": (ctypes.c_int, [IP, ctypes.c_uint64, DP]),
}

_lib = None


def load(path=LIB_PATH):
    """Load the library and attach signatures; raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libmilc_ks_gb300.so not built (run __graft_entry__.build()); "
                           "there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


MKS_INT_LEAPFROG, MKS_INT_OMELYAN, MKS_INT_2G1F, MKS_INT_3G1F = 0, 1, 2, 3
MKS_RHMC_MAX_PSEUDO = 16


class RatFunc(ctypes.Structure):
    _fields_ = [("order", ctypes.c_int), ("res", DP), ("pole", DP)]


class Pseudofermion(ctypes.Structure):
    _fields_ = [("naik_eps", ctypes.c_double), ("md", RatFunc), ("gr", RatFunc), ("fa", RatFunc),
                ("resid_md", ctypes.c_double), ("resid_fa", ctypes.c_double), ("resid_gr", ctypes.c_double),
                ("max_cg", ctypes.c_int)]


class RhmcParams(ctypes.Structure):
    _fields_ = [("beta", ctypes.c_double), ("u0", ctypes.c_double), ("nflavors", ctypes.c_int),
                ("epsilon", ctypes.c_double), ("steps", ctypes.c_int), ("int_alg", ctypes.c_int),
                ("n_pseudo", ctypes.c_int), ("pf", ctypes.POINTER(Pseudofermion)),
                ("prec_md", ctypes.c_int), ("prec_fa", ctypes.c_int), ("prec_gr", ctypes.c_int),
                ("nrestart", ctypes.c_int), ("refresh", ctypes.c_int), ("prec_force", ctypes.c_int)]


class RhmcResult(ctypes.Structure):
    _fields_ = [("g0", ctypes.c_double), ("h0", ctypes.c_double), ("f0", ctypes.c_double),
                ("g1", ctypes.c_double), ("h1", ctypes.c_double), ("f1", ctypes.c_double),
                ("delta_s", ctypes.c_double), ("plaq_ss", ctypes.c_double), ("plaq_st", ctypes.c_double),
                ("grsource_sum", ctypes.c_double * MKS_RHMC_MAX_PSEUDO), ("cg_iters", ctypes.c_longlong),
                ("n_solves", ctypes.c_int), ("unconverged", ctypes.c_int), ("n_gauge_force", ctypes.c_int),
                ("n_fermion_force", ctypes.c_int), ("t_total", ctypes.c_double), ("t_solve", ctypes.c_double),
                ("t_fermion_force", ctypes.c_double), ("t_gauge_force", ctypes.c_double),
                ("t_links", ctypes.c_double)]


class MksError(RuntimeError):
    pass


def check(status, what=""):
    if status < 0:
        msg = load().mks_error_string(status)
        raise MksError("%s failed: status %d (%s)" % (what, status, msg.decode() if msg else "?"))
    return status
