"""Generate the golden fixtures in this folder from MILC itself.

MILC's CPU code is compiled from the reference sources by oracle/ref/Makefile
into oracle/_ref/libmilc_ref_{hisq,asqtad}.so (only where the reference tree
exists).  This script feeds it seeded synthetic fields (the package's host
generator) and stores inputs and MILC's outputs as .npz files:

  hisq_4x4x4x8.npz    HISQ U(3) action, two Naik groups (eps 0, -0.1):
                      thin links, V, W, fat/long links per group, D on
                      every parity, CG, multi-shift CG, M^-1, fermion force
  asqtad_4x4x4x8.npz  asqtad action (u0 = 1): fat/long links, D, CG

Run:  python tests/golden/make_golden.py
Each action runs in its own process (MILC keeps one global lattice).
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

DIMS = (4, 4, 4, 8)
MASS = 0.05
EPS_NAIK = (0.0, -0.1)


def _hisq(path):
    import milc_qcd_gb300 as m
    from oracle.oracle import MilcRef, EVEN, ODD, EVENANDODD
    U = m.gen_thin_links(DIMS, 101, 0.3)
    ref = MilcRef(DIMS, "hisq", EPS_NAIK)
    ref.set_thin_links(U)
    ref.build_links()
    out = {"dims": np.array(DIMS), "thin": U, "thin_phased": ref.thin_links_phased(),
           "eps_naik": np.array(EPS_NAIK), "mass": np.array(MASS)}
    _, Vl, W = ref.hisq_aux()
    out["V"], out["W"] = Vl, W
    for g in range(len(EPS_NAIK)):
        out["fat%d" % g], out["lng%d" % g] = ref.fn_links(g)
    src = m.gen_vector(DIMS, 102, m.EVENANDODD)
    out["src"] = src
    for name, par in (("even", EVEN), ("odd", ODD), ("both", EVENANDODD)):
        out["dslash_" + name] = ref.dslash(src, par)
    b = m.gen_vector(DIMS, 103, m.EVEN)
    it, x, q = ref.congrad(b, np.zeros_like(b), MASS, EVEN, 1e-9, 0.0, 40, 10)
    out.update(cg_src=b, cg_x=x, cg_qic=q, cg_iters=np.array(it))
    offs = np.array([0.01, 0.03, 0.1, 0.5])
    it, psim, frsq = ref.multicg_offset(b, offs, EVEN, 1e-10)
    out.update(ms_offsets=offs, ms_psim=psim, ms_iters=np.array(it))
    it, x, q = ref.mat_invert_uml(src, np.zeros_like(src), MASS, 1e-10)
    out.update(mi_x=x, mi_iters=np.array(it))
    xxx = np.stack([m.gen_vector(DIMS, 110 + j, m.EVENANDODD) for j in range(3)])
    res = np.array([0.2, 0.5, 0.9])
    orders = np.array([2, 1], dtype=np.int32)
    mom0 = m.gen_momenta(DIMS, 111)
    mom = ref.fermion_force(0.07, res, xxx, orders=orders, mom=mom0)
    out.update(ff_xxx=xxx, ff_res=res, ff_orders=orders, ff_eps=np.array(0.07), ff_mom0=mom0, ff_mom=mom)
    np.savez_compressed(path, **out)
    return path


def _asqtad(path):
    import milc_qcd_gb300 as m
    from oracle.oracle import MilcRef, EVEN
    U = m.gen_thin_links(DIMS, 201, 0.3)
    ref = MilcRef(DIMS, "asqtad")
    ref.set_thin_links(U)
    ref.build_links()
    fat, lng = ref.fn_links(0)
    src = m.gen_vector(DIMS, 202, m.EVENANDODD)
    b = m.gen_vector(DIMS, 203, m.EVEN)
    it, x, q = ref.congrad(b, np.zeros_like(b), MASS, EVEN, 1e-9, 0.0, 40, 10)
    np.savez_compressed(path, dims=np.array(DIMS), thin=U, thin_phased=ref.thin_links_phased(), fat=fat, lng=lng,
                        src=src, dslash_both=ref.dslash(src, 3), cg_src=b, cg_x=x, cg_qic=q,
                        cg_iters=np.array(it), mass=np.array(MASS))
    return path


def main():
    from oracle.oracle import ref_available
    if not (ref_available("hisq") and ref_available("asqtad")):
        from oracle.oracle import build_ref
        build_ref()
    ctx = mp.get_context("spawn")
    for fn, name in ((_hisq, "hisq_4x4x4x8.npz"), (_asqtad, "asqtad_4x4x4x8.npz")):
        with ctx.Pool(1) as pool:
            print(pool.apply(fn, (os.path.join(HERE, name),)))


if __name__ == "__main__":
    main()
