"""Parity at the benchmark's own sizes (HISQ, seeded exp(i 0.3 H) links):

* D_eo in FP64 on 32^3x64 against the oracle (1e-13);
* the production solve -- 8 sources in one block, FP32 inner CG with FP64
  reliable updates, |r|/|b| = 1e-10, m = 0.01 -- every source's true
  residual recomputed with the oracle's FP64 D, and every solution against
  the oracle's FP64 CG (MILC's d_congrad5_fn_milc.c) of the same source;
* the 11-offset multi-shift (sigma_i = 4m^2 + s_i, s_i log-uniform in
  [1e-4, 1]) in mixed precision: every shift's exact residual through the
  oracle's D, the solutions against the oracle's FP64 multi-shift CG, and
  the FP64 multi-shift's iteration count against the oracle's;
* the config-4 force chain on 16^3x32: a 6-term rational function
  (residues in [0.1, 1], offsets log-uniform in [1e-3, 1]) solved by the
  FP64 multi-shift to 1e-12, then the HISQ fermion force: the force kernels
  on the same solutions against the oracle's force (1e-10), and the GPU's
  whole chain against the oracle's (1e-8).

The GPU solves read the oracle's fat and long links, so both sides apply the
same operator.  The oracle runs on the host cores: these tests take a few
minutes there."""
import numpy as np
import pytest

from conftest import hisq_setup, rel

pytestmark = pytest.mark.gpu

DIMS = (32, 32, 32, 64)
MASS = 0.01
SEED_LINKS = 20251203


@pytest.fixture(scope="module")
def big(gpu, oracle_cls):
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS, seed=SEED_LINKS)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(DIMS)
    m.load_fn_links(fat, lng)
    return m, orc, fat, lng


def _true_residual(orc, fat, lng, b, x, sigma):
    """|b - (sigma - D_eo D_oe) x| / |b| on the even sites, oracle D, FP64."""
    Vh = b.shape[0] // 2
    Dx = orc.dslash(fat, lng, orc.dslash(fat, lng, x, 0x01), 0x02)
    r = b[:Vh] - (sigma * x[:Vh] - Dx[:Vh])
    return float(np.linalg.norm(r) / np.linalg.norm(b[:Vh]))


def test_dslash_fp64_32c64(big):
    m, orc, fat, lng = big
    src = m.gen_vector(DIMS, 4001, m.EVENANDODD)
    for parity in (m.EVEN, m.ODD):
        out = np.zeros_like(src)
        m.dslash_fn_field(src, out, parity)
        ref = orc.dslash(fat, lng, src, parity)
        assert rel(out, ref) < 1e-13, (parity, rel(out, ref))


def test_block_cg_8_sources_fp32_inner_32c64(big):
    m, orc, fat, lng = big
    nsrc = 8
    srcs = [m.gen_vector(DIMS, 4242 + k, m.EVEN) for k in range(nsrc)]
    xs = [np.zeros_like(s) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=10, parity=m.EVEN, prec=m.PREC_SINGLE)
    it, per = m.ks_congrad_block_parity(srcs, xs, qic, MASS)
    Vh = srcs[0].shape[0] // 2
    for k in range(nsrc):
        assert per[k].converged == 1, k
        assert per[k].reliable_updates >= 5, k
        assert _true_residual(orc, fat, lng, srcs[k], xs[k], 4 * MASS ** 2) <= 1e-10, k
    # MILC's FP64 CG of every source (independent solves run in lockstep)
    _, xo, out = orc.congrad_multi(fat, lng, srcs, [np.zeros_like(s) for s in srcs], MASS, m.EVEN, 1e-10, 0.0,
                                   1000, 10)
    for k in range(nsrc):
        assert out[k][6] == 1, k
        err = float(np.linalg.norm(xs[k][:Vh] - xo[k][:Vh]) / np.linalg.norm(xo[k][:Vh]))
        assert err < 1e-10, (k, err)


def test_multishift_11_offsets_32c64(big):
    m, orc, fat, lng = big
    b = m.gen_vector(DIMS, 4242, m.EVEN)
    offs = 4 * MASS ** 2 + np.logspace(-4, 0, 11)
    Vh = b.shape[0] // 2
    it_o, po, _ = orc.multicg_offset(fat, lng, b, offs, m.EVEN, 1e-10)
    # FP64: MILC's algorithm, the oracle's iteration count
    p64 = [np.zeros_like(b) for _ in offs]
    q64 = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, parity=m.EVEN, prec=m.PREC_DOUBLE)
    it64, _ = m.ks_multicg_offset_field(b, p64, offs, q64)
    assert abs(it64 - it_o) <= 1, (it64, it_o)
    # mixed precision (FP32 multi-shift, FP64 reliable updates and refinement)
    psim = [np.zeros_like(b) for _ in offs]
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, parity=m.EVEN, prec=m.PREC_SINGLE)
    it, per = m.ks_multicg_offset_field(b, psim, offs, qic)
    # The criterion is each shift's exact residual (1e-10, recomputed here with
    # the oracle's FP64 D).  Solutions are compared more loosely: MILC's
    # multi-shift stops updating a shift as soon as that shift's own residual
    # meets the target, so two solutions that both meet it may differ by up
    # to (condition number) x 1e-10.  The same algorithm in FP64 stops at the
    # same iterations and agrees closely; the mixed solve is refined further.
    errs = []
    for j, s in enumerate(offs):
        assert per[j].converged == 1, j
        assert _true_residual(orc, fat, lng, b, psim[j], s) <= 1e-10, j
        assert _true_residual(orc, fat, lng, b, p64[j], s) <= 1.5e-10, j  # MILC stops on the iterated residual
        e_mixed, e_64 = (float(np.linalg.norm(x[:Vh] - po[j][:Vh]) / np.linalg.norm(po[j][:Vh]))
                         for x in (psim[j], p64[j]))
        errs.append((j, e_mixed, e_64))
    assert all(e_mixed < 1e-8 and e_64 < 1e-9 for _, e_mixed, e_64 in errs), errs


def test_force_chain_6_terms_16c32(gpu, oracle_cls):
    """Pseudofermion phi (Gaussian, even sites) -> X_j = (M^dag M + sigma_j)^-1
    phi by the FP64 multi-shift to 1e-12 -> HISQ fermion force with residues
    r_j, on the GPU and in the oracle."""
    m = gpu
    dims = (16, 16, 16, 32)
    U, orc, L = hisq_setup(m, oracle_cls, dims, seed=77)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(dims)
    m.load_hisq_links(U)
    rng = np.random.default_rng(4)
    residues = np.sort(rng.uniform(0.1, 1.0, 6))
    offsets = np.logspace(-3, 0, 6)
    phi = m.gen_vector(dims, 4444, m.EVEN)
    Vh = phi.shape[0] // 2
    psim = [np.zeros_like(phi) for _ in offsets]
    qic = m.QuarkInvertControl(resid=1e-12, max=2000, nrestart=5, parity=m.EVEN, prec=m.PREC_DOUBLE)
    m.ks_multicg_offset_field(phi, psim, offsets, qic)
    _, po, _ = orc.multicg_offset(fat, lng, phi, offsets, m.EVEN, 1e-12, 2000)
    for j, s in enumerate(offsets):
        # MILC's multi-shift stops each shift on its iterated residual
        assert _true_residual(orc, fat, lng, phi, psim[j], s) <= 1.5e-12, j
        assert rel(psim[j][:Vh], po[j][:Vh]) < 1e-9, (j, rel(psim[j][:Vh], po[j][:Vh]))

    def xxx_of(sols):
        out = []
        for x in sols:
            x = x.copy()
            x[Vh:] = 0.0
            Dx = orc.dslash(fat, lng, x, m.ODD)
            x[Vh:] = Dx[Vh:]   # X on even sites, D_oe X on odd sites (MILC's layout of the force input)
            out.append(x)
        return np.stack(out)

    mom0 = m.gen_momenta(dims, 6)
    mom_o = orc.fermion_force_hisq(U, 0.02, residues, xxx_of(po), mom=mom0)
    # the force kernels on the same solutions: 1e-10
    mom_g = mom0.copy()
    m.eo_fermion_force_multi(0.02, list(residues), list(xxx_of(po)), mom_g)
    assert rel((mom_g - mom0)[..., :9], (mom_o - mom0)[..., :9]) < 1e-10
    # the whole GPU chain (its own solves) against the oracle's chain
    mom_c = mom0.copy()
    m.eo_fermion_force_multi(0.02, list(residues), list(xxx_of(psim)), mom_c)
    assert rel((mom_c - mom0)[..., :9], (mom_o - mom0)[..., :9]) < 1e-8
