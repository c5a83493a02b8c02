"""CG solvers on the GPU against the oracle (MILC's ks_congrad_parity semantics)."""
import numpy as np
import pytest

from conftest import hisq_setup, rel

pytestmark = pytest.mark.gpu

DIMS = (8, 8, 8, 8)


def _setup(m, oracle_cls, dims=DIMS):
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(dims)
    m.load_fn_links(fat, lng)
    return orc, fat, lng


@pytest.mark.parametrize("parity", ["EVEN", "ODD"])
def test_fp64_cg_matches_oracle(gpu, oracle_cls, parity):
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    par = getattr(m, parity)
    b = m.gen_vector(DIMS, 21, par)
    x0 = m.gen_vector(DIMS, 22, par) * 0.1
    qic = m.QuarkInvertControl(resid=1e-9, max=40, nrestart=10, parity=par, prec=m.PREC_DOUBLE)
    x = x0.copy()
    it = m.ks_congrad_parity(b, x, qic, 0.05)
    it_o, xo, out = orc.congrad(fat, lng, b, x0, 0.05, par, 1e-9, 0.0, 40, 10)
    # same algorithm, same restarts: identical iteration count, solution to rounding
    assert it == it_o and qic.final_iters == int(out[4])
    assert qic.final_restart == int(out[5]) and qic.converged == int(out[6]) == 1
    assert rel(x, xo) < 1e-11
    assert abs(qic.final_rsq - out[0]) <= 1e-6 * out[0]


@pytest.mark.parametrize("prec", ["PREC_SINGLE", "PREC_HALF"])
def test_mixed_cg_reaches_fp64_tolerance(gpu, oracle_cls, prec):
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    b = m.gen_vector(DIMS, 31, m.EVEN)
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=getattr(m, prec))
    x = np.zeros_like(b)
    m.ks_congrad_parity(b, x, qic, 0.02)
    assert qic.converged == 1 and qic.final_rsq < 1e-20
    assert qic.reliable_updates >= 1
    _, xo, _ = orc.congrad(fat, lng, b, np.zeros_like(b), 0.02, m.EVEN, 1e-13, 0.0, 2000, 5)
    # |x - x*| / |x*| <= cond * |r|/|b|; at m=0.02 on these links the bound is ~1e-8
    assert rel(x, xo) < 1e-7
    # true residual recomputed here in FP64 through the oracle
    Dx = orc.dslash(fat, lng, orc.dslash(fat, lng, x, m.ODD), m.EVEN)
    r = b - (4 * 0.02 ** 2 * x - Dx)
    V2 = b.shape[0] // 2
    assert np.linalg.norm(r[:V2]) / np.linalg.norm(b[:V2]) < 1.01e-10


def test_zero_source_gives_zero(gpu, oracle_cls):
    m = gpu
    _setup(m, oracle_cls)
    b = np.zeros((int(np.prod(DIMS)), 6))
    x = np.ones_like(b)
    qic = m.QuarkInvertControl(resid=1e-8, parity=m.EVEN)
    it = m.ks_congrad_parity(b, x, qic, 0.05)
    V2 = b.shape[0] // 2
    assert it == 0 and np.all(x[:V2] == 0) and np.all(x[V2:] == 1)


@pytest.mark.parametrize("prec", ["PREC_DOUBLE", "PREC_SINGLE", "PREC_HALF"])
@pytest.mark.parametrize("nsrc", [3, 8])
def test_block_cg_each_source_matches_single(gpu, oracle_cls, prec, nsrc):
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    srcs = [m.gen_vector(DIMS, 100 + k, m.EVEN) for k in range(nsrc)]
    xs = [np.zeros_like(s) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=getattr(m, prec))
    it, per = m.ks_congrad_block_parity(srcs, xs, qic, 0.02)
    for k in range(nsrc):
        assert per[k].converged == 1
        _, xo, _ = orc.congrad(fat, lng, srcs[k], np.zeros_like(srcs[k]), 0.02, m.EVEN, 1e-13, 0.0, 2000, 5)
        assert rel(xs[k], xo) < 1e-7, (k, rel(xs[k], xo))


@pytest.mark.parametrize("prec", ["PREC_SINGLE", "PREC_HALF"])
def test_block_cg_16_sources_larger_lattice(gpu, oracle_cls, prec):
    """16 sources on 16^4: reduction grids with thousands of blocks and
    16-row BLAS launches (multi-level reduction, scratch sizing)."""
    m = gpu
    dims = (16, 16, 16, 16)
    orc, fat, lng = _setup(m, oracle_cls, dims)
    srcs = [m.gen_vector(dims, 300 + k, m.EVEN) for k in range(16)]
    xs = [np.zeros_like(s) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=getattr(m, prec))
    it, per = m.ks_congrad_block_parity(srcs, xs, qic, 0.05)
    assert it > 10
    assert all(p.converged == 1 for p in per)
    for k in (0, 7, 15):
        _, xo, _ = orc.congrad(fat, lng, srcs[k], np.zeros_like(srcs[k]), 0.05, m.EVEN, 1e-13, 0.0, 2000, 5)
        assert rel(xs[k], xo) < 1e-7, (k, rel(xs[k], xo))


@pytest.mark.parametrize("prec", ["PREC_DOUBLE", "PREC_SINGLE"])
def test_mat_invert_uml_matches_oracle(gpu, oracle_cls, prec):
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    src = m.gen_vector(DIMS, 41, m.EVENANDODD)
    x = np.zeros_like(src)
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, prec=getattr(m, prec))
    m.mat_invert_uml_field(src, x, qic, 0.05)
    _, xo, _ = orc.mat_invert_uml(fat, lng, src, np.zeros_like(src), 0.05, 1e-12)
    assert rel(x, xo) < 1e-8
    # M x = src, checked with the oracle's D
    Mx = 2 * 0.05 * x + orc.dslash(fat, lng, x, m.EVENANDODD)
    assert rel(Mx, src) < 1e-9


@pytest.mark.parametrize("prec", ["PREC_DOUBLE", "PREC_SINGLE"])
def test_mat_invert_block_uml_matches_oracle(gpu, oracle_cls, prec):
    """mat_invert_block_uml (generic_ks/mat_invert.c:409-483): M^-1 of several
    sources in one call; each solution against the oracle's single-source
    mat_invert_uml and checked through M x = src with the oracle's D."""
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    nsrc = 5
    srcs = [m.gen_vector(DIMS, 140 + k, m.EVENANDODD) * (1.0 + 0.5 * k) for k in range(nsrc)]
    # the even half of dst is the even solve's initial guess (as in MILC); the
    # odd half is rebuilt from it and polished
    xs = [np.full_like(s, 0.25) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, prec=getattr(m, prec))
    it = m.mat_invert_block_uml(srcs, xs, qic, 0.05)
    assert it > 0
    for k in range(nsrc):
        _, xo, _ = orc.mat_invert_uml(fat, lng, srcs[k], np.zeros_like(srcs[k]), 0.05, 1e-12)
        assert rel(xs[k], xo) < 1e-8, (k, rel(xs[k], xo))
        Mx = 2 * 0.05 * xs[k] + orc.dslash(fat, lng, xs[k], m.EVENANDODD)
        assert rel(Mx, srcs[k]) < 1e-9, k


def test_graph_replay_with_kernel_timing(gpu, oracle_cls):
    """Solver batches replay as CUDA graphs after their first (eager) run;
    with kernel timing on, the replays carry their own event-record nodes and
    are counted and timed like eager launches."""
    import ctypes
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    lib = m._lib.load()
    b = m.gen_vector(DIMS, 91, m.EVEN)
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=m.PREC_SINGLE)
    lib.mks_timing_reset()
    lib.mks_timing_enable(1)
    xs = []
    for rep in range(3):
        x = np.zeros_like(b)
        m.ks_congrad_parity(b, x, qic, 0.02)
        assert qic.converged == 1
        xs.append(x)
    t, n = ctypes.c_double(), ctypes.c_longlong()
    m.check(lib.mks_timing_get(1, ctypes.byref(t), ctypes.byref(n)), "timing")
    lib.mks_timing_enable(0)
    assert n.value > 3 * 2 * 20 and t.value > 0
    # replayed solves give the same answer as the eager first one
    assert rel(xs[2], xs[0]) < 1e-12 and rel(xs[1], xs[0]) < 1e-12


@pytest.mark.parametrize("nsrc", [5, 8, 16])
def test_block_cg_tma_staged_links(gpu, oracle_cls, monkeypatch, nsrc):
    """The FP32 multi-source D_eo whose links are staged per tile in shared
    memory by TMA bulk copies (shape forced through MKS_SHAPE; a lattice no
    other test uses, so the shape is chosen afresh): every source reaches the
    oracle's solution, and the shape in use is the staged kernel's (block =
    tile sites x G threads per site: 24 x 8 or 16 x 16 here)."""
    import ctypes
    m = gpu
    dims = (8, 12, 8, 8)
    G = 8 if nsrc <= 8 else 16
    monkeypatch.setenv("MKS_SHAPE", "1:%d:%d:1:tma" % (nsrc, G))
    m.set_lattice((4, 4, 4, 4))   # a lattice change drops the shapes chosen earlier
    orc, fat, lng = _setup(m, oracle_cls, dims)
    srcs = [m.gen_vector(dims, 500 + k, m.EVEN) for k in range(nsrc)]
    xs = [np.zeros_like(s) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=m.PREC_SINGLE)
    it, per = m.ks_congrad_block_parity(srcs, xs, qic, 0.03)
    Gq, nb, block = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    m.check(m._lib.load().mks_tuned_shape(m.PREC_SINGLE, nsrc, ctypes.byref(Gq), ctypes.byref(nb),
                                          ctypes.byref(block)), "mks_tuned_shape")
    assert (Gq.value, nb.value, block.value) == (G, 1, 24 * 8 if G == 8 else 16 * 16)
    for k in range(nsrc):
        assert per[k].converged == 1
        _, xo, _ = orc.congrad(fat, lng, srcs[k], np.zeros_like(srcs[k]), 0.03, m.EVEN, 1e-13, 0.0, 2000, 5)
        assert rel(xs[k], xo) < 1e-7, (k, rel(xs[k], xo))


@pytest.mark.parametrize("flags,variant", [("p", 2), ("g", 4), ("a2", 19), ("a3", 27)])
@pytest.mark.parametrize("nsrc", [3, 8])
def test_block_cg_variant_kernels(gpu, oracle_cls, monkeypatch, flags, variant, nsrc):
    """The FP32 multi-source D_eo variants the autotuner can be offered
    (software-pipelined link loads, persistent grid, cp.async link buffers
    with 2 or 3 stages), each forced through MKS_SHAPE for both D launches
    of the iteration: the variant reported in use is the forced one and every
    source reaches the oracle's solution."""
    m = gpu
    dims = (8, 8, 12, 8)
    NB = 2 if nsrc <= 4 else 4
    monkeypatch.setenv("MKS_SHAPE", "1:%d:2:%d:256:%s" % (nsrc, NB, flags))
    m.set_lattice((4, 4, 4, 4))   # a lattice change drops the shapes chosen earlier
    orc, fat, lng = _setup(m, oracle_cls, dims)
    srcs = [m.gen_vector(dims, 700 + k, m.ODD) for k in range(nsrc)]
    xs = [np.zeros_like(s) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.ODD, prec=m.PREC_SINGLE)
    it, per = m.ks_congrad_block_parity(srcs, xs, qic, 0.05)
    assert m._lib.load().mks_tuned_variant(m.PREC_SINGLE, nsrc, 0) == variant
    for k in range(nsrc):
        assert per[k].converged == 1
        _, xo, _ = orc.congrad(fat, lng, srcs[k], np.zeros_like(srcs[k]), 0.05, m.ODD, 1e-13, 0.0, 2000, 5)
        assert rel(xs[k], xo) < 1e-7, (k, rel(xs[k], xo))


def test_tuner_source_count_classes(gpu, oracle_cls):
    """The autotuner chooses one shape per class of source counts (1, 2,
    3-4, 5-8, 9-16), tuned for the class's widest count: after a 5-source
    block solve on a fresh lattice the 5- and the 8-source D_eo have the
    same shape, wide enough for 8 sources, and the solve is correct."""
    import ctypes
    m = gpu
    dims = (8, 8, 8, 12)
    m.set_lattice((4, 4, 4, 4))   # a lattice change drops the shapes chosen earlier
    orc, fat, lng = _setup(m, oracle_cls, dims)
    srcs = [m.gen_vector(dims, 900 + k, m.EVEN) for k in range(5)]
    xs = [np.zeros_like(s) for s in srcs]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=m.PREC_SINGLE)
    m.ks_congrad_block_parity(srcs, xs, qic, 0.04)
    lib = m._lib.load()
    shapes = []
    for n in (5, 8):
        G, nb, block = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        m.check(lib.mks_tuned_shape(m.PREC_SINGLE, n, ctypes.byref(G), ctypes.byref(nb), ctypes.byref(block)),
                "mks_tuned_shape")
        shapes.append((G.value, nb.value, block.value))
    assert shapes[0] == shapes[1] and shapes[0][0] * shapes[0][1] >= 8
    for k in range(5):
        _, xo, _ = orc.congrad(fat, lng, srcs[k], np.zeros_like(srcs[k]), 0.04, m.EVEN, 1e-13, 0.0, 2000, 5)
        assert rel(xs[k], xo) < 1e-7, (k, rel(xs[k], xo))


@pytest.mark.parametrize("parity", ["EVEN", "ODD"])
def test_block_cg_page_locked_host_arrays(gpu, oracle_cls, parity):
    """Page-locked host arrays are read and written in place by the layout
    kernels (no staging copy): the solutions equal those of pageable arrays
    bit for bit, and the other parity's half of each destination is kept."""
    torch = pytest.importorskip("torch")
    m = gpu
    orc, fat, lng = _setup(m, oracle_cls)
    par = getattr(m, parity)
    nsrc = 3
    srcs = [m.gen_vector(DIMS, 300 + k, par) for k in range(nsrc)]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=par, prec=m.PREC_SINGLE)
    V2 = srcs[0].shape[0] // 2
    solve = slice(0, V2) if par == m.EVEN else slice(V2, None)
    keep = slice(V2, None) if par == m.EVEN else slice(0, V2)
    xs = [np.full_like(s, 0.5) for s in srcs]
    for x in xs:
        x[solve] = 0.0
    ref = [x.copy() for x in xs]
    m.ks_congrad_block_parity(srcs, ref, qic, 0.03)
    ps = [torch.from_numpy(s).pin_memory().numpy() for s in srcs]
    px = [torch.from_numpy(x).pin_memory().numpy() for x in xs]
    it, per = m.ks_congrad_block_parity(ps, px, qic, 0.03)
    for k in range(nsrc):
        assert per[k].converged == 1
        assert np.array_equal(px[k], ref[k])
        assert np.all(px[k][keep] == 0.5)
