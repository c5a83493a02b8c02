"""Domain decomposition in t with halo exchange (milc_qcd_gb300/domain.py).

CPU: two gloo ranks each hold one t-slab extended by ghost slices, fill the
ghosts of the links and of the source by point-to-point exchange, apply the
oracle's D_eo on their local lattice, and the interiors reassemble the
global D_eo bit for bit; a CG over the two ranks (global sums by
all_reduce) reaches the single-domain solution.
GPU: two sub-domains on one device, each D_eo run by the library on its
extended local lattice, reassemble the global GPU D_eo bit for bit."""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, rel

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as tmp  # noqa: E402

DIMS = (4, 4, 4, 16)
MASS = 0.1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _global_problem():
    import milc_qcd_gb300 as m
    from oracle.oracle import Oracle
    U = m.apply_phases(DIMS, m.gen_thin_links(DIMS, 61, 0.3))
    orc = Oracle(DIMS)
    L = orc.hisq_links(U)
    src = m.gen_vector(DIMS, 62, m.EVENANDODD)
    return orc, L["fat"][0], L["lng"][0], src


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from milc_qcd_gb300.domain import TSlabs
    from oracle.oracle import Oracle, EVEN, ODD
    _, fat, lng, src = _global_problem()
    D = TSlabs(DIMS, world)
    orc = Oracle(D.local_dims)
    # links: interior from the rank's own slab, ghosts by exchange (once per link load)
    fat_l = D.exchange_dist(D.scatter_interior(fat, rank), rank)
    lng_l = D.exchange_dist(D.scatter_interior(lng, rank), rank)
    src_l = D.exchange_dist(D.scatter_interior(src, rank), rank)
    out = {}
    for name, par in (("even", EVEN), ("odd", ODD)):
        d = orc.dslash(fat_l, lng_l, src_l, par)
        out[name] = (D.interior_global(rank), d[D.interior()])
    # CG on 4m^2 - D_eo D_oe (even sites) with global sums over the ranks
    Vh_l = int(np.prod(D.local_dims)) // 2
    even = D.interior()[D.interior() < Vh_l]

    def gsum(a):
        t = torch.tensor([float(a)], dtype=torch.float64)
        dist.all_reduce(t)
        return float(t.item())

    def op(v):
        v = D.exchange_dist(v, rank)
        t = orc.dslash(fat_l, lng_l, v, ODD)
        t[:Vh_l] = 0
        t = D.exchange_dist(t, rank)
        w = orc.dslash(fat_l, lng_l, t, EVEN)
        res = np.zeros_like(v)
        res[even] = 4 * MASS * MASS * v[even] - w[even]
        return res

    b = np.zeros_like(src_l)
    b[even] = src_l[even]
    x = np.zeros_like(b)
    r = b.copy()
    p = r.copy()
    rr = gsum((r[even] ** 2).sum())
    bb = rr
    for _ in range(500):
        Ap = op(p)
        a = rr / gsum((p[even] * Ap[even]).sum())
        x[even] += a * p[even]
        r[even] -= a * Ap[even]
        rr_new = gsum((r[even] ** 2).sum())
        if rr_new < 1e-24 * bb:
            break
        p[even] = r[even] + (rr_new / rr) * p[even]
        rr = rr_new
    out["cg"] = (D.interior_global(rank), x[D.interior()])
    q.put((rank, out))
    dist.destroy_process_group()


def test_two_rank_halo_exchange_and_cg(lib, oracle_cls):
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    pc = tmp.start_processes(_worker, args=(2, port, q), nprocs=2, join=False, start_method="spawn")
    parts = dict(q.get(timeout=300) for _ in range(2))   # drain before joining: the results are large
    while not pc.join(timeout=60):
        pass
    orc, fat, lng, src = _global_problem()
    V = src.shape[0]
    for name, par in (("even", 0x02), ("odd", 0x01)):
        want = orc.dslash(fat, lng, src, par)
        got = np.zeros_like(src)
        for r in range(2):
            idx, vals = parts[r][name]
            got[idx] = vals
        lo, hi = (0, V // 2) if par == 0x02 else (V // 2, V)
        assert np.array_equal(got[lo:hi], want[lo:hi])
    b = src.copy()
    b[V // 2:] = 0
    _, xo, _ = orc.congrad(fat, lng, b, np.zeros_like(b), MASS, 0x02, 1e-12, 0.0, 500, 5)
    got = np.zeros_like(src)
    for r in range(2):
        idx, vals = parts[r]["cg"]
        got[idx] = vals
    assert rel(got[:V // 2], xo[:V // 2]) < 1e-10


@pytest.mark.gpu
def test_two_subdomains_on_one_gpu(gpu, oracle_cls):
    from milc_qcd_gb300.domain import TSlabs
    m = gpu
    _, fat, lng, src = _global_problem()
    m.set_lattice(DIMS)
    m.load_fn_links(fat, lng)
    want = m.dslash_fn_field(src, np.zeros_like(src), m.EVENANDODD)
    D = TSlabs(DIMS, 2)
    locs = {k: [D.scatter_interior(f, r) for r in range(2)] for k, f in (("fat", fat), ("lng", lng), ("src", src))}
    for k in locs:
        D.exchange_local(locs[k])
    got = np.zeros_like(src)
    for r in range(2):
        m.set_lattice(D.local_dims)
        m.load_fn_links(locs["fat"][r], locs["lng"][r])
        d = m.dslash_fn_field(locs["src"][r], np.zeros_like(locs["src"][r]), m.EVENANDODD)
        D.gather_interior(d, r, got)
    assert np.array_equal(got, want)


def test_site_index_table_matches_library(lib):
    """The vectorised MILC site map equals the library's mks_site_index."""
    import ctypes
    from milc_qcd_gb300.domain import _site_index_table
    dims = (4, 6, 2, 8)
    tab = _site_index_table(dims)
    L = lib._lib.load()
    d4 = (ctypes.c_int * 4)(*dims)
    for t in range(dims[3]):
        for z in range(dims[2]):
            for y in range(dims[1]):
                for x in range(dims[0]):
                    assert tab[t, z, y, x] == L.mks_site_index(d4, (ctypes.c_int * 4)(x, y, z, t))
    assert sorted(tab.reshape(-1)) == list(range(int(np.prod(dims))))
