"""The allocation-free D_eo entry point (mks_dslash_fn_field_dev_noalloc).

Some callers cannot call cudaMalloc when they apply the operator -- for
example an application that has handed nearly all device memory to its own
pool allocator.  This entry point keeps its staging buffers in a fixed device
array instead of allocating them.  Its results must equal those of the
allocating entry point (mks_dslash_fn_field_dev) on the same inputs, call
after call, since every call reuses the same array.

This file is named to be collected last: if it fails, a run that stops at the
first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import hisq_setup, rel

pytestmark = pytest.mark.gpu

LIMIT_SITES = 349525  # 32 MiB of FP64 input + output staging


def _call(lib, name, src_t, dst_t, parity):
    return getattr(lib, name)(ctypes.c_void_p(src_t.data_ptr()), ctypes.c_void_p(dst_t.data_ptr()), parity, 0)


def _pair(torch, lib, src, parity, fill=3.0):
    out_ref, out_na = torch.full_like(src, fill), torch.full_like(src, fill)
    assert _call(lib, "mks_dslash_fn_field_dev", src, out_ref, parity) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert _call(lib, "mks_dslash_fn_field_dev_noalloc", src, out_na, parity) == 0
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return out_na.cpu().numpy(), out_ref.cpu().numpy(), free0, free1


def test_noalloc_dslash_matches_allocating_entry_point(gpu, oracle_cls):
    torch = pytest.importorskip("torch")
    m = gpu
    lib = m._lib.load()
    dims = (8, 8, 8, 8)
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    m.set_lattice(dims)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    V = int(np.prod(dims))
    for call, (seed, parity) in enumerate([(61, m.EVENANDODD), (62, m.EVEN), (63, m.ODD)]):
        src = torch.from_numpy(m.gen_vector(dims, seed, m.EVENANDODD)).cuda()
        a, b, free0, free1 = _pair(torch, lib, src, parity)
        # the array and the kernels were made resident by mks_init: no call,
        # the first included, takes device memory
        assert free1 == free0, (call, free0 - free1)
        # same tolerance as the other FP64 D_eo tests
        assert rel(a, b) < 1e-13, (call, rel(a, b))
        if parity == m.EVEN:
            assert np.all(a[V // 2:] == 3.0)  # the other parity is left untouched
        if parity == m.ODD:
            assert np.all(a[:V // 2] == 3.0)
        ref = orc.dslash(L["fat"][0], L["lng"][0], src.cpu().numpy(), parity, dst=np.full_like(a, 3.0))
        assert rel(a, ref) < 1e-13, (call, rel(a, ref))


def test_noalloc_dslash_near_size_limit(gpu):
    """24^4 = 331,776 sites, just under the array's 349,525-site limit: two
    calls in a row (both parities) against the allocating entry point."""
    torch = pytest.importorskip("torch")
    m = gpu
    lib = m._lib.load()
    dims = (24, 24, 24, 24)
    assert int(np.prod(dims)) <= LIMIT_SITES
    m.set_lattice(dims)
    m.load_hisq_links(m.apply_phases(dims, m.gen_thin_links(dims, 17, 0.3)))
    for seed, parity in ((71, m.EVEN), (72, m.ODD)):
        src = torch.from_numpy(m.gen_vector(dims, seed, m.EVENANDODD)).cuda()
        a, b, free0, free1 = _pair(torch, lib, src, parity, fill=-1.0)
        assert free1 == free0
        assert rel(a, b) < 1e-13, (parity, rel(a, b))


def test_noalloc_dslash_rejects_lattice_beyond_limit(gpu, oracle_cls):
    m = gpu
    lib = m._lib.load()
    dims = (8, 8, 8, 8)
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    try:
        m.set_lattice((32, 32, 32, 16))  # 524288 sites > 349525: rejected before any work
        m.load_hisq_links(m.apply_phases((32, 32, 32, 16), m.gen_thin_links((32, 32, 32, 16), 5, 0.3)))
        st = lib.mks_dslash_fn_field_dev_noalloc(None, None, m.EVEN, 0)
        assert st == -1  # MKS_ERR_ARG
    finally:
        m.set_lattice(dims)
        m.load_fn_links(L["fat"][0], L["lng"][0])
