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


def _call(lib, name, src_t, dst_t, parity):
    return getattr(lib, name)(ctypes.c_void_p(src_t.data_ptr()), ctypes.c_void_p(dst_t.data_ptr()), parity, 0)


def test_noalloc_dslash_matches_allocating_entry_point(gpu, oracle_cls):
    torch = pytest.importorskip("torch")
    m = gpu
    lib = m._lib.load()
    dims = (8, 8, 8, 8)
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    m.set_lattice(dims)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    for call, (seed, parity) in enumerate([(61, m.EVENANDODD), (62, m.EVEN)]):
        src = torch.from_numpy(m.gen_vector(dims, seed, m.EVENANDODD)).cuda()
        fill = torch.full_like(src, 3.0)
        out_ref, out_na = fill.clone(), fill.clone()
        assert _call(lib, "mks_dslash_fn_field_dev", src, out_ref, parity) == 0
        assert _call(lib, "mks_dslash_fn_field_dev_noalloc", src, out_na, parity) == 0, call
        torch.cuda.synchronize()
        a, b = out_na.cpu().numpy(), out_ref.cpu().numpy()
        # same tolerance as the other FP64 D_eo tests
        assert rel(a, b) < 1e-13, (call, rel(a, b))
        if parity == m.EVEN:
            V = a.shape[0]
            assert np.all(a[V // 2:] == 3.0)  # the other parity is left untouched
        # and against the oracle
        ref = orc.dslash(L["fat"][0], L["lng"][0], src.cpu().numpy(), parity, dst=np.full_like(a, 3.0))
        assert rel(a, ref) < 1e-13


def test_noalloc_dslash_rejects_lattice_beyond_limit(gpu, oracle_cls):
    m = gpu
    lib = m._lib.load()
    dims = (8, 8, 8, 8)
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    m.set_lattice(dims)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    m.set_lattice((32, 32, 32, 16))  # 524288 sites > 349525: rejected before any work
    st = lib.mks_dslash_fn_field_dev_noalloc(None, None, m.EVEN, 0)
    assert st == -1  # MKS_ERR_ARG
    m.set_lattice(dims)
