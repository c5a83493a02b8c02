"""Host-side synthetic inputs: SU(3) thin links, phases, determinism."""
import numpy as np


def test_thin_links_are_su3_and_deterministic(lib):
    dims = (4, 4, 4, 6)
    U = lib.gen_thin_links(dims, 5, 0.3)
    assert np.array_equal(U, lib.gen_thin_links(dims, 5, 0.3))
    assert not np.array_equal(U, lib.gen_thin_links(dims, 6, 0.3))
    M = U.reshape(-1, 3, 3, 2)
    Mc = M[..., 0] + 1j * M[..., 1]
    assert np.abs(np.einsum("nij,nkj->nik", Mc, Mc.conj()) - np.eye(3)).max() < 1e-14
    assert np.abs(np.linalg.det(Mc) - 1).max() < 1e-14
    # exp(i a H): eigen-phases small for a = 0.3
    assert np.abs(np.angle(np.linalg.eigvals(Mc))).max() < 3.0


def test_phases_match_oracle(lib, oracle_cls):
    dims = (4, 6, 4, 8)
    U = lib.gen_thin_links(dims, 9, 0.3)
    assert np.array_equal(lib.apply_phases(dims, U), oracle_cls(dims).rephase(U))


def test_vector_parity_and_normalisation(lib):
    dims = (8, 8, 8, 8)
    V = int(np.prod(dims))
    e = lib.gen_vector(dims, 1, lib.EVEN)
    assert np.all(e[V // 2:] == 0) and np.any(e[: V // 2] != 0)
    both = lib.gen_vector(dims, 1, lib.EVENANDODD)
    assert np.array_equal(both[: V // 2], e[: V // 2])
    assert abs(np.mean(both ** 2) - 0.5) < 0.02  # MILC's exp(-x^2) normalisation


def test_oracle_generators_equal_product_generators(lib, oracle_cls):
    """The oracle library compiles the same generator source (mks_synth.h):
    a process that does not load the product library (the CPU reference arm
    of the benchmark) builds bit-identical links, sources and momenta."""
    from oracle import oracle as O
    dims = (4, 6, 4, 8)
    assert np.array_equal(O.gen_thin_links(dims, 11, 0.2), lib.gen_thin_links(dims, 11, 0.2))
    for parity in (lib.EVEN, lib.ODD, lib.EVENANDODD):
        assert np.array_equal(O.gen_vector(dims, 12, parity), lib.gen_vector(dims, 12, parity))
    assert np.array_equal(O.gen_momenta(dims, 13), lib.gen_momenta(dims, 13))
