"""The oracle's HISQ force against central finite differences of
S_lin(U) = 2 Re sum_j res_j X_j^dag D_eo[links(U)] Y_j, whose derivative at
fixed X, Y is exactly the force (random su(3) directions, eps = 1e-5)."""
import numpy as np
import pytest

scipy_linalg = pytest.importorskip("scipy.linalg")


def _unc(mm):
    A = np.zeros((3, 3), complex)
    A[0, 1] = mm[0] + 1j * mm[1]; A[0, 2] = mm[2] + 1j * mm[3]; A[1, 2] = mm[4] + 1j * mm[5]
    A[1, 0] = -np.conj(A[0, 1]); A[2, 0] = -np.conj(A[0, 2]); A[2, 1] = -np.conj(A[1, 2])
    A[0, 0] = 1j * mm[6]; A[1, 1] = 1j * mm[7]; A[2, 2] = 1j * mm[8]
    return A


@pytest.mark.parametrize("eps_naik,orders", [((0.0,), [2]), ((0.0, -0.2), [1, 1])])
def test_force_finite_differences(lib, oracle_cls, eps_naik, orders):
    dims = (4, 4, 4, 6)
    V = int(np.prod(dims))
    U = lib.apply_phases(dims, lib.gen_thin_links(dims, 3, 0.3))
    orc = oracle_cls(dims)
    res = [0.3, 0.7]
    xxx = np.stack([lib.gen_vector(dims, 10 + j, lib.EVENANDODD) for j in range(2)])
    # mom = TA(2 eps U K_U) with eps = 1: tr(mom A) = 2 Re tr(U K_U A) = dS/dt
    P = orc.fermion_force_hisq(U, 1.0, res, xxx, orders=orders, eps_naik=eps_naik)
    rng = np.random.default_rng(7)
    for _ in range(10):
        x, mu = int(rng.integers(V)), int(rng.integers(4))
        H = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        A = (H - H.conj().T) / 2
        A -= np.trace(A) / 3 * np.eye(3)

        def S(t):
            U2 = U.copy()
            M = U2[x, mu].reshape(3, 3, 2)
            Mc = scipy_linalg.expm(t * A) @ (M[..., 0] + 1j * M[..., 1])
            U2[x, mu] = np.stack([Mc.real, Mc.imag], -1).reshape(18)
            return orc.force_action(U2, res, xxx, orders=orders, eps_naik=eps_naik)

        h = 1e-5
        fd = (S(h) - S(-h)) / (2 * h)
        an = np.trace(_unc(P[x, mu]) @ A).real
        assert abs(fd - an) <= 1e-7 * max(1.0, abs(an)), (x, mu, fd, an)
