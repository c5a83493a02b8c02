"""The force as a forward/backward pair through the C ABI, wrapped in a
torch.autograd.Function (test harness only).

forward:  S(U) = 2 Re sum_j res_j X_j^dag D_eo[links(U)] Y_j, with the links
          built on the GPU from the thin links U (mks_load_links_from_thin)
          and D_eo applied on the GPU (mks_dslash_fn_field);
backward: dS/dU from mks_fermion_force_adjoint.
Checked along random su(3) directions U(t) = exp(t A) U against central
finite differences of the forward (h = 1e-5), and the adjoint against the
projected update of the force entry points."""
import numpy as np
import pytest

from conftest import rel

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 8)


def _real18(c):
    return torch.view_as_real(c.reshape(c.shape[:-2] + (9,))).reshape(c.shape[:-2] + (18,))


def _cmat(r):
    return torch.view_as_complex(r.reshape(r.shape[:-1] + (9, 2)).contiguous()).reshape(r.shape[:-1] + (3, 3))


def make_function(m, action, eps_naik, orders, u0=1.0):
    Vh = int(np.prod(DIMS)) // 2

    def load(U):
        if action == "hisq":
            m.load_hisq_links(U, eps_naik)
        else:
            m.load_asqtad_links(U, u0)

    def slot_of(j):
        g, acc = 0, orders[0]
        while j >= acc and g + 1 < len(orders):
            g += 1
            acc += orders[g]
        return g

    class Bilinear(torch.autograd.Function):
        @staticmethod
        def forward(ctx, U, xxx, res):
            Un = np.ascontiguousarray(U.detach().numpy())
            load(Un)
            S = 0.0
            for j, x in enumerate(xxx):
                Y = x.copy()
                Y[:Vh] = 0.0
                D = m.dslash_fn_field(Y, np.zeros_like(x), m.EVEN, slot_of(j))
                S += 2.0 * res[j] * float(np.dot(x[:Vh].ravel(), D[:Vh].ravel()))
            ctx.save_for_backward(U)
            ctx.xxx, ctx.res = xxx, res
            return torch.tensor(S, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            (U,) = ctx.saved_tensors
            load(np.ascontiguousarray(U.detach().numpy()))
            K = m.fermion_force_adjoint(ctx.res, ctx.xxx, list(orders) if action == "hisq" else None,
                                        len(orders) if action == "hisq" else 1)
            # dS = 2 Re tr(K dU): the gradient w.r.t. (Re U, Im U) is 2 K^dag
            Kc = _cmat(torch.from_numpy(K))
            G = _real18(2.0 * Kc.conj().transpose(-1, -2))
            return g * G, None, None

    return Bilinear


def _su3_direction(gen, shape):
    A = torch.complex(torch.from_numpy(gen.normal(size=shape + (3, 3))),
                      torch.from_numpy(gen.normal(size=shape + (3, 3))))
    A = 0.5 * (A - A.conj().transpose(-1, -2))
    tr = torch.diagonal(A, dim1=-2, dim2=-1).sum(-1) / 3.0
    return A - tr[..., None, None] * torch.eye(3, dtype=A.dtype)


@pytest.mark.parametrize("action,eps_naik,orders", [("hisq", (0.0,), (3,)), ("hisq", (0.0, -0.1), (2, 1)),
                                                    ("asqtad", (0.0,), (3,))])
def test_autograd_directional_derivative(gpu, action, eps_naik, orders):
    m = gpu
    m.set_lattice(DIMS)
    U0 = m.apply_phases(DIMS, m.gen_thin_links(DIMS, 71, 0.3))
    xxx = [m.gen_vector(DIMS, 72 + j, m.EVENANDODD) for j in range(3)]
    res = [0.3, 0.6, 0.9]
    F = make_function(m, action, eps_naik, orders, u0=0.9)
    Uc = _cmat(torch.from_numpy(U0))
    gen = np.random.default_rng(73)
    h = 1e-5
    for _ in range(20 if action == "hisq" and len(orders) == 1 else 6):
        A = _su3_direction(gen, tuple(Uc.shape[:-2]))

        def S_at(t):
            return F.apply(_real18(torch.matrix_exp(t * A) @ Uc), xxx, res)

        t = torch.zeros((), dtype=torch.float64, requires_grad=True)
        S = S_at(t.to(torch.complex128))
        S.backward()
        with torch.no_grad():
            fd = (S_at(torch.tensor(h, dtype=torch.complex128)) - S_at(torch.tensor(-h, dtype=torch.complex128))) / (2 * h)
        assert abs(t.grad.item() - fd.item()) <= 1e-6 * max(1.0, abs(fd.item())), (t.grad.item(), fd.item())


def test_adjoint_matches_projected_force(gpu):
    m = gpu
    m.set_lattice(DIMS)
    U = m.apply_phases(DIMS, m.gen_thin_links(DIMS, 81, 0.3))
    m.load_hisq_links(U, (0.0, -0.1))
    xxx = [m.gen_vector(DIMS, 82 + j, m.EVENANDODD) for j in range(3)]
    res, orders, eps = [0.2, 0.5, 0.9], [2, 1], 0.07
    K = m.fermion_force_adjoint(res, xxx, orders, 2)
    mom = np.zeros((U.shape[0], 4, 10))
    m.eo_fermion_force_multi(eps, res, xxx, mom, n_orders_naik=orders, n_naiks=2)
    G = _cmat(torch.from_numpy(U)) @ _cmat(torch.from_numpy(K)) * (2.0 * eps)
    G = 0.5 * (G - G.conj().transpose(-1, -2))
    tr = torch.diagonal(G, dim1=-2, dim2=-1).sum(-1) / 3.0
    G = (G - tr[..., None, None] * torch.eye(3, dtype=G.dtype)).numpy()
    assert rel(G[..., 0, 1].real, mom[..., 0]) < 1e-13
    assert rel(G[..., 1, 2].imag, mom[..., 5]) < 1e-13
    assert rel(G[..., 2, 2].imag, mom[..., 8]) < 1e-12
