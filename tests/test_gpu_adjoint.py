"""Adjoint recomposition (prodm_recompose_adjoint) and its forward pair
(prodm_recompose_packed), hierarchical basis; the orthogonal basis through
the _basis entry points (forward against the FP64 oracle, adjoint by the
dot-product test).

* forward: equal to the oracle's reposition + recompose (bit for bit in both
  precisions: the same uncontracted operations);
* adjoint: equal to the oracle's reverse-mode restatement (scatter form, FP64)
  and satisfying <R c, g> = <c, R^T g>;
* gradient of a quantity of interest with respect to the level coefficients,
  through a torch.autograd.Function defined here (test harness only):
  against central finite differences (eps = 1e-3, FP64 on the host with the
  oracle's recomposition) and against the FP64 host gradient.
"""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
O = oracle.oracle()

SHAPES = [((65, 65, 65), 3), ((17, 9, 33), 2), ((40, 33, 21), 2), ((100,), 5), ((33, 64), 4), ((12, 10, 7), 1),
          ((16, 16, 16), 2), ((9, 9, 9), 0)]


def api():
    from prodm_gb300 import api as a
    return a


@pytest.mark.parametrize("shape,L", SHAPES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_forward_matches_oracle(shape, L, dt):
    rng = np.random.default_rng(len(shape) * 7 + L)
    c = rng.standard_normal(int(np.prod(shape))).astype(dt)
    got = api().recompose_packed(torch.from_numpy(c).cuda(), shape, L).cpu().numpy()
    ref = O.recompose_packed(c, shape, L)
    assert np.array_equal(got.view(np.uint8), ref.view(np.uint8))


@pytest.mark.parametrize("shape,L", SHAPES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_adjoint_matches_oracle_and_dot_product(shape, L, dt):
    rng = np.random.default_rng(len(shape) * 11 + L)
    g = rng.standard_normal(shape).astype(dt)
    got = api().recompose_adjoint(torch.from_numpy(g).cuda(), L).cpu().numpy()
    ref = O.recompose_adjoint(g.astype(np.float64), shape, L)
    tol = (1e-6 if dt == np.float32 else 1e-13) * float(np.abs(ref).max())
    assert np.max(np.abs(got.astype(np.float64) - ref)) <= tol
    if dt == np.float64:
        c = rng.standard_normal(int(np.prod(shape)))
        f = api().recompose_packed(torch.from_numpy(c).cuda(), shape, L).cpu().numpy()
        lhs, rhs = float(np.sum(f * g)), float(np.sum(c * got))
        assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + float(np.sum(np.abs(f * g))))


ORTH_SHAPES = [((65, 65, 65), 3), ((17, 9, 33), 2), ((40, 33, 21), 2), ((100,), 5), ((33, 64), 4), ((12, 10, 7), 1),
               ((9, 9, 9), 0), ((6, 20, 9), 1), ((33, 17, 5), 1)]


@pytest.mark.parametrize("shape,L", ORTH_SHAPES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_orthogonal_forward_matches_oracle(shape, L, dt):
    """Orthogonal basis: the packed recomposition (each level's L2 correction
    removed from its coarse box, then the interpolation) against the FP64
    oracle's recomposition of the same packed coefficients."""
    rng = np.random.default_rng(len(shape) * 5 + L)
    c = rng.standard_normal(int(np.prod(shape))).astype(dt)
    got = api().recompose_packed(torch.from_numpy(c).cuda(), shape, L, basis="orthogonal").cpu().numpy()
    ref = O.recompose_packed(c.astype(np.float64), shape, L, False)
    tol = (2e-5 if dt == np.float32 else 1e-12) * float(np.abs(ref).max())
    assert np.max(np.abs(got.astype(np.float64) - ref)) <= tol


@pytest.mark.parametrize("shape,L", ORTH_SHAPES)
def test_orthogonal_adjoint_dot_product(shape, L):
    """<R c, g> = <c, R^T g> for the orthogonal recomposition (FP64), and the
    fp32 adjoint within float rounding of the FP64 one."""
    rng = np.random.default_rng(len(shape) * 13 + L)
    g = rng.standard_normal(shape)
    c = rng.standard_normal(int(np.prod(shape)))
    f = api().recompose_packed(torch.from_numpy(c).cuda(), shape, L, basis="orthogonal").cpu().numpy()
    gc = api().recompose_adjoint(torch.from_numpy(g).cuda(), L, basis="orthogonal").cpu().numpy()
    lhs, rhs = float(np.sum(f * g)), float(np.sum(c * gc))
    assert abs(lhs - rhs) <= 1e-11 * (float(np.sum(np.abs(f * g))) + float(np.sum(np.abs(c * gc))))
    g32 = api().recompose_adjoint(torch.from_numpy(g.astype(np.float32)).cuda(), L, basis="orthogonal").cpu().numpy()
    assert np.max(np.abs(g32.astype(np.float64) - gc)) <= 2e-5 * float(np.abs(gc).max())
    if L > 0:   # the correction's share is not zero: the hierarchical transpose differs
        gh = api().recompose_adjoint(torch.from_numpy(g).cuda(), L).cpu().numpy()
        assert np.max(np.abs(gh - gc)) > 1e-6 * float(np.abs(gc).max())


class Recompose(torch.autograd.Function):
    """packed level coefficients -> field, with the adjoint kernel as backward"""

    @staticmethod
    def forward(ctx, coef, shape, L):
        ctx.L = L
        return api().recompose_packed(coef, shape, L)

    @staticmethod
    def backward(ctx, grad):
        return api().recompose_adjoint(grad.contiguous(), ctx.L), None, None


def qoi(kind, V, rho):
    vv = V[0] * V[0] + V[1] * V[1] + V[2] * V[2]
    if kind == "vmag":
        return vv.sqrt().sum()
    return (0.5 * rho * vv).sum()


def host_qoi_and_grad(kind, V, rho):
    vv = V[0] ** 2 + V[1] ** 2 + V[2] ** 2
    if kind == "vmag":
        m = np.sqrt(vv)
        return float(m.sum()), [V[i] / m for i in range(3)], None
    return float((0.5 * rho * vv).sum()), [rho * V[i] for i in range(3)], 0.5 * vv


@pytest.mark.parametrize("kind", ["vmag", "ke"])
def test_qoi_gradient_vs_finite_differences_and_fp64_host(kind):
    from prodm_gb300 import fields
    n, L = 65, 3
    shape = (n, n, n)
    vel = fields.divergence_free_velocity(n, seed=3, dtype=torch.float64)
    rho = fields.lognormal_density(n, seed=4, dtype=torch.float64)
    # packed level coefficients of each field (device decomposition)
    coefs = []
    for f in vel + [rho]:
        m = api().MDRField(shape, torch.float64, L, 60, "grouped", "hierarchical", "max")
        m.refactor(f.cuda().contiguous())
        coefs.append(m.coefficients().clone())
    c = [x.clone().requires_grad_(True) for x in coefs]
    V = [Recompose.apply(c[i], shape, L) for i in range(3)]
    R = Recompose.apply(c[3], shape, L)
    J = qoi(kind, V, R)
    J.backward()
    grads = [x.grad.cpu().numpy() if x.grad is not None else np.zeros(x.numel()) for x in c]

    # FP64 host gradient: pointwise dQ/dV on the host, oracle adjoint
    hc = [x.detach().cpu().numpy() for x in coefs]
    hV = [O.recompose_packed(hc[i], shape, L) for i in range(3)]
    hR = O.recompose_packed(hc[3], shape, L)
    Jh, gV, gR = host_qoi_and_grad(kind, hV, hR)
    assert abs(Jh - float(J.detach())) <= 1e-12 * abs(Jh)
    host = [O.recompose_adjoint(gV[i], shape, L) for i in range(3)]
    host.append(O.recompose_adjoint(gR, shape, L) if gR is not None else np.zeros_like(hc[3]))
    for f in range(4):
        scale = float(np.abs(host[f]).max()) + 1e-300
        assert np.max(np.abs(grads[f] - host[f])) <= 1e-12 * scale, f

    # central differences, eps = 1e-3, FP64 host evaluation
    eps = 1e-3
    rng = np.random.default_rng(7)
    offs = np.concatenate([[0], np.cumsum(O.level_elements(shape, L).astype(np.int64))])
    fields_to_check = range(4) if kind == "ke" else range(3)
    for f in fields_to_check:
        for l in range(L + 1):
            for j in rng.integers(offs[l], offs[l + 1], 3):
                vals = []
                for sgn in (1.0, -1.0):
                    cc = [x.copy() for x in hc]
                    cc[f][j] += sgn * eps
                    Vp = [O.recompose_packed(cc[i], shape, L) for i in range(3)]
                    Rp = O.recompose_packed(cc[3], shape, L)
                    vals.append(host_qoi_and_grad(kind, Vp, Rp)[0])
                fd = (vals[0] - vals[1]) / (2 * eps)
                an = grads[f][j]
                assert abs(fd - an) <= 1e-5 * max(abs(an), 1e-3 * float(np.abs(grads[f]).max())), (f, l, j, fd, an)
