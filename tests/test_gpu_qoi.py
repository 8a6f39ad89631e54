"""QoI-bounded retrieval (prodm_gb300.qoi): the reference's uniform-halving
loop against the QoI-guided per-(field, level) budgets, on divergence-free
velocity fields and a lognormal density.

Both must meet the pointwise bound max |Q(V~) - Q(V)| <= tau (checked against
the original fields, and through the rigorous propagated bound); the guided
retrieval must not read more bytes. The level influence used by the guided
bound (forward recomposition of level indicators) must agree with the
per-level norms of the adjoint at a point.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def data(n, kind):
    from prodm_gb300 import fields
    V = [v.cuda() for v in fields.divergence_free_velocity(n, seed=5)]
    if kind == "ke":
        V.append(fields.lognormal_density(n, seed=6).cuda())
    return V


def test_level_influence_matches_adjoint_norms():
    from prodm_gb300 import qoi
    shape, L = (33, 33, 33), 3
    r, off = qoi.level_influence(shape, L)
    rng = np.random.default_rng(0)
    for i in rng.integers(0, int(np.prod(shape)), 12).tolist() + [0, int(np.prod(shape)) - 1]:
        w = qoi.point_level_weights(shape, L, i, off)
        np.testing.assert_allclose(w, r[:, i].cpu().numpy(), rtol=1e-6, atol=1e-7)
    # convex interpolation: every point's influences lie in [0, 1], level 0 reaches all points
    assert float(r.min()) >= 0 and float(r.max()) <= 1 + 1e-6
    assert float(r[0].min()) > 1 - 1e-6


@pytest.mark.parametrize("kind", ["vmag", "ke"])
@pytest.mark.parametrize("rel", [1e-2, 1e-3])
def test_guided_meets_bound_with_fewer_bytes(kind, rel):
    from prodm_gb300 import qoi
    n, L = 65, 3
    x = data(n, kind)
    Vt = [v.double() for v in x[:3]]
    q = qoi.qoi_value(kind, Vt, x[3].double() if kind == "ke" else None)
    tau = qoi.value_range(q) * rel
    base = qoi.halving_retrieve(kind, x, tau, rel, L)
    ours = qoi.guided_retrieve(kind, x, tau, rel, L)
    for res in (base, ours):
        assert res["met"], res
        assert res["bound"] <= tau
        assert res["achieved"] <= res["bound"] * (1 + 1e-6) + 1e-12
    assert ours["bytes"] <= base["bytes"], (ours["bytes"], base["bytes"])


def test_ge_qoi_device_kernels_match_reference_fixtures():
    """prodm_qoi_ge_values / prodm_qoi_ge_bounds against the reference's
    qoi_utils.hpp outputs (tests/golden/qoi.npz): products, quotients and
    square roots bit for bit; PT and mu (the reference takes pow(x, 7) and
    pow(x, 3), the kernel multiplication chains) within 1e-14."""
    import os
    from prodm_gb300 import api
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "qoi.npz"))
    t = {k: torch.from_numpy(g[k]).cuda() for k in ("vx", "vy", "vz", "p", "d")}
    vals = api.qoi_ge_values(t["vx"], t["vy"], t["vz"], t["p"], t["d"])
    for k, v in zip(("vtot", "temp", "c", "mach", "pt", "mu"), vals):
        got = v.cpu().numpy()
        if k in ("pt", "mu"):
            np.testing.assert_allclose(got, g[k], rtol=1e-14, atol=0)
        else:
            assert np.array_equal(got, g[k], equal_nan=True), k
    bv, bt, mx = api.qoi_ge_bounds([t["vx"], t["vy"], t["vz"]], g["ebs_v"], t["p"], t["d"], *g["eb_pd"])
    assert np.array_equal(bv.cpu().numpy(), g["bound_vtot"])
    assert np.array_equal(bt.cpu().numpy(), g["bound_t"])
    m = mx.cpu().numpy()
    assert m[0] == g["bound_vtot"].max() and m[1] == g["bound_t"].max()
    # one QoI at a time; invalid requests raise
    bv2, bt2, _ = api.qoi_ge_bounds([t["vx"], t["vy"], t["vz"]], g["ebs_v"])
    assert bt2 is None and torch.equal(bv2, bv)
    from prodm_gb300._lib import ProdmError
    with pytest.raises(ProdmError):
        api.qoi_ge_bounds([t["vx"], t["vy"], t["vz"]], (-1.0, 0.0, 0.0))
