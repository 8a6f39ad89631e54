"""Full-size workloads on the device, checked through size-independent
properties (the oracle would take hours at these sizes):

* 1025 x 1025 x 513 fp64 tanh shear layer + 1e-6 relative noise, 9 levels,
  60 planes, grouped encoder, orthogonal basis, L-inf retrieval at relative
  bounds 1e-3 .. 1e-9 of the value range: every retrieval meets its bound,
  the plane counts only grow, and all planes are at least as close as the
  tightest bound.
* 513^3 fp32 Gaussian random field, 8 levels, 32 planes, negabinary encoder,
  squared-error tables, relative L2 bounds 1e-2 .. 1e-6: every retrieval
  meets its bound.
"""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_fp64_shear_layer_1025x1025x513_linf():
    from prodm_gb300 import api, fields
    shape, L, B = (1025, 1025, 513), 8, 60
    x = fields.shear_layer(shape, delta=0.05, noise_rel=1e-6, seed=9, dtype=torch.float64, device="cuda")
    vr = float(x.max() - x.min())
    mdr = api.MDRField(shape, torch.float64, L, B, "grouped", "orthogonal", "max")
    mdr.refactor(x)
    out = torch.empty_like(x)
    prev = np.zeros(L + 1, np.int64)
    for rel in (1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9):
        tol = rel * vr
        mdr.retrieve(tol, out=out, interpreter="sign_exclude", estimator="max_ob")
        err = float((out - x).abs().max())
        idx = mdr.index().astype(np.int64)
        assert np.all(idx >= prev)
        prev = idx
        print("rel %.0e  max error %.3e  bound %.3e  planes %s" % (rel, err, tol, idx.tolist()))
        assert err <= tol, (rel, err, tol)
    # all planes: at least as close as the tightest bound
    full = mdr.retrieve_planes([B] * (L + 1))
    assert float((full - x).abs().max()) <= 1e-9 * vr
    del mdr, x, out, full
    torch.cuda.empty_cache()


def test_fp32_grf_513_l2():
    from prodm_gb300 import api, fields
    shape, L, B = (513, 513, 513), 7, 32
    x = fields.spectral_grf(shape, slope=-5.0 / 3.0, seed=1234, device="cuda")
    norm2 = float((x.double() ** 2).sum())
    mdr = api.MDRField(shape, torch.float32, L, B, "negabinary", "hierarchical", "squared")
    mdr.refactor(x)
    out = torch.empty_like(x)
    for rel in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
        tol = rel * rel * norm2
        mdr.retrieve(tol, out=out, interpreter="negabinary", estimator="l2_hb")
        achieved = float(((out.double() - x.double()) ** 2).sum())
        print("rel %.0e  achieved rel L2 %.3e" % (rel, math.sqrt(achieved / norm2)))
        assert achieved <= tol, (rel, achieved, tol)
    del mdr, x, out
    torch.cuda.empty_cache()
