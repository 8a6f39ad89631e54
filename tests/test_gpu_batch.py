"""Batched refactor / retrieve against the oracle and against the single-field
device path: the plane counts the oracle interpreter picks from the batch's
sizes and level bounds, reconstructions equal to the oracle's decode ->
reposition -> recompose bit for bit, level bounds within float rounding of the
oracle's decomposition; and the same streams, plane counts and
reconstructions as the single-field path (the batched launches run the same
per-row / per-chunk code)."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_batch_matches_single_field_path():
    from prodm_gb300 import api, fields
    shapes = [(33, 33, 33), (65, 65, 65), (129, 65), (33, 65, 17), (1000,), (9, 9, 9), (257, 129), (33, 1025)]
    xs = [fields.spectral_grf(s, slope=-2.0, seed=i).contiguous() for i, s in enumerate(shapes)]
    levels = [fields.batch_level(s, api.max_level(s)) for s in shapes]
    batch = api.MDRBatch(xs, levels, 32)
    batch.refactor()
    tols = []
    for i, x in enumerate(xs):
        vr = float(x.max() - x.min())
        tols.append(vr * 10.0 ** (-2 - i % 4))
    batch.set_tolerances(tols)
    batch.reset()
    outs = batch.retrieve("negabinary", "max_hb")
    torch.cuda.synchronize()
    for i, (s, x) in enumerate(zip(shapes, xs)):
        one = api.MDRField(s, torch.float32, levels[i], 32, "negabinary", "hierarchical", "max")
        one.refactor(x)
        sz1, b1, _ = one.level_info()
        idxb, szb, bb = batch.field_info(i)
        assert np.array_equal(szb, sz1)
        np.testing.assert_array_equal(bb, b1)
        for l in range(levels[i] + 1):
            assert np.array_equal(batch.export_level(i, l), one.export_level(l)), (i, l)
        out1 = one.retrieve(tols[i], interpreter="negabinary", estimator="max_hb")
        assert np.array_equal(one.index(), idxb)
        assert torch.equal(out1, outs[i]), i
        assert float((outs[i] - x).abs().max()) <= tols[i]


@pytest.mark.parametrize("values,tall", [(256, "1"), (1056, "1"), (4224, "1"), (8192, "1"), (1056, "0"), (4224, "0")])
def test_batch_fused_unit_shapes_match_single_field_path(values, tall, monkeypatch):
    """Every tile shape the autotuner may pick (values per unit of the fused
    finest levels; at 8192 the units of 257-wide rows no longer fit a TMA box
    and take the cp.async kernel) gives the single-field path's
    reconstructions bit for bit, with the planes staged by one tall box per
    unit or (PRODM_TMA_TALL=0) by one box per plane."""
    from prodm_gb300 import api, fields
    monkeypatch.setenv("PRODM_TMA_TALL", tall)
    shapes = [(65, 65, 65), (129, 33), (33, 65, 17), (17, 513), (9, 9, 9), (33, 257)]
    xs = [fields.spectral_grf(s, slope=-2.0, seed=60 + i).contiguous() for i, s in enumerate(shapes)]
    levels = [fields.batch_level(s, api.max_level(s)) for s in shapes]
    batch = api.MDRBatch(xs, levels, 32)
    batch.set_fused_unit(values)
    tols = [float(x.max() - x.min()) * 10.0 ** (-2 - i % 3) for i, x in enumerate(xs)]
    batch.set_tolerances(tols)
    batch.refactor()
    batch.reset()
    outs = batch.retrieve("negabinary", "max_hb")
    torch.cuda.synchronize()
    batch.status()
    for i, (s, x) in enumerate(zip(shapes, xs)):
        one = api.MDRField(s, torch.float32, levels[i], 32, "negabinary", "hierarchical", "max")
        one.refactor(x)
        out1 = one.retrieve(tols[i], interpreter="negabinary", estimator="max_hb")
        assert torch.equal(out1, outs[i]), (values, i)


@pytest.mark.parametrize("ws,min_row", [("1", "257"), ("0", "257"), ("1", "65")])
def test_batch_warp_specialised_fused_levels_match_single_field_path(ws, min_row, monkeypatch):
    """Fused finest levels with rows of 257 values (the warp-specialised
    batched kernel by default, 11-row units, plane counts changing from field
    to field; PRODM_BATCH_WS=0 the 8-warp one) give the single-field path's
    reconstructions bit for bit, next to fields of the other fused classes."""
    from prodm_gb300 import api, fields
    monkeypatch.setenv("PRODM_BATCH_WS", ws)
    monkeypatch.setenv("PRODM_BATCH_WS_MIN_ROW", min_row)   # 65: the 65^3 field too
    shapes = [(33, 33, 257), (17, 65, 257), (65, 65, 65), (9, 9, 9), (40, 33, 257)]
    xs = [fields.spectral_grf(s, slope=-2.0, seed=80 + i).contiguous() for i, s in enumerate(shapes)]
    levels = [fields.batch_level(s, api.max_level(s)) for s in shapes]
    batch = api.MDRBatch(xs, levels, 32)
    tols = [float(x.max() - x.min()) * 10.0 ** (-1 - i % 5) for i, x in enumerate(xs)]
    batch.set_tolerances(tols)
    batch.refactor()
    batch.reset()
    outs = batch.retrieve("negabinary", "max_hb")
    torch.cuda.synchronize()
    batch.status()
    for i, (s, x) in enumerate(zip(shapes, xs)):
        one = api.MDRField(s, torch.float32, levels[i], 32, "negabinary", "hierarchical", "max")
        one.refactor(x)
        out1 = one.retrieve(tols[i], interpreter="negabinary", estimator="max_hb")
        assert torch.equal(out1, outs[i]), (ws, i)


def test_batch_patch_items_match_single_field_path(monkeypatch):
    """The batched decomposition and recomposition with patch work items on
    every 2^k + 1 level (PRODM_PATCH_MIN_ITEMS=1) give the single-field row
    kernels' streams and reconstructions bit for bit."""
    from prodm_gb300 import api, fields
    monkeypatch.setenv("PRODM_PATCH_MIN_ITEMS", "1")
    shapes = [(65, 65, 65), (129, 33), (33, 65, 17), (20, 31, 64)]
    xs = [fields.spectral_grf(s, slope=-2.0, seed=80 + i).contiguous() for i, s in enumerate(shapes)]
    levels = [fields.batch_level(s, api.max_level(s)) for s in shapes]
    batch = api.MDRBatch(xs, levels, 32)
    tols = [float(x.max() - x.min()) * 10.0 ** (-2 - i % 3) for i, x in enumerate(xs)]
    batch.set_tolerances(tols)
    batch.refactor()
    batch.reset()
    outs = [o.clone() for o in batch.retrieve("negabinary", "max_hb")]
    torch.cuda.synchronize()
    monkeypatch.setenv("PRODM_DECOMPOSE_PATCH", "0")
    for i, (s, x) in enumerate(zip(shapes, xs)):
        one = api.MDRField(s, torch.float32, levels[i], 32, "negabinary", "hierarchical", "max")
        one.refactor(x)
        for l in range(levels[i] + 1):
            assert np.array_equal(batch.export_level(i, l), one.export_level(l)), (i, l)
        out1 = one.retrieve(tols[i], interpreter="negabinary", estimator="max_hb")
        assert torch.equal(out1, outs[i]), i


def test_batch_matches_oracle():
    """Each field of a batch checked against the oracle alone (not through the
    single-field path): the oracle interpreter (negabinary look-ahead,
    MaxErrorEstimatorHB on the max-collector tables of the batch's level
    bounds) picks the batch's plane counts; the oracle's retrieval of the
    batch's level streams with those counts equals the batch's output bit for
    bit; the oracle's FP64 decomposition of the field gives the same stream
    sizes and level bounds within 1e-6 of max|x|; every bound is met."""
    import oracle
    from prodm_gb300 import api, fields
    O = oracle.oracle()
    B = 32
    shapes = [(65, 65, 65), (129, 65), (33, 65, 17), (1000,), (9, 9, 9), (40, 33, 21), (17, 1025), (20, 31, 64)]
    xs = [fields.spectral_grf(s, slope=-2.0, seed=40 + i).contiguous() for i, s in enumerate(shapes)]
    levels = [fields.batch_level(s, api.max_level(s)) for s in shapes]
    batch = api.MDRBatch(xs, levels, B)
    batch.refactor()
    tols = [float(x.max() - x.min()) * 10.0 ** (-1 - i % 5) for i, x in enumerate(xs)]
    batch.set_tolerances(tols)
    batch.reset()
    outs = [o.clone() for o in batch.retrieve("negabinary", "max_hb")]
    torch.cuda.synchronize()
    for i, (s, x) in enumerate(zip(shapes, xs)):
        L = levels[i]
        xh = x.cpu().numpy()
        idx, sizes, bounds = batch.field_info(i)
        blob = np.concatenate([batch.export_level(i, l) for l in range(L + 1)])
        errs = np.stack([O.max_collect(np.float32(b), B, np.float32) for b in bounds])
        idx_o, _ = O.interpret("negabinary", "max_hb", sizes, errs, tols[i], np.zeros(L + 1, np.uint8),
                               ndims=len(s))
        assert np.array_equal(idx, idx_o), (i, idx, idx_o)
        rec_o = O.retrieve(s, L, B, blob, sizes, bounds.astype(np.float32), idx, "negabinary", True)
        out = outs[i].cpu().numpy()
        assert np.array_equal(out.view(np.uint32), rec_o.view(np.uint32)), i
        ref = O.refactor(xh, L, B, "negabinary")
        assert np.array_equal(ref["sizes"], sizes), i
        np.testing.assert_allclose(bounds, ref["bounds"], rtol=0, atol=1e-6 * float(np.abs(xh).max()))
        assert float(np.abs(out - xh).max()) <= tols[i]


def test_batch_graph_capture_and_autotune(tmp_path, monkeypatch):
    from prodm_gb300 import api, autotune, fields
    monkeypatch.setenv("PRODM_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    shapes = [(65, 65, 65), (129, 129), (33, 65, 17)]
    xs = [fields.spectral_grf(s, seed=10 + i) for i, s in enumerate(shapes)]
    batch = api.MDRBatch(xs, None, 32)
    tuned, timings = autotune.tune(batch, reps=1)
    for stage, shape in tuned.items():
        if stage == "fused_unit":
            assert shape[0] in autotune.UNIT_CANDIDATES
        else:
            assert shape in autotune.STAGE_CANDIDATES[stage]
    assert len(timings) == sum(len(c) for c in autotune.STAGE_CANDIDATES.values()) + len(autotune.UNIT_CANDIDATES)
    assert autotune.tune(batch)[0] == tuned            # served from the cache
    batch.set_tolerances([1e-3] * 3)
    ref = None
    for capture in (False, True):
        if capture:
            g = torch.cuda.CUDAGraph()
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                batch.refactor(); batch.reset(); batch.retrieve()
            torch.cuda.current_stream().wait_stream(s)
            with torch.cuda.graph(g):
                batch.refactor(); batch.reset(); batch.retrieve()
            g.replay()
            torch.cuda.synchronize()
            for a, b in zip(ref, batch.outs):
                assert torch.equal(a, b)
        else:
            batch.refactor(); batch.reset(); batch.retrieve()
            torch.cuda.synchronize()
            ref = [o.clone() for o in batch.outs]


@pytest.mark.parametrize("tall,ws", [("1", "0"), ("0", "0"), ("1", "1")])
def test_batch_fused_tile_wait_timeout_is_reported_and_recoverable(tall, ws, monkeypatch):
    """The batched TMA fused kernel bounds its waits for plane tiles: with the
    expected byte count raised (the test hook) every wait runs out, the kernel
    reports PRODM_ETIMEOUT through prodm_batch_status (once) and the next
    retrieval equals the one before."""
    from prodm_gb300 import api, fields
    from prodm_gb300._lib import ProdmError
    monkeypatch.setenv("PRODM_TMA_TALL", tall)
    monkeypatch.setenv("PRODM_BATCH_WS", ws)
    shapes = [(65, 65, 65), (129, 129), (33, 65, 17), (33, 33, 257)]
    xs = [fields.spectral_grf(s, seed=20 + i) for i, s in enumerate(shapes)]
    batch = api.MDRBatch(xs, None, 32)
    batch.set_tolerances([float(x.max() - x.min()) * 1e-3 for x in xs])
    batch.refactor()
    batch.reset()
    good = [o.clone() for o in batch.retrieve()]
    batch.status()
    api.debug_tile_wait(64, 20000)
    try:
        batch.reset()
        batch.retrieve()
        with pytest.raises(ProdmError) as e:
            batch.status()
        assert e.value.status == 4          # PRODM_ETIMEOUT
    finally:
        api.debug_tile_wait(0, 0)
    batch.status()                          # reported once
    batch.reset()
    for a, b in zip(batch.retrieve(), good):
        assert torch.equal(a, b)
