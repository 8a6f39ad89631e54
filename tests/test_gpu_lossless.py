"""Lossless stage on the device (prodm_lossless_*): the ZCB codec and
AdaptiveLevelCompressor's stopping rule against the oracle.

* every encoder / per-bit fixture level: the device's stopping index equals
  the oracle rule on the oracle codec's sizes, the stored bytes equal the
  oracle's (compressed planes bit for bit, the others raw), and decoding the
  stored planes in two calls gives the raw streams back;
* larger sparse and dense planes, input at an odd byte offset;
* malformed stored streams are rejected.
"""
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
O = oracle.oracle()
HERE = os.path.dirname(os.path.abspath(__file__))


def api():
    from prodm_gb300 import api as a
    return a


def levels():
    out = []
    for name in ("encoders", "perbit"):
        g = np.load(os.path.join(HERE, "golden", name + ".npz"))
        for c in list(g["cases"])[::3]:
            out.append((name, str(c)))
    return out


def expected(blob, sizes, latter):
    offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
    comp = [O.zcb_compress(blob[offs[p]:offs[p + 1]]) for p in range(len(sizes))]
    stop, flags = O.adaptive_stopping(sizes, [c.size for c in comp], latter)
    parts = [comp[p] if flags[p] else blob[offs[p]:offs[p + 1]] for p in range(len(sizes))]
    return stop, flags, np.concatenate(parts) if parts else np.zeros(0, np.uint8), \
        np.array([p.size for p in parts], np.uint32)


@pytest.mark.parametrize("name,case", levels())
@pytest.mark.parametrize("latter", [26, 3])
def test_level_matches_oracle_and_round_trips(name, case, latter):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    blob, sizes = g[case + "_blob"], g[case + "_sizes"]
    stop, flags, stored, ssz = expected(blob, sizes, latter)
    out, osz, dstop = api().compress_level(torch.from_numpy(blob).cuda(), sizes, latter)
    assert dstop == stop
    assert np.array_equal(osz, ssz)
    assert np.array_equal(out.cpu().numpy(), stored)
    B = len(sizes)
    s1 = max(1, B // 2)
    offs = np.concatenate([[0], np.cumsum(osz.astype(np.int64))])
    raw_offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
    for a, b in ((0, s1), (s1, B)):
        raw, rsz = api().decompress_level(out[offs[a]:offs[b]], osz[a:b], a, b - a, dstop, latter,
                                          raw_capacity=int(raw_offs[b] - raw_offs[a]) + 16)
        assert np.array_equal(rsz, sizes[a:b])
        assert np.array_equal(raw.cpu().numpy(), blob[raw_offs[a]:raw_offs[b]])


@pytest.mark.parametrize("n", [1, 4095, 4096, 4097, 3 * 1024 * 1024 + 5])
@pytest.mark.parametrize("offset", [0, 1])
def test_large_planes_and_odd_offsets(n, offset):
    rng = np.random.default_rng(n + offset)
    planes = []
    for dens in (0.0, 0.0005, 0.02, 0.3, 1.0):
        planes.append(((rng.random(n) < dens) * rng.integers(1, 256, n)).astype(np.uint8))
    sizes = np.array([p.size for p in planes], np.uint32)
    blob = np.concatenate(planes)
    stop, flags, stored, ssz = expected(blob, sizes, 26)
    buf = torch.zeros(blob.size + offset, dtype=torch.uint8, device="cuda")
    buf[offset:] = torch.from_numpy(blob).cuda()
    out, osz, dstop = api().compress_level(buf[offset:], sizes, 26)
    assert dstop == stop and np.array_equal(osz, ssz)
    assert np.array_equal(out.cpu().numpy(), stored)
    raw, rsz = api().decompress_level(out, osz, 0, len(sizes), dstop, 26, raw_capacity=blob.size + 16)
    assert np.array_equal(raw.cpu().numpy(), blob)


def test_malformed_streams_rejected():
    from prodm_gb300._lib import ProdmError
    raw = (np.arange(20000) % 7 == 0).astype(np.uint8)
    comp = O.zcb_compress(raw)
    d = torch.from_numpy(comp).cuda()
    with pytest.raises(ProdmError):                       # shorter than its header
        api().decompress_level(d[:8], [8], 0, 1, 5, 26, raw_capacity=30000)
    bad = comp.copy()
    bad[8] = 99                                           # chunk count does not match the length
    with pytest.raises(ProdmError):
        api().decompress_level(torch.from_numpy(bad).cuda(), [bad.size], 0, 1, 5, 26, raw_capacity=30000)
    bad = comp.copy()
    bad[12:16] = 0                                        # first chunk ends before its masks
    with pytest.raises(ProdmError):
        api().decompress_level(torch.from_numpy(bad).cuda(), [bad.size], 0, 1, 5, 26, raw_capacity=30000)
    with pytest.raises(ProdmError):                       # truncated data area
        api().decompress_level(d[:comp.size - 200], [comp.size - 200], 0, 1, 5, 26, raw_capacity=30000)
    raw2, _ = api().decompress_level(d, [comp.size], 0, 1, 5, 26, raw_capacity=30000)
    assert np.array_equal(raw2.cpu().numpy(), raw)


def oracle_stored(res, L, B, latter):
    """per level: raw streams -> (stored bytes, stored sizes, stopping index, flags)"""
    sizes = res["sizes"].reshape(L + 1, B)
    offs = np.concatenate([[0], np.cumsum(sizes.sum(axis=1).astype(np.int64))])
    out = []
    for l in range(L + 1):
        blob = res["blob"][offs[l]:offs[l + 1]]
        out.append(expected(blob, sizes[l], latter))
    return out


CASES = [((65, 65, 65), 3, np.float32, 32, "negabinary", "squared", "negabinary", "l2_hb"),
         ((33, 40, 21), 2, np.float32, 32, "grouped", "max", "sign_exclude", "max_hb"),
         ((17, 17, 17), 3, np.float64, 60, "perbit", "max", "sign_exclude", "max_hb")]


@pytest.mark.parametrize("shape,L,dt,B,enc,col,interp,est", CASES)
def test_handle_with_lossless_stage(shape, L, dt, B, enc, col, interp, est, tmp_path):
    rng = np.random.default_rng(B + L)
    field = (np.cumsum(rng.standard_normal(shape), axis=-1) + 0.05 * rng.standard_normal(shape)).astype(dt)
    tdt = torch.float32 if dt == np.float32 else torch.float64
    m = api().MDRField(shape, tdt, L, B, enc, "hierarchical", col)
    m.refactor(torch.from_numpy(field).cuda())
    raw_sizes, _, _ = m.level_info()
    m.set_lossless(26)
    res = O.refactor(field, L, B, enc, True)
    exp = oracle_stored(res, L, B, 26)
    sizes, _, _ = m.level_info()
    for l in range(L + 1):
        stop, flags, stored, ssz = exp[l]
        assert np.array_equal(sizes[l], ssz), l
        assert np.array_equal(m.export_level(l), stored), l
    meta = m.metadata()
    vr = float(field.max() - field.min())
    norm2 = float((field.astype(np.float64) ** 2).sum())
    tols = [r * r * norm2 for r in (1e-2, 1e-4)] if est == "l2_hb" else [r * vr for r in (1e-2, 1e-4)]
    outs, idxs = [], []
    for tol in tols:
        out = m.retrieve(tol, interpreter=interp, estimator=est)
        idx = m.index()
        ref = O.retrieve(shape, L, B, res["blob"], res["sizes"], res["bounds"], idx, enc, True, dt)
        assert np.array_equal(out.cpu().numpy(), ref)
        outs.append(out.clone())
        idxs.append(idx)
    # the stored files, loaded in two pieces per level, retrieve the same
    files = [m.export_level(l) for l in range(L + 1)]
    r = api().MDRField(shape, tdt, L, B, enc, "hierarchical", col)
    r.load_metadata(meta)
    s2, _, _ = r.level_info()
    assert np.array_equal(s2, sizes)
    for half in (0, 1):
        for l in range(L + 1):
            cut = len(files[l]) // 2
            if half == 0:
                r.load_level(l, files[l][:cut], 0)
            else:
                r.load_level(l, files[l][cut:], cut)
        if half == 0:   # expands the planes complete in the first pieces
            r.retrieve_planes([0] * (L + 1))
    for tol, o, idx in zip(tols, outs, idxs):
        got = r.retrieve(tol, interpreter=interp, estimator=est)
        assert np.array_equal(r.index(), idx)
        assert torch.equal(got, o)
    # off again: the raw sizes are the cost model
    m.set_lossless(None)
    s3, _, _ = m.level_info()
    assert np.array_equal(s3, raw_sizes)


def reference_or_skip():
    """The reference harness with libzstd (it writes the zstd level files)."""
    import importlib
    if importlib.import_module("oracle.build_oracle").zstd_library() is None:
        pytest.skip("no libzstd on this host")
    R = oracle.reference()
    if R is None:
        pytest.skip("the reference harness is not built on this host")
    return R


# shapes the reference's composed classes take (some 2-D and thin shapes
# make them exit or crash, which would end the test process)
REF_ZSTD_CASES = [("negabinary", 26, (65, 65, 65), 3), ("grouped", 20, (33, 40, 21), 2),
                  ("negabinary", 64, (65, 33, 33), 3)]


@pytest.mark.parametrize("enc,latter,shape,L", REF_ZSTD_CASES)
def test_reference_zstd_level_files(enc, latter, shape, L, tmp_path):
    """Level files and metadata written by the reference's ComposedRefactor
    with its zstd stage (AdaptiveLevelCompressor(latter)) load into the
    device handle: the plane counts, retrieved (stored) bytes and
    reconstructions equal the reference ComposedReconstructor's on the same
    files, every bound met; the files go in in consecutive pieces per
    tolerance, as the reference's retriever reads them."""
    R = reference_or_skip()
    B = 32
    rng = np.random.default_rng(latter + L)
    field = (np.cumsum(rng.standard_normal(shape), axis=-1) + 0.05 * rng.standard_normal(shape)).astype(np.float32)
    vr = float(field.max() - field.min())
    tols = [r * vr for r in (1e-2, 1e-4, 1e-6)]
    outs, ret = R.composed_zstd(field, L, B, enc, latter, tols, str(tmp_path))
    meta = (tmp_path / "metadata.bin").read_bytes()
    files = [(tmp_path / ("level_%d.bin" % l)).read_bytes() for l in range(L + 1)]
    m = api().MDRField(shape, torch.float32, L, B, enc, "hierarchical", "max")
    m.set_zstd_latter(latter)
    m.load_metadata(meta)
    stored, _, _ = m.level_info()
    loaded = [0] * (L + 1)
    for t, tol in enumerate(tols):
        m.interpret(tol, interpreter="sign_exclude", estimator="max_hb")
        idx = m.index()
        for l in range(L + 1):
            need = int(stored[l, :idx[l]].astype(np.int64).sum())
            if need > loaded[l]:
                m.load_level(l, np.frombuffer(files[l][loaded[l]:need], np.uint8), loaded[l])
                loaded[l] = need
        assert sum(loaded) == int(ret[t]), (t, sum(loaded), int(ret[t]))
        out = m.reconstruct().cpu().numpy()
        np.testing.assert_allclose(out, outs[t], rtol=0, atol=2e-6 * float(np.abs(field).max()))
        assert float(np.abs(out - field).max()) <= tol


def test_wrong_latter_index_is_reported(tmp_path):
    """zstd files read with a latter index other than the writer's: a plane
    that is not a zstd frame is reported as corrupt (and nothing hangs)."""
    from prodm_gb300._lib import ProdmError
    R = reference_or_skip()
    shape, L, B = (65, 65, 65), 3, 32
    rng = np.random.default_rng(3)
    field = np.cumsum(rng.standard_normal(shape), axis=-1).astype(np.float32)
    R.composed_zstd(field, L, B, "negabinary", 64, [1e-3], str(tmp_path))
    m = api().MDRField(shape, torch.float32, L, B, "negabinary", "hierarchical", "max")
    m.set_zstd_latter(20)   # planes 20.. taken as frames; the writer left them raw
    m.load_metadata((tmp_path / "metadata.bin").read_bytes())
    for l in range(L + 1):
        m.load_level(l, np.frombuffer((tmp_path / ("level_%d.bin" % l)).read_bytes(), np.uint8), 0)
    with pytest.raises(ProdmError):
        m.retrieve_planes([B] * (L + 1))
