"""Level files on disk (prodm_mdr_write_level_file / prodm_mdr_load_level_file):
the files are the exported level bytes, and a handle fed by byte ranges of
them (two ranges per level, through cuFile or pinned staging) retrieves what
the device-resident handle retrieves; with the lossless stage too; a level
larger than the staging chunk; missing files and short reads are errors."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def api():
    from prodm_gb300 import api as a
    return a


CASES = [((65, 65, 65), 3, torch.float32, 32, "negabinary", "squared", "negabinary", "l2_hb", None),
         ((33, 40, 21), 2, torch.float32, 32, "grouped", "max", "sign_exclude", "max_hb", None),
         ((17, 17, 17), 3, torch.float64, 60, "perbit", "max", "sign_exclude", "max_hb", None),
         ((65, 65, 65), 3, torch.float32, 32, "negabinary", "squared", "negabinary", "l2_hb", 26),
         ((33, 40, 21), 2, torch.float32, 32, "grouped", "max", "sign_exclude", "max_hb", 26),
         ((257, 257, 257), 6, torch.float32, 32, "negabinary", "max", "negabinary", "max_hb", None)]


@pytest.mark.parametrize("shape,L,dt,B,enc,col,interp,est,latter", CASES)
def test_level_files_round_trip(shape, L, dt, B, enc, col, interp, est, latter, tmp_path):
    from prodm_gb300 import fields
    x = fields.spectral_grf(shape, seed=L + B, dtype=dt, device="cuda")
    m = api().MDRField(shape, dt, L, B, enc, "hierarchical", col)
    m.refactor(x)
    if latter is not None:
        m.set_lossless(latter)
    for l in range(L + 1):
        m.write_level_file(l, tmp_path / ("level_%d.bin" % l))
        assert (tmp_path / ("level_%d.bin" % l)).read_bytes() == m.export_level(l).tobytes(), l
    r = api().MDRField(shape, dt, L, B, enc, "hierarchical", col)
    r.load_metadata(m.metadata())
    assert r.file_read_mode() == -1
    for l in range(L + 1):
        f = tmp_path / ("level_%d.bin" % l)
        n = f.stat().st_size
        cut = n // 3
        r.load_level_file(l, f, 0, 0, cut)
        r.load_level_file(l, f, cut, cut, n - cut)
    assert r.file_read_mode() in (0, 1)
    if est == "l2_hb":
        norm2 = float((x.double() ** 2).sum())
        tols = [rel * rel * norm2 for rel in (1e-2, 1e-4)]
    else:
        vr = float(x.max() - x.min())
        tols = [rel * vr for rel in (1e-2, 1e-4)]
    for tol in tols:
        a = m.retrieve(tol, interpreter=interp, estimator=est)
        b = r.retrieve(tol, interpreter=interp, estimator=est)
        assert np.array_equal(m.index(), r.index())
        assert torch.equal(a, b)


@pytest.mark.parametrize("enc,dt,B,latter", [("negabinary", torch.float32, 32, None),
                                              ("grouped", torch.float32, 32, None),
                                              ("perbit", torch.float64, 60, None),
                                              ("grouped", torch.float32, 32, 26)])
def test_export_into_pinned_on_a_side_stream(enc, dt, B, latter):
    """exports into pinned memory are stream-ordered: issued finest level
    first on a second stream, each is the level file once its event is done;
    device exports and a refactor with other data invalidate nothing stale"""
    from prodm_gb300 import fields
    shape, L = (45, 38, 29), 3
    m = api().MDRField(shape, dt, L, B, enc, "hierarchical", "max")
    for seed in (1, 2):
        x = fields.spectral_grf(shape, seed=seed, dtype=dt, device="cuda")
        m.refactor(x)
        if latter is not None:
            m.set_lossless(latter)
        want = [m.export_level(l) for l in range(L + 1)]
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        outs, evs = [None] * (L + 1), [None] * (L + 1)
        for l in reversed(range(L + 1)):
            outs[l] = torch.empty(len(want[l]) + 3, dtype=torch.uint8, pin_memory=True)
            assert m.export_level_into(l, outs[l], side) == len(want[l])
            evs[l] = torch.cuda.Event()
            evs[l].record(side)
        for l in range(L + 1):
            evs[l].synchronize()
            assert outs[l][:len(want[l])].numpy().tobytes() == want[l].tobytes(), (seed, l)
            d = torch.empty(len(want[l]), dtype=torch.uint8, device="cuda")
            assert m.export_level_into(l, d) == len(want[l])
            assert d.cpu().numpy().tobytes() == want[l].tobytes(), (seed, l)
    with pytest.raises(ValueError):
        m.export_level_into(0, torch.empty(16, dtype=torch.uint8))      # pageable


@pytest.mark.parametrize("enc,dt,B,latter", [("negabinary", torch.float32, 32, None),
                                              ("grouped", torch.float32, 32, None),
                                              ("perbit", torch.float64, 60, None),
                                              ("negabinary", torch.float32, 32, 26)])
def test_export_level_ranges(enc, dt, B, latter):
    """byte ranges of a level file (prodm_mdr_export_level_range) equal the
    same bytes of the whole export: ranges inside one plane row, across rows,
    on row boundaries, empty and whole, into device and pinned host memory;
    ranges past the end are errors"""
    from prodm_gb300 import fields
    from prodm_gb300._lib import ProdmError
    shape, L = (45, 38, 29), 3
    m = api().MDRField(shape, dt, L, B, enc, "hierarchical", "max")
    m.refactor(fields.spectral_grf(shape, seed=5, dtype=dt, device="cuda"))
    if latter is not None:
        m.set_lossless(latter)
    rng = np.random.default_rng(B)
    for l in range(L + 1):
        want = m.export_level(l)
        n = len(want)
        row = n // B
        cuts = [(0, n), (0, 0), (n, 0), (0, 1), (n - 1, 1), (1, n - 2)]      # (offset, length)
        if row:
            cuts += [(row, row), (row - 1, 2), (row // 2, 3 * row), (2 * row + 3, row - 3)]
        for _ in range(6):
            a, b = sorted(int(v) for v in rng.integers(0, n + 1, 2))
            cuts.append((a, b - a))
        for a, nb in cuts:
            a = min(max(a, 0), n)
            nb = min(max(nb, 0), n - a)
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            h = torch.empty(nb, dtype=torch.uint8, pin_memory=True)
            m.export_level_range_into(l, a, h, side)
            side.synchronize()
            assert h.numpy().tobytes() == want[a:a + nb].tobytes(), (l, a, nb)
            d = torch.empty(nb, dtype=torch.uint8, device="cuda")
            m.export_level_range_into(l, a, d)
            assert d.cpu().numpy().tobytes() == want[a:a + nb].tobytes(), (l, a, nb)
        with pytest.raises(ProdmError):
            m.export_level_range_into(l, n - 2, torch.empty(3, dtype=torch.uint8, device="cuda"))


def test_file_errors(tmp_path):
    from prodm_gb300._lib import ProdmError
    shape = (33, 33, 33)
    x = torch.randn(shape, device="cuda")
    m = api().MDRField(shape, torch.float32, 2, 32, "negabinary", "hierarchical", "max")
    m.refactor(x)
    m.write_level_file(2, tmp_path / "l2.bin")
    r = api().MDRField(shape, torch.float32, 2, 32, "negabinary", "hierarchical", "max")
    with pytest.raises(ProdmError):                     # metadata first
        r.load_level_file(2, tmp_path / "l2.bin")
    r.load_metadata(m.metadata())
    with pytest.raises(ProdmError):                     # no such file
        r.load_level_file(2, tmp_path / "missing.bin", 0, 0, 100)
    n = (tmp_path / "l2.bin").stat().st_size
    with pytest.raises(ProdmError):                     # past the end of the file
        r.load_level_file(2, tmp_path / "l2.bin", 0, 0, n + 64)
