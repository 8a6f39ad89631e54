"""Device-resident refactor / retrieve (MDRField) against the oracle.

* coefficients: within 1e-6 (fp32) / 1e-13 (fp64) of max|x| against the FP64
  oracle decomposition, in the interleaved level order;
* streams: the exported level files are bit-exact with the oracle encoder fed
  the GPU's own coefficients (the oracle encoder is pinned to the reference);
* squared-error tables: within 1e-12 of the oracle's (the reference's
  per-value double sums) on the GPU's coefficients (n * 2^-53 for levels of n
  values, the rounding of the oracle's sequential sum), bitwise reproducible;
* retrieval: the same plane counts as the oracle interpreter on the same
  tables, and on the tables the oracle computes itself from the GPU's
  coefficients; reconstruction within float rounding of the oracle's, and the
  achieved error within the requested bound.
"""
import math

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
O = oracle.oracle()


def api():
    from prodm_gb300 import api as a
    return a


def fields():
    from prodm_gb300 import fields as f
    return f


def oracle_levels(coef_nat, shape, L):
    """level buffers from an in-place decomposed array (oracle interleaver)."""
    ld = O.level_dims(shape, L)
    out = []
    for l in range(L + 1):
        coarse = ld[l - 1] if l else np.zeros(len(shape), np.uint32)
        out.append(O.interleave(coef_nat, shape, ld[l], coarse))
    return out


CASES = [
    ((33, 33, 33), 3, "grouped", "hierarchical", np.float32),
    ((65, 65, 65), 3, "negabinary", "hierarchical", np.float32),
    ((65, 65, 65), 3, "grouped", "orthogonal", np.float32),
    ((40, 33, 21), 2, "negabinary", "orthogonal", np.float32),
    ((129, 65), 5, "grouped", "hierarchical", np.float32),
    ((1000,), 6, "negabinary", "hierarchical", np.float32),
    ((33, 33, 33), 3, "grouped", "orthogonal", np.float64),
    ((17, 9, 33), 2, "negabinary", "hierarchical", np.float64),
    ((9, 9, 9), 2, "negabinary", "hierarchical", np.float32),     # level 0 = 27 values < one block
    ((16, 16, 16), 0, "grouped", "hierarchical", np.float32),     # no decomposition
]


@pytest.mark.parametrize("shape,L,enc,basis,dt", CASES)
def test_refactor_matches_oracle(shape, L, enc, basis, dt):
    B = 32 if dt == np.float32 else 60
    tdt = torch.float32 if dt == np.float32 else torch.float64
    x = fields().sinusoids(shape, seed=len(shape) + L, dtype=tdt).cpu().numpy()
    mdr = api().MDRField(shape, tdt, L, B, enc, basis, "squared")
    mdr.refactor(torch.from_numpy(x).cuda())
    coef = mdr.coefficients().cpu().numpy()
    ref_nat = O.decompose(x.astype(np.float64), shape, L, basis == "hierarchical")
    ref_levels = oracle_levels(ref_nat, shape, L)
    offs = np.concatenate([[0], np.cumsum(mdr.level_elements.astype(np.int64))])
    tol = (1e-6 if dt == np.float32 else 1e-13) * float(np.abs(x).max())
    sizes, bounds, errs = mdr.level_info()
    for l in range(L + 1):
        got = coef[offs[l]:offs[l + 1]]
        assert np.max(np.abs(got.astype(np.float64) - ref_levels[l])) <= tol, l
        # the streams of the GPU coefficients are what the oracle encoder makes of them
        mx = O.max_abs(got)
        assert bounds[l] == (float(mx) * 4 if enc == "negabinary" else float(mx))
        e = math.frexp(float(mx))[1]
        ob, osz, oerr = O.encode(enc, got, e, B, dt == np.float32)
        assert np.array_equal(sizes[l], osz)
        assert np.array_equal(mdr.export_level(l), ob), l
        if dt == np.float32:
            np.testing.assert_allclose(errs[l], oerr, rtol=1e-12, atol=0)


@pytest.mark.parametrize("enc", ["grouped", "negabinary"])
@pytest.mark.parametrize("basis", ["hierarchical", "orthogonal"])
def test_progressive_retrieve_linf(enc, basis):
    shape, L, B = (65, 65, 65), 3, 32
    x = fields().sinusoids(shape, seed=11).cpu().numpy()
    mdr = api().MDRField(shape, torch.float32, L, B, enc, basis, "max")
    mdr.refactor(torch.from_numpy(x).cuda())
    sizes, bounds, _ = mdr.level_info()
    blob = np.concatenate([mdr.export_level(l) for l in range(L + 1)])
    vr = float(x.max() - x.min())
    est = "max_hb" if basis == "hierarchical" else "max_ob"
    idx_o = np.zeros(L + 1, np.uint8)
    for rel in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
        tol = rel * vr
        out = mdr.retrieve(tol, interpreter="sign_exclude", estimator=est).cpu().numpy()
        idx = mdr.index()
        errs = np.stack([O.max_collect(np.float32(b), B, np.float32) for b in bounds])
        idx_o, _ = O.interpret("sign_exclude", est, sizes, errs, tol, idx_o, ndims=3)
        assert np.array_equal(idx, idx_o)
        rec_o = O.retrieve(shape, L, B, blob, sizes, bounds.astype(np.float32), idx, enc, basis == "hierarchical")
        np.testing.assert_allclose(out, rec_o, rtol=0, atol=2e-6 * float(np.abs(x).max()))
        assert float(np.abs(out - x).max()) <= tol


def test_l2_retrieve_meets_bound_and_matches_interpreter():
    shape, L, B = (65, 65, 65), 3, 32
    x = fields().spectral_grf(shape, seed=5).cpu().numpy()
    mdr = api().MDRField(shape, torch.float32, L, B, "negabinary", "hierarchical", "squared")
    mdr.refactor(torch.from_numpy(x).cuda())
    sizes, bounds, errs = mdr.level_info()
    norm2 = float(np.sum(x.astype(np.float64) ** 2))
    idx_o = np.zeros(L + 1, np.uint8)
    for rel in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
        tol = (rel ** 2) * norm2
        out = mdr.retrieve(tol, interpreter="negabinary", estimator="l2_hb").cpu().numpy()
        idx = mdr.index()
        idx_o, _ = O.interpret("negabinary", "l2_hb", sizes, errs, tol, idx_o, ndims=3)
        assert np.array_equal(idx, idx_o)
        achieved = float(np.sum((out.astype(np.float64) - x) ** 2))
        assert achieved <= tol, (rel, achieved, tol)


@pytest.mark.parametrize("n,L", [(257, 6), (513, 7)])
def test_l2_plane_choices_equal_oracle_tables(n, L):
    # the headline workload (and its 257^3 sample): the tables the oracle
    # computes from the GPU's coefficients, fed to the oracle interpreter, pick
    # the planes the device picked for every relative L2 tolerance
    shape, B = (n, n, n), 32
    x = fields().spectral_grf(shape, slope=-5.0 / 3.0, seed=1234)
    mdr = api().MDRField(shape, torch.float32, L, B, "negabinary", "hierarchical", "squared")
    mdr.refactor(x)
    sizes, bounds, errs = mdr.level_info()
    mdr.refactor(x)
    assert mdr.level_info()[2].tobytes() == errs.tobytes()          # bitwise reproducible
    coef = mdr.coefficients().cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(mdr.level_elements.astype(np.int64))])
    oerrs = np.zeros_like(errs)
    for l in range(L + 1):
        c = coef[offs[l]:offs[l + 1]]
        e = math.frexp(float(O.max_abs(c)))[1]
        oerrs[l] = O.encode("negabinary", c, e, B, True)[2]
    # the device tables are exact sums rounded once; the oracle (like the
    # reference) adds n terms one by one in double, whose rounding error grows
    # up to about n * 2^-53 relative (5e-11 measured for 14.8 M values)
    for l in range(L + 1):
        rtol = max(1e-12, float(mdr.level_elements[l]) * 2.0 ** -53)
        np.testing.assert_allclose(errs[l], oerrs[l], rtol=rtol, atol=0)
    xh = x.cpu().numpy()
    norm2 = float(np.sum(xh.astype(np.float64) ** 2))
    out = torch.empty_like(x)
    mdr.reset()
    idx_o = np.zeros(L + 1, np.uint8)
    for rel in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
        tol = (rel ** 2) * norm2
        mdr.retrieve(tol, out=out, interpreter="negabinary", estimator="l2_hb")
        idx_o, _ = O.interpret("negabinary", "l2_hb", sizes, oerrs, tol, idx_o, ndims=3)
        assert np.array_equal(mdr.index(), idx_o), rel
        achieved = float(((out.double() - x.double()) ** 2).sum().item())
        assert achieved <= tol, (rel, achieved, tol)


def test_all_planes_roundtrip_and_reset():
    shape, L, B = (129, 129, 129), 5, 32
    x = fields().spectral_grf(shape, seed=2)
    mdr = api().MDRField(shape, torch.float32, L, B, "negabinary", "hierarchical", "max")
    mdr.refactor(x)
    out = mdr.retrieve_planes([B] * (L + 1))
    sizes, bounds, _ = mdr.level_info()
    # all planes: quantisation (sum of level quanta) plus fp32 rounding of the
    # recomposition (a few ulp of the field magnitude per level)
    quanta = sum(math.ldexp(1.0, math.frexp(b / 4)[1] + 2 - B) for b in bounds)
    rounding = 2 * (L + 1) * float(np.finfo(np.float32).eps) * float(x.abs().max())
    assert float((out - x).abs().max()) <= quanta + rounding
    mdr.reset()
    assert not mdr.index().any()
    z = mdr.retrieve_planes([0] * (L + 1))
    assert float(z.abs().max()) == 0.0


def test_constant_and_zero_fields():
    for val in (0.0, 3.5):
        shape = (33, 33, 33)
        x = torch.full(shape, val, dtype=torch.float32, device="cuda")
        mdr = api().MDRField(shape, torch.float32, 3, 32, "grouped", "hierarchical", "max")
        mdr.refactor(x)
        out = mdr.retrieve(1e-6)
        assert float((out - x).abs().max()) <= 1e-6


def test_invalid_requests_raise():
    from prodm_gb300._lib import ProdmError
    with pytest.raises(ProdmError):
        api().MDRField((65, 65, 65), torch.float32, 6, 32)      # above max level 5
    with pytest.raises(ProdmError):
        api().MDRField((65, 65, 65), torch.float32, 3, 33)      # > 32 planes for fp32
    with pytest.raises(ProdmError):
        api().MDRField((65, 65, 65), torch.float64, 3, 64, "grouped")


def test_metadata_and_level_files_match_reference_composed_refactor():
    """GPU refactor of the golden field reproduces the reference ComposedRefactor
    byte for byte: level files and metadata (whose reference layout is a prefix
    of ours; an extension carries the squared-error tables)."""
    g = np.load(__import__("golden_io").GOLDEN + "/composed.npz")
    field = g["field"]
    for enc in ("grouped", "negabinary"):
        mdr = api().MDRField(field.shape, torch.float32, 3, 32, enc, "hierarchical", "max")
        mdr.refactor(torch.from_numpy(field).cuda())
        files = np.concatenate([mdr.export_level(l) for l in range(4)])
        assert files.tobytes() == g[enc + "_levels"].tobytes()
        meta = mdr.metadata()
        ref = g[enc + "_metadata"].tobytes()
        assert meta[:len(ref)] == ref
        assert meta[len(ref):len(ref) + 4] == b"SQER"


@pytest.mark.parametrize("enc", ["grouped", "negabinary"])
def test_reconstructor_fed_from_reference_files(enc):
    """load_metadata + load_level from the reference's own level files, then the
    progressive retrieval of the reference driver (sign-exclude greedy, max HB
    estimator); results equal the reference's reconstruction up to float
    rounding whenever every level received planes."""
    g = np.load(__import__("golden_io").GOLDEN + "/composed.npz")
    field = g["field"]
    meta = g[enc + "_metadata"].tobytes()
    lb = g[enc + "_level_bytes"]
    levels = np.split(g[enc + "_levels"], np.cumsum(lb)[:-1])
    rec = api().MDRField(field.shape, torch.float32, 3, 32, enc, "hierarchical", "max")
    rec.load_metadata(meta)
    sizes, _, _ = rec.level_info()
    loaded = [0] * 4
    for t, tol in enumerate(g["tols"]):
        rec.interpret(float(tol), "sign_exclude", "max_hb")
        idx = rec.index()
        for l in range(4):
            need = int(sizes[l, :idx[l]].astype(np.int64).sum())
            if need > loaded[l]:
                rec.load_level(l, levels[l][loaded[l]:need], offset=loaded[l])
                loaded[l] = need
        out = rec.reconstruct().cpu().numpy()
        assert float(np.abs(out - field).max()) <= float(tol)
        if (idx > 0).all():
            np.testing.assert_allclose(out, g[enc + "_recon"][t], rtol=0, atol=1e-5 * float(np.abs(field).max()))


FUSED_SHAPES = [((65, 65, 65), 3), ((48, 40, 64), 2), ((33, 40, 129), 3), ((129, 129, 129), 4), ((200, 131), 4),
                ((33, 33, 1025), 2), ((40, 33, 301), 3), ((33, 33, 513), 3), ((40, 36, 411), 2), ((33, 32, 801), 2),
                ((129, 513), 3), ((65, 9, 513), 2), ((65, 17, 513), 2)]


@pytest.mark.parametrize("shape,L,B,tall,nd", [(s, L, 32, "1", "5") for s, L in FUSED_SHAPES] +
                         [((65, 65, 65), 3, 32, "0", "5"), ((33, 33, 513), 3, 32, "0", "5"),
                          ((129, 513), 3, 32, "0", "5"), ((65, 65, 65), 3, 20, "1", "5"),
                          ((33, 33, 513), 3, 24, "1", "5"), ((33, 33, 513), 3, 32, "1", "8"),
                          ((40, 33, 301), 3, 32, "1", "8"), ((40, 36, 411), 2, 32, "1", "6"),
                          ((65, 17, 513), 2, 32, "0", "6")])
def test_fused_finest_level_retrieval_is_bit_exact(shape, L, B, tall, nd, monkeypatch):
    """fp32 negabinary hierarchical: the finest level is decoded inside the
    recomposition kernel (odd and even row lengths take different kernels;
    odd rows of up to ~360 values the 8-warp TMA kernel, longer ones up to
    ~990 values the warp-specialised one: units of 11 rows where their tile
    rows fit 192 words, else of 8 rows with 160- and 256-word tile rows;
    longer still the cp.async kernel);
    the other levels go through the multi-level decoder. The TMA kernels stage
    a unit's planes by one box of all 32 plane rows (with PRODM_TMA_TALL=0 by
    one box per plane). The output equals the oracle's decode -> reposition ->
    recompose in float bit for bit, also for streams of fewer than 32 planes
    and for 5, 6 or 8 decode warps in the warp-specialised kernel
    (PRODM_WS_ND)."""
    monkeypatch.setenv("PRODM_TMA_TALL", tall)
    monkeypatch.setenv("PRODM_WS_ND", nd)
    x = fields().spectral_grf(shape, seed=sum(shape)).cpu().numpy()
    mdr = api().MDRField(shape, torch.float32, L, B, "negabinary", "hierarchical", "max")
    mdr.refactor(torch.from_numpy(x).cuda())
    sizes, bounds, _ = mdr.level_info()
    blob = np.concatenate([mdr.export_level(l) for l in range(L + 1)])
    rng = np.random.default_rng(len(shape) + L)
    cases = [np.zeros(L + 1, np.uint8), np.full(L + 1, B, np.uint8)]
    cases += [rng.integers(0, B + 1, L + 1).astype(np.uint8) for _ in range(4)]
    cases += [np.full(L + 1, k, np.uint8) for k in (1, 2, 7, 16, 17, 31) if k <= B]
    for idx in cases:
        mdr.reset()
        out = mdr.retrieve_planes([int(v) for v in idx]).cpu().numpy()
        ref = O.retrieve(shape, L, B, blob, sizes, bounds.astype(np.float32), idx, "negabinary", True)
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), idx


@pytest.mark.parametrize("tall", ["1", "0"])
@pytest.mark.parametrize("shape", [(65, 65, 65), (33, 33, 513)])
def test_fused_tile_wait_timeout_is_reported_and_recoverable(shape, tall, monkeypatch):
    """The fused finest-level kernels (the 8-warp form at 65^3, the
    warp-specialised form at 33 x 33 x 513) wait for their TMA plane tiles on
    mbarriers, each wait bounded. With the expected byte count raised (the test
    hook) no tile ever completes: every CTA gives up after a short limit,
    reports PRODM_ETIMEOUT and returns; the status is cleared once read and
    the next retrieval is exact again."""
    from prodm_gb300._lib import ProdmError
    monkeypatch.setenv("PRODM_TMA_TALL", tall)
    L = 3
    x = fields().spectral_grf(shape, seed=11, device="cuda")
    m = api().MDRField(shape, torch.float32, L, 32, "negabinary", "hierarchical", "max")
    m.refactor(x)
    idx = [16] * (L + 1)
    good = m.retrieve_planes(idx).clone()
    m.status()
    api().debug_tile_wait(64, 20000)
    try:
        m.reset()
        m.retrieve_planes(idx)
        with pytest.raises(ProdmError) as e:
            m.status()
        assert e.value.status == 4          # PRODM_ETIMEOUT
    finally:
        api().debug_tile_wait(0, 0)
    m.status()                              # reported once
    m.reset()
    assert torch.equal(m.retrieve_planes(idx), good)


@pytest.mark.parametrize("shape,L,dt", [((65, 65, 65), 3, np.float32), ((33, 17, 9), 2, np.float32),
                                        ((129, 65), 4, np.float32), ((17, 9, 129), 2, np.float32),
                                        ((33, 33, 33), 3, np.float64), ((17, 9, 33), 2, np.float64)])
def test_patch_kernels_bit_identical_to_row_kernels(shape, L, dt, monkeypatch):
    """The patch decomposition and recomposition (2^k + 1 grids; forced onto
    small grids with PRODM_PATCH_MIN_ITEMS=1) give the row kernels'
    coefficients, streams and reconstructions bit for bit (PRODM_DECOMPOSE_PATCH=0
    keeps every level on the row kernels); the fp32 reconstructions also equal
    the oracle's decode -> reposition -> recompose."""
    B = 32 if dt == np.float32 else 60
    tdt = torch.float32 if dt == np.float32 else torch.float64
    x = fields().spectral_grf(shape, seed=sum(shape), dtype=tdt)
    idx = [min(B, 9 + 3 * l) for l in range(L + 1)]
    res = {}
    for mode in ("patch", "rows"):
        monkeypatch.setenv("PRODM_PATCH_MIN_ITEMS", "1")
        monkeypatch.setenv("PRODM_DECOMPOSE_PATCH", "1" if mode == "patch" else "0")
        m = api().MDRField(shape, tdt, L, B, "negabinary", "hierarchical", "max")
        m.refactor(x)
        coef = m.coefficients().cpu().numpy()
        blob = np.concatenate([m.export_level(l) for l in range(L + 1)])
        out = m.retrieve_planes(idx).cpu().numpy()
        res[mode] = (coef, blob, out, m.level_info())
        m.close()
    for a, b in zip(res["patch"][:3], res["rows"][:3]):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    if dt == np.float32:
        sizes, bounds, _ = res["patch"][3]
        ref = O.retrieve(shape, L, B, res["patch"][1], sizes, bounds.astype(np.float32), np.array(idx, np.uint8),
                         "negabinary", True)
        assert np.array_equal(res["patch"][2].view(np.uint32), ref.view(np.uint32))
