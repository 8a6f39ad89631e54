"""The oracle restatement against golden vectors produced by the reference's
own classes (tests/golden/make_golden.py). CPU only."""
import numpy as np
import pytest

import oracle
from golden_io import encoder_cases, load, split_streams

O = oracle.oracle()


@pytest.mark.parametrize("case", [c[0] for c in encoder_cases()])
def test_encoder_streams_bit_exact(case):
    g = load("encoders")
    dt, kind, n, B = case.split("_")
    n, B = int(n[1:]), int(B[1:])
    x = g[case + "_x"]
    e = int(g[case + "_exp"])
    collect = (case + "_errs") in g.files
    blob, sizes, errs = O.encode(kind, x, e, B, collect)
    assert np.array_equal(sizes, g[case + "_sizes"])
    assert np.array_equal(blob, g[case + "_blob"])
    if collect:
        np.testing.assert_allclose(errs, g[case + "_errs"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("case", [c[0] for c in encoder_cases()])
def test_progressive_decode_bit_exact(case):
    g = load("encoders")
    dt, kind, n, B = case.split("_")
    n, B = int(n[1:]), int(B[1:])
    blob, sizes = g[case + "_blob"], g[case + "_sizes"]
    e = int(g[case + "_exp"])
    s1 = int(g[case + "_split"])
    offs = split_streams(blob, sizes)
    dtype = np.dtype(dt)
    if kind == "negabinary":
        d1 = O.nb_decode(blob[offs[0]:offs[s1]], sizes[:s1], n, e, 0, s1, dtype)
        d2 = O.nb_decode(blob[offs[s1]:offs[B]], sizes[s1:], n, e, s1, B - s1, dtype)
    else:
        st = O.grouped_state(dtype)
        d1 = st.decode(blob[offs[0]:offs[s1]], sizes[:s1], n, e, 0, s1, 0)
        d2 = st.decode(blob[offs[s1]:offs[B]], sizes[s1:], n, e, s1, B - s1, 0)
    assert d1.tobytes() == g[case + "_dec1"].tobytes()
    assert d2.tobytes() == g[case + "_dec2"].tobytes()


def test_collectors_match_reference():
    g = load("collectors")
    for key in g["cases"]:
        key = str(key)
        B = int(key.split("_")[0][1:])
        x = g[key + "_x"]
        mx = np.float32(np.max(np.abs(x)))
        np.testing.assert_array_equal(O.sq_collect(x, B, mx), g[key + "_sq"])
        np.testing.assert_array_equal(O.max_collect(mx * np.float32(4), B, np.float32), g[key + "_max"])


def test_interpreters_match_reference():
    g = load("interpreters")
    for key in g["cases"]:
        key = str(key)
        t = int(g[key + "_trial"])
        idx, rsz = O.interpret(str(g[key + "_kind"]), str(g[key + "_est"]), g["t%d_sizes" % t], g["t%d_errs" % t],
                               float(g[key + "_tol"]), g[key + "_idx0"], ndims=3, s=0.5)
        assert np.array_equal(idx, g[key + "_idx"]), key
        assert np.array_equal(rsz, g[key + "_rsz"]), key


def test_level_geometry_matches_reference():
    g = load("geometry")
    for key in g["cases"]:
        key = str(key)
        dims, L = g[key + "_dims"], int(g[key + "_L"])
        assert np.array_equal(O.level_dims(dims, L), g[key + "_ld"])
        assert np.array_equal(O.level_elements(dims, L), g[key + "_le"])
    for i in range(4):
        x = g["il%d_x" % i]
        buf = O.interleave(x, x.shape, g["il%d_fine" % i], g["il%d_coarse" % i])
        assert np.array_equal(buf, g["il%d_buf" % i])
        y = np.zeros_like(x)
        O.reposition(buf, y, x.shape, g["il%d_fine" % i], g["il%d_coarse" % i])
        fine, coarse = g["il%d_fine" % i], g["il%d_coarse" % i]
        sl = tuple(slice(0, int(f)) for f in fine)
        mask = np.zeros(x.shape, bool)
        mask[sl] = True
        if coarse.any():
            mask[tuple(slice(0, int(c)) for c in coarse)] = False
        assert np.array_equal(y[mask], x[mask])


@pytest.mark.parametrize("enc", ["grouped", "negabinary"])
def test_composed_refactor_level_files_match_reference(enc):
    g = load("composed")
    field = g["field"]
    res = O.refactor(field, 3, 32, enc, True)
    assert res["blob"].tobytes() == g[enc + "_levels"].tobytes()


@pytest.mark.parametrize("enc", ["grouped", "negabinary"])
def test_composed_retrieve_meets_tolerance_like_reference(enc):
    g = load("composed")
    field = g["field"]
    res = O.refactor(field, 3, 32, enc, True)
    L, B = 3, 32
    idx = np.zeros(L + 1, np.uint8)
    dtype = np.float32
    for t, tol in enumerate(g["tols"]):
        errs = np.stack([O.max_collect(b, B, dtype) for b in res["bounds"]])
        idx, _ = O.interpret("sign_exclude", "max_hb", res["sizes"], errs, float(tol), idx, dtype=dtype)
        rec = O.retrieve(field.shape, L, B, res["blob"], res["sizes"], res["bounds"], idx, enc, True, dtype)
        err = np.max(np.abs(rec - field))
        assert err <= tol
        ref = g[enc + "_recon"][t]
        # the reference accumulates progressive deltas; the oracle re-decodes all
        # retrieved planes. Same planes => same result up to float rounding.
        if (idx > 0).all():
            np.testing.assert_allclose(rec, ref, atol=1e-5 * float(np.abs(field).max()), rtol=0)


def test_ge_qoi_utilities_match_reference():
    """oracle restatement of qoi_utils.hpp (values, V_TOT and T estimates)
    against the reference's own functions on the same points, bit for bit"""
    g = load("qoi")
    O = oracle.oracle()
    vals = O.qoi_values(g["vx"], g["vy"], g["vz"], g["p"], g["d"])
    for k, v in zip(("vtot", "temp", "c", "mach", "pt", "mu"), vals):
        assert np.array_equal(v, g[k], equal_nan=True), k
    assert np.array_equal(O.qoi_vtot_bound(g["vx"], g["vy"], g["vz"], g["ebs_v"]), g["bound_vtot"])
    assert np.array_equal(O.qoi_t_bound(g["p"], g["d"], *g["eb_pd"]), g["bound_t"])
    # the edge points exercise every branch of the rules; a negative density
    # gives a negative temperature, whose square root is NaN in the reference too
    assert np.all(g["bound_vtot"][:4] > 0) and np.any(g["bound_t"][8:12] == 0)
    assert np.isnan(g["c"][[9, 11]]).all() and not np.isnan(g["c"][[8, 10]]).any()


def _perbit_cases():
    return [str(c) for c in load("perbit")["cases"]]


@pytest.mark.parametrize("case", _perbit_cases())
def test_perbit_streams_and_progressive_decode_bit_exact(case):
    """oracle PerBit encode / progressive decode (three steps through one
    decoder state) against PerBitBPEncoder<T, uint32_t> itself"""
    g = load("perbit")
    dt, n, B = case.split("_")
    n, B, dtype = int(n[1:]), int(B[1:]), np.dtype(dt)
    x, e = g[case + "_x"], int(g[case + "_exp"])
    blob, sizes = O.pb_encode(x, e, B)
    assert np.array_equal(sizes, g[case + "_sizes"])
    assert np.array_equal(blob, g[case + "_blob"])
    offs = split_streams(blob, sizes)
    dec = O.perbit_state(dtype)
    total = np.zeros(n, dtype)
    for i, (a, b) in enumerate(g[case + "_steps"]):
        d = dec.decode(blob[offs[a]:offs[b]], sizes[a:b], n, e, int(a), int(b - a), 0)
        assert np.array_equal(d.view(np.uint8), g["%s_dec%d" % (case, i)].view(np.uint8)), i
        total = total + d
    # all planes: every element within one unit of the last plane
    assert np.all(np.abs(total.astype(np.float64) - x.astype(np.float64)) <= np.ldexp(1.0, e - B) * (1 + 1e-6))


def test_perbit_composed_level_files_and_retrieval_match_reference():
    g = load("perbit")
    field = g["composed_field"]
    L, B = 3, 60
    res = O.refactor(field, L, B, "perbit", True)
    assert res["blob"].tobytes() == g["composed_levels"].tobytes()
    idx = np.zeros(L + 1, np.uint8)
    for t, tol in enumerate(g["composed_tols"]):
        errs = np.stack([O.max_collect(b, B, np.float64) for b in res["bounds"]])
        idx, _ = O.interpret("sign_exclude", "max_hb", res["sizes"], errs, float(tol), idx, dtype=np.float64)
        rec = O.retrieve(field.shape, L, B, res["blob"], res["sizes"], res["bounds"], idx, "perbit", True,
                         np.float64)
        assert np.max(np.abs(rec - field)) <= tol
        # same planes as the reference: the bytes it read are the planes' sizes
        sz = res["sizes"].reshape(L + 1, B).astype(np.int64)
        planes = sum(int(sz[l, :idx[l]].sum()) for l in range(L + 1))
        assert planes == int(g["composed_retrieved"][t]), t
        np.testing.assert_allclose(rec, g["composed_recon"][t], atol=1e-12 * float(np.abs(field).max()), rtol=0)


def test_adaptive_stopping_rule_matches_reference():
    """AdaptiveLevelCompressor's rule restated (oracle) on the reference's own
    zstd sizes: same stopping index, same sizes left, on every fixture level
    and latter index"""
    g = load("lossless")
    for key in g["cases"]:
        key = str(key)
        raw, zs = g[key + "_raw"], g[key + "_zstd"]
        stop, flags = O.adaptive_stopping(raw, zs, int(g[key + "_latter"]))
        assert stop == int(g[key + "_stop"]), key
        assert np.array_equal(np.where(flags == 1, zs, raw), g[key + "_left"]), key


@pytest.mark.parametrize("n", [0, 1, 3, 4, 5, 4095, 4096, 4097, 12289])
def test_zcb_codec_round_trip(n):
    """the lossless stage's codec (oracle restatement): every density round
    trips; all-zero data keeps only the header and each chunk's word masks"""
    rng = np.random.default_rng(n)
    for dens in (0.0, 0.001, 0.05, 0.5, 1.0):
        raw = ((rng.random(n) < dens) * rng.integers(1, 256, n)).astype(np.uint8)
        comp = O.zcb_compress(raw)
        assert np.array_equal(O.zcb_decompress(comp, n), raw)
        if dens == 0.0:
            nch = (n + 4095) // 4096
            assert comp.size == 12 + 4 * nch + 128 * nch
    with pytest.raises(ValueError):
        O.zcb_decompress(np.zeros(11, np.uint8), 100)
