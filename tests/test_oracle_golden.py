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
