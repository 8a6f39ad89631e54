"""CUDA components through the C ABI against the reference's golden vectors
and the oracle. Bit-exact for streams, decoded values, interleave order and
interpreter indices; error tables within rtol 1e-12: the fp32 encoder tables
are exact integer sums rounded once to double, the fp64 tables and the
squared-error collector fp64 sums in a fixed order, while the reference adds
its terms one by one in double (a relative difference of a few 1e-16 per
term at the fixture sizes). Tables are bitwise reproducible run to run."""
import math

import numpy as np
import pytest
import torch

import oracle
from golden_io import encoder_cases, load, split_streams

pytestmark = pytest.mark.gpu

O = oracle.oracle()
ERR_RTOL = 1e-12


def api():
    from prodm_gb300 import api as a
    return a


def tdt(npdt):
    return torch.float32 if np.dtype(npdt) == np.float32 else torch.float64


@pytest.mark.parametrize("case", [c[0] for c in encoder_cases()])
def test_encode_matches_reference_streams(case):
    g = load("encoders")
    dt, kind, n, B = case.split("_")
    B = int(B[1:])
    x = torch.from_numpy(g[case + "_x"]).cuda()
    e = int(g[case + "_exp"])
    collect = (case + "_errs") in g.files
    blob, sizes, errs = api().encode(kind, x, e, B, collect)
    assert np.array_equal(sizes, g[case + "_sizes"])
    assert np.array_equal(blob.cpu().numpy(), g[case + "_blob"])
    if collect:
        np.testing.assert_allclose(errs, g[case + "_errs"], rtol=ERR_RTOL, atol=1e-30)


@pytest.mark.parametrize("case", [c[0] for c in encoder_cases()])
def test_progressive_decode_matches_reference(case):
    g = load("encoders")
    dt, kind, n, B = case.split("_")
    n, B = int(n[1:]), int(B[1:])
    blob, sizes = g[case + "_blob"], g[case + "_sizes"]
    e = int(g[case + "_exp"])
    s1 = int(g[case + "_split"])
    offs = split_streams(blob, sizes)
    dec = api().ProgressiveDecoder(kind, tdt(dt))
    b1 = torch.from_numpy(blob[offs[0]:offs[s1]].copy()).cuda()
    b2 = torch.from_numpy(blob[offs[s1]:offs[B]].copy()).cuda()
    d1 = dec.decode(b1, sizes[:s1], n, e, 0, s1, 0, B).cpu().numpy()
    d2 = dec.decode(b2, sizes[s1:], n, e, s1, B - s1, 0, B).cpu().numpy()
    assert d1.tobytes() == g[case + "_dec1"].tobytes()
    assert d2.tobytes() == g[case + "_dec2"].tobytes()


def test_interleave_matches_reference():
    g = load("geometry")
    for i in range(4):
        x = g["il%d_x" % i]
        fine, coarse = g["il%d_fine" % i], g["il%d_coarse" % i]
        buf = api().interleave(torch.from_numpy(x).cuda(), fine, coarse)
        assert np.array_equal(buf.cpu().numpy(), g["il%d_buf" % i])
        y = torch.zeros_like(torch.from_numpy(x)).cuda()
        api().reposition(buf, y, fine, coarse)
        expect = np.zeros_like(x)
        O.reposition(g["il%d_buf" % i], expect, x.shape, fine, coarse)
        assert np.array_equal(y.cpu().numpy(), expect)


def test_level_geometry_matches_reference():
    g = load("geometry")
    for key in g["cases"]:
        key = str(key)
        ld, le = api().level_dims(list(g[key + "_dims"]), int(g[key + "_L"]))
        assert np.array_equal(ld, g[key + "_ld"])
        assert np.array_equal(le.astype(np.uint32), g[key + "_le"])


def test_interpreters_match_reference():
    g = load("interpreters")
    cases = [str(k) for k in g["cases"]]
    for key in cases:
        t = int(g[key + "_trial"])
        idx, rsz = api().interpret(str(g[key + "_kind"]), str(g[key + "_est"]), g["t%d_sizes" % t],
                                   g["t%d_errs" % t], float(g[key + "_tol"]), g[key + "_idx0"], ndims=3, s=0.5)
        assert np.array_equal(idx, g[key + "_idx"]), key
        assert np.array_equal(rsz, g[key + "_rsz"]), key


def test_collectors_match_reference():
    g = load("collectors")
    for key in g["cases"]:
        key = str(key)
        B = int(key.split("_")[0][1:])
        x = g[key + "_x"]
        mx = np.float32(np.max(np.abs(x)))
        sq = api().collect_squared(torch.from_numpy(x).cuda(), B, float(mx))
        np.testing.assert_allclose(sq, g[key + "_sq"], rtol=ERR_RTOL, atol=1e-30)
        np.testing.assert_array_equal(api().collect_max(float(mx * np.float32(4)), B), g[key + "_max"])


SHAPES = [((65, 65, 65), 3), ((17, 9, 33), 2), ((12, 10, 7), 1), ((100,), 5), ((33, 65), 4), ((20, 21, 22), 3),
          ((5, 5, 5), 1), ((129, 40), 4)]


@pytest.mark.parametrize("shape,L", SHAPES)
@pytest.mark.parametrize("basis", ["hierarchical", "orthogonal"])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_decompose_matches_fp64_oracle(shape, L, basis, dt):
    rng = np.random.default_rng(hash((shape, L)) % 2 ** 32)
    x = rng.standard_normal(shape).astype(dt)
    ref = O.decompose(x.astype(np.float64), shape, L, basis == "hierarchical")
    d = torch.from_numpy(x.copy()).cuda()
    api().decompose(d, L, basis)
    got = d.cpu().numpy().astype(np.float64)
    scale = float(np.abs(x).max())
    tol = (1e-6 if dt == np.float32 else 1e-13) * scale
    assert np.max(np.abs(got - ref)) <= tol
    api().recompose(d, L, basis)
    back = d.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(back - x)) <= tol * 4


def test_squared_collector_edge_values():
    x = np.array([0.0, -0.0, 1e-30, -1e-30, 2.0 ** -20, 1.0, -1.0, 0.75, 3.0e-8], np.float32)
    x = np.tile(x, 40)
    mx = np.float32(np.max(np.abs(x)))
    for B in (1, 8, 23, 32):
        got = api().collect_squared(torch.from_numpy(x).cuda(), B, float(mx))
        np.testing.assert_allclose(got, O.sq_collect(x, B, mx), rtol=ERR_RTOL, atol=1e-30)


@pytest.mark.parametrize("kind", ["negabinary", "grouped"])
@pytest.mark.parametrize("n", [1, 5, 31, 32, 33, 1000, 70001])
def test_encode_small_and_ragged_levels(kind, n):
    # n < 32: one short block (the reference's block loop wraps there)
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n).astype(np.float32)
    e = math.frexp(float(np.abs(x).max()))[1]
    for B in (1, 2, 17, 32):
        blob, sizes, errs = api().encode(kind, torch.from_numpy(x).cuda(), e, B, True)
        ob, osz, oerr = O.encode(kind, x, e, B, True)
        assert np.array_equal(sizes, osz)
        assert np.array_equal(blob.cpu().numpy(), ob)
        np.testing.assert_allclose(errs, oerr, rtol=ERR_RTOL, atol=1e-30)


@pytest.mark.parametrize("kind", ["negabinary", "grouped"])
def test_encode_fp64_large(kind):
    rng = np.random.default_rng(3)
    x = (rng.standard_normal(200003) * 1e-5).astype(np.float64)
    x[1000:5000] = 0
    e = math.frexp(float(np.abs(x).max()))[1]
    for B in (33, 60):
        blob, sizes, _ = api().encode(kind, torch.from_numpy(x).cuda(), e, B, False)
        ob, osz, _ = O.encode(kind, x, e, B, False)
        assert np.array_equal(sizes, osz)
        assert np.array_equal(blob.cpu().numpy(), ob)


@pytest.mark.parametrize("kind", ["negabinary", "grouped"])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_error_tables_are_reproducible(kind, dt):
    # many CTAs, values on both sides of 2^23 after scaling, zero runs
    rng = np.random.default_rng(17)
    n = 3_000_017
    x = (rng.standard_normal(n) * np.exp(rng.uniform(-12, 0, n))).astype(dt)
    x[100:5000] = 0
    e = math.frexp(float(np.abs(x).max()))[1]
    B = 32 if dt == np.float32 else 60
    xd = torch.from_numpy(x).cuda()
    tabs = [api().encode(kind, xd, e, B, True)[2] for _ in range(3)]
    assert tabs[0].tobytes() == tabs[1].tobytes() == tabs[2].tobytes()
    _, _, oerr = O.encode(kind, x, e, B, True)
    np.testing.assert_allclose(tabs[0], oerr, rtol=1e-11, atol=0)
    sq = [api().collect_squared(xd, B, float(np.abs(x).max())) for _ in range(2)]
    assert sq[0].tobytes() == sq[1].tobytes()
