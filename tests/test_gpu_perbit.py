"""Per-bit bitplane encoder on the device (PRODM_ENC_PERBIT) against the
reference's PerBitBPEncoder<T, uint32_t> (golden fixtures, tests/golden/perbit.npz)
and the oracle restatement.

* prodm_encode: streams and sizes bit for bit;
* prodm_progressive_decode: the reference's three-step progressive decode of
  its own streams, bit for bit (the per-bit parse of plane after plane);
* the device-resident pipeline (fp64, 60 planes, hierarchical basis, max
  collector, SignExclude interpreter): level files equal to the reference's,
  plane choices and reconstructions equal to the oracle's, and the same
  reconstruction when the reference's level files are loaded instead;
* sizes where the parse pipeline runs through many chunks, and malformed
  stream sizes rejected.
"""
import math
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
O = oracle.oracle()
HERE = os.path.dirname(os.path.abspath(__file__))


def golden():
    return np.load(os.path.join(HERE, "golden", "perbit.npz"))


def api():
    from prodm_gb300 import api as a
    return a


def cases():
    return [str(c) for c in golden()["cases"]]


@pytest.mark.parametrize("case", cases())
def test_encode_and_progressive_decode_match_reference(case):
    g = golden()
    dt, n, B = case.split("_")
    n, B, dtype = int(n[1:]), int(B[1:]), {"float32": torch.float32, "float64": torch.float64}[dt]
    x, e = g[case + "_x"], int(g[case + "_exp"])
    blob, sizes, _ = api().encode("perbit", torch.from_numpy(x).cuda(), e, B)
    assert np.array_equal(sizes, g[case + "_sizes"])
    assert np.array_equal(blob.cpu().numpy(), g[case + "_blob"])
    ref_blob = torch.from_numpy(g[case + "_blob"]).cuda()
    offs = np.concatenate([[0], np.cumsum(g[case + "_sizes"].astype(np.int64))])
    dec = api().ProgressiveDecoder("perbit", dtype)
    for i, (a, b) in enumerate(g[case + "_steps"]):
        a, b = int(a), int(b)
        out = dec.decode(ref_blob[offs[a]:offs[b]], g[case + "_sizes"][a:b], n, e, a, b - a, 0, B)
        assert np.array_equal(out.cpu().numpy().view(np.uint8), g["%s_dec%d" % (case, i)].view(np.uint8)), i


def test_pipeline_fp64_60_planes_matches_reference_and_oracle():
    g = golden()
    field = g["composed_field"]
    L, B = 3, 60
    shape = field.shape
    m = api().MDRField(shape, torch.float64, L, B, "perbit", "hierarchical", "max")
    m.refactor(torch.from_numpy(field).cuda())
    files = np.concatenate([m.export_level(l) for l in range(L + 1)])
    assert files.tobytes() == g["composed_levels"].tobytes()
    res = O.refactor(field, L, B, "perbit", True)
    sizes, bounds, _ = m.level_info()
    assert np.array_equal(sizes.ravel(), res["sizes"].ravel())
    out = torch.empty(shape, dtype=torch.float64, device="cuda")
    idx = np.zeros(L + 1, np.uint8)
    for t, tol in enumerate(g["composed_tols"]):
        m.retrieve(float(tol), out=out, interpreter="sign_exclude", estimator="max_hb")
        errs = np.stack([O.max_collect(b, B, np.float64) for b in res["bounds"]])
        idx, _ = O.interpret("sign_exclude", "max_hb", res["sizes"], errs, float(tol), idx, dtype=np.float64)
        assert np.array_equal(m.index(), idx), t
        ref = O.retrieve(shape, L, B, res["blob"], res["sizes"], res["bounds"], idx, "perbit", True, np.float64)
        got = out.cpu().numpy()
        assert np.array_equal(got, ref), t
        assert np.max(np.abs(got - field)) <= tol
        # the reference sums progressive deltas: equal up to rounding
        np.testing.assert_allclose(got, g["composed_recon"][t], atol=1e-12 * float(np.abs(field).max()), rtol=0)


def test_pipeline_from_reference_level_files():
    """the reference's own level files + metadata, loaded in two pieces per
    level: the per-bit parse feeds the same reconstruction as a device refactor"""
    g = golden()
    field = g["composed_field"]
    L, B = 3, 60
    shape = field.shape
    lb = g["composed_level_bytes"]
    offs = np.concatenate([[0], np.cumsum(lb)])
    dev = api().MDRField(shape, torch.float64, L, B, "perbit", "hierarchical", "max")
    dev.refactor(torch.from_numpy(field).cuda())
    m = api().MDRField(shape, torch.float64, L, B, "perbit", "hierarchical", "max")
    m.load_metadata(g["composed_metadata"].tobytes())
    out = torch.empty(shape, dtype=torch.float64, device="cuda")
    ref_out = torch.empty_like(out)
    for half in (0, 1):
        for l in range(L + 1):
            lvl = g["composed_levels"][offs[l]:offs[l + 1]]
            cut = len(lvl) // 2
            if half == 0:
                m.load_level(l, lvl[:cut], 0)
            else:
                m.load_level(l, lvl[cut:], cut)
        sizes, _, _ = m.level_info()
        csum = np.cumsum(sizes.astype(np.int64), axis=1)
        # planes fully inside the loaded bytes
        idx = [int(np.searchsorted(csum[l], lb[l] // 2 if half == 0 else lb[l], side="right")) for l in range(L + 1)]
        m.retrieve_planes(idx, out=out)
        dev.retrieve_planes(idx, out=ref_out)
        assert torch.equal(out, ref_out), (half, idx)
    tol = float(g["composed_tols"][1])
    m.reset()
    dev.reset()
    m.retrieve(tol, out=out, interpreter="sign_exclude", estimator="max_hb")
    dev.retrieve(tol, out=ref_out, interpreter="sign_exclude", estimator="max_hb")
    assert torch.equal(out, ref_out)
    assert float((out.cpu() - torch.from_numpy(field)).abs().max()) <= tol


@pytest.mark.parametrize("shape,L,dt,B", [((65, 65, 65), 3, np.float32, 32), ((33, 64), 4, np.float64, 63),
                                          ((1000,), 5, np.float32, 20), ((17, 9, 33), 2, np.float64, 60)])
def test_pipeline_shapes_match_oracle(shape, L, dt, B):
    rng = np.random.default_rng(len(shape) * 100 + B)
    field = (np.cumsum(rng.standard_normal(shape), axis=-1) + 0.01 * rng.standard_normal(shape)).astype(dt)
    tdt = torch.float32 if dt == np.float32 else torch.float64
    m = api().MDRField(shape, tdt, L, B, "perbit", "hierarchical", "max")
    m.refactor(torch.from_numpy(field).cuda())
    res = O.refactor(field, L, B, "perbit", True)
    files = np.concatenate([m.export_level(l) for l in range(L + 1)])
    assert files.tobytes() == res["blob"].tobytes()
    vr = float(field.max() - field.min())
    for rel in (1e-2, 1e-4, 1e-6):
        out = m.retrieve(rel * vr, interpreter="sign_exclude", estimator="max_hb")
        idx = m.index()
        ref = O.retrieve(shape, L, B, res["blob"], res["sizes"], res["bounds"], idx, "perbit", True, dt)
        assert np.array_equal(out.cpu().numpy(), ref), rel
        # met, unless every plane is retrieved and B limits the precision
        err = float(np.max(np.abs(ref.astype(np.float64) - field)))
        assert err <= rel * vr * (1 + 1e-6) or np.all(idx == B), (rel, err, idx)


@pytest.mark.parametrize("dt,scale", [(np.float64, 1e-300), (np.float64, 1e300), (np.float64, 1e-310),
                                      (np.float32, 1e-36), (np.float32, 1e36), (np.float32, 1e-42)])
def test_extreme_exponents_match_oracle(dt, scale):
    """level exponents far from 0 (subnormal values, scalings outside the
    normal range): the device encode / decode paths against the oracle"""
    rng = np.random.default_rng(int(abs(math.log10(scale))))
    n = 4099
    B = 60 if dt == np.float64 else 32
    x = (rng.standard_normal(n) * scale).astype(dt)
    x[rng.random(n) < 0.1] = 0
    mx = float(np.abs(x).max())
    e = math.frexp(mx)[1]
    blob, sizes = O.pb_encode(x, e, B)
    tdt = torch.float32 if dt == np.float32 else torch.float64
    gblob, gsizes, _ = api().encode("perbit", torch.from_numpy(x).cuda(), e, B)
    assert np.array_equal(gsizes, sizes) and np.array_equal(gblob.cpu().numpy(), blob)
    offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
    dev = api().ProgressiveDecoder("perbit", tdt)
    st = O.perbit_state(dt)
    d = torch.from_numpy(blob).cuda()
    for a, b in [(0, 5), (5, B)]:
        got = dev.decode(d[offs[a]:offs[b]], sizes[a:b], n, e, a, b - a, 0, B).cpu().numpy()
        ref = st.decode(blob[offs[a]:offs[b]], sizes[a:b], n, e, a, b - a, 0)
        assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), (a, b)


@pytest.mark.parametrize("dt,B,n", [(np.float64, 60, 300001), (np.float32, 32, 1 << 20)])
def test_parse_many_chunks(dt, B, n):
    """one level large enough that the plane pipeline wraps its ring many
    times; decoded in four calls against the oracle's progressive decode"""
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) * np.exp(rng.uniform(-12, 0, n))).astype(dt)
    x[rng.random(n) < 0.2] = 0
    e = math.frexp(float(np.abs(x).max()))[1]
    blob, sizes = O.pb_encode(x, e, B)
    tdt = torch.float32 if dt == np.float32 else torch.float64
    gblob, gsizes, _ = api().encode("perbit", torch.from_numpy(x).cuda(), e, B)
    assert np.array_equal(gsizes, sizes) and np.array_equal(gblob.cpu().numpy(), blob)
    offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
    dev = api().ProgressiveDecoder("perbit", tdt)
    st = O.perbit_state(dt)
    d = torch.from_numpy(blob).cuda()
    steps = [(0, 7), (7, 19), (19, 20), (20, B)]
    for a, b in steps:
        got = dev.decode(d[offs[a]:offs[b]], sizes[a:b], n, e, a, b - a, 0, B).cpu().numpy()
        ref = st.decode(blob[offs[a]:offs[b]], sizes[a:b], n, e, a, b - a, 0)
        assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), (a, b)


def test_malformed_or_out_of_order_streams_rejected():
    from prodm_gb300._lib import ProdmError
    rng = np.random.default_rng(3)
    n, B = 5000, 32
    x = rng.standard_normal(n).astype(np.float32)
    e = math.frexp(float(np.abs(x).max()))[1]
    blob, sizes = O.pb_encode(x, e, B)
    d = torch.from_numpy(blob).cuda()
    dec = api().ProgressiveDecoder("perbit", torch.float32)
    bad = sizes.copy()
    bad[0] -= 8                                 # stream 0 said to end one word early
    with pytest.raises(ProdmError):
        dec.decode(d, bad, n, e, 0, 1, 0, B)
    dec2 = api().ProgressiveDecoder("perbit", torch.float32)
    with pytest.raises(ProdmError):            # a level starts at plane 0
        dec2.decode(d[int(sizes[0]):], sizes[1:], n, e, 1, 2, 0, B)
    dec2.decode(d, sizes, n, e, 0, 3, 0, B)
    with pytest.raises(ProdmError):            # and continues where it stopped
        dec2.decode(d, sizes[5:], n, e, 5, 2, 0, B)
    with pytest.raises(ProdmError):            # the squared collector is not a per-bit option
        api().MDRField((33, 33, 33), torch.float32, 2, 32, "perbit", "hierarchical", "squared")
