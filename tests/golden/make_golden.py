"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference tree is present: the reference's MDR headers are
compiled by oracle/build_oracle.build_ref (oracle/_ref/libprodm_ref.so) and
every fixture below is produced by calling the reference's own classes
(NegaBinaryBPEncoder, GroupedBPEncoder, PerBitBPEncoder, AdaptiveLevelCompressor, MaxErrorCollector,
SquaredErrorCollector, the greedy size interpreters, DirectInterleaver,
compute_level_dims/elements and the ComposedRefactor -> ComposedReconstructor
pair). Inputs are seeded and stored beside the outputs so that the fixtures
do not depend on floating-point library differences between hosts.

Usage:  python tests/golden/make_golden.py
"""
import math
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

ENC_N = (32, 33, 63, 64, 65, 95, 127, 128, 729, 4184)
ENC_N64 = (64, 65, 127, 128, 129, 191, 729, 4184)


def coeff_like(rng, n, dt, scale):
    x = rng.standard_normal(n) * scale
    x[rng.random(n) < 0.15] = 0.0
    x = x.astype(dt)
    if n > 8:
        x[0] = 0.0
        x[1] = -0.0
        x[2] = -(2.0 ** -3) * scale
        x[3] = 2.0 ** math.floor(math.log2(scale))  # exact power of two
    if n > 64:
        x[40:72] = 0.0                             # an all-zero block
    return x


def encoder_fixtures(R, rng):
    out = {}
    cases = []
    for dt, ns, Bs in ((np.float32, ENC_N, (2, 8, 31, 32)), (np.float64, ENC_N64, (2, 33, 60))):
        for kind in ("negabinary", "grouped"):
            for n in ns:
                for B in Bs:
                    scale = float(rng.choice([1e-3, 1.0, 1e3]))
                    x = coeff_like(rng, n, dt, scale)
                    mx = float(np.max(np.abs(x)))
                    e = math.frexp(mx)[1]
                    collect = dt == np.float32
                    blob, sizes, errs = R.encode(kind, x, e, B, collect)
                    # progressive decode in two steps as the reconstructor does
                    dec = R.decoder(kind, dt)
                    s1 = max(1, B // 3)
                    offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
                    d1 = dec.decode(blob[offs[0]:offs[s1]], sizes[:s1], n, e, 0, s1, 0)
                    d2 = dec.decode(blob[offs[s1]:offs[B]], sizes[s1:], n, e, s1, B - s1, 0)
                    key = "%s_%s_n%d_B%d" % (np.dtype(dt).name, kind, n, B)
                    out[key + "_x"] = x
                    out[key + "_exp"] = np.int32(e)
                    out[key + "_blob"] = blob
                    out[key + "_sizes"] = sizes
                    if collect:
                        out[key + "_errs"] = errs
                    out[key + "_dec1"] = d1
                    out[key + "_dec2"] = d2
                    out[key + "_split"] = np.int32(s1)
                    cases.append(key)
    out["cases"] = np.array(cases)
    return out


def collector_fixtures(R, rng):
    out = {}
    cases = []
    for B in (8, 16, 32):
        for scale in (1e-2, 1.0, 1e4):
            x = (rng.standard_normal(2000) * scale).astype(np.float32)
            x[rng.random(2000) < 0.1] = 0
            mx = np.float32(np.max(np.abs(x)))
            key = "B%d_s%g" % (B, scale)
            out[key + "_x"] = x
            out[key + "_sq"] = R.sq_collect(x, B, mx)
            out[key + "_max"] = R.max_collect(mx * np.float32(4), B, np.float32)
            cases.append(key)
    out["cases"] = np.array(cases)
    return out


def interpreter_fixtures(R, rng):
    out = {}
    cases = []
    t = 0
    for trial in range(60):
        nl = int(rng.integers(1, 9))
        B = int(rng.choice([8, 32]))
        sizes = rng.integers(0 if trial % 4 == 0 else 1, 5000, size=(nl, B)).astype(np.uint32)
        errs = np.sort(rng.random((nl, B + 1)) * 10.0 ** rng.integers(-3, 3, size=(nl, 1)), axis=1)[:, ::-1].copy()
        if trial % 5 == 0:
            errs[:, 1:] = np.round(errs[:, 1:], 1)  # ties
        out["t%d_sizes" % trial] = sizes
        out["t%d_errs" % trial] = errs
        for kind in ("greedy", "sign_exclude", "negabinary"):
            for est in ("max_hb", "max_ob", "l2_hb", "snorm"):
                tol = float(10.0 ** rng.uniform(-4, 1))
                idx0 = np.zeros(nl, np.uint8) if trial % 2 else rng.integers(0, B // 2, nl).astype(np.uint8)
                idx, rsz = R.interpret(kind, est, sizes, errs, tol, idx0, ndims=3, s=0.5)
                key = "c%d" % t
                out[key + "_trial"] = np.int32(trial)
                out[key + "_tol"] = np.float64(tol)
                out[key + "_idx0"] = idx0
                out[key + "_idx"] = idx
                out[key + "_rsz"] = rsz
                out[key + "_kind"] = np.array(kind)
                out[key + "_est"] = np.array(est)
                cases.append(key)
                t += 1
    out["cases"] = np.array(cases)
    return out


def geometry_fixtures(R, rng):
    out = {}
    cases = []
    shapes = [((65, 65, 65), 3), ((513, 513, 513), 7), ((1025, 1025, 513), 8), ((129, 257, 65), 5),
              ((33, 33, 33), 3), ((100,), 5), ((12, 10, 7), 1)]
    for i, (shape, L) in enumerate(shapes):
        ld, le = R.level_dims_elements(shape, L)
        out["g%d_dims" % i] = np.array(shape, np.uint32)
        out["g%d_L" % i] = np.int32(L)
        out["g%d_ld" % i] = ld
        out["g%d_le" % i] = le
        cases.append("g%d" % i)
    # interleave / reposition of the reference DirectInterleaver (1-D and 3-D)
    for i, (shape, fine, coarse) in enumerate([((9, 10, 11), (9, 10, 11), (5, 6, 6)), ((9, 10, 11), (5, 6, 6), (3, 4, 4)),
                                               ((40,), (40,), (21,)), ((9, 10, 11), (3, 4, 4), (0, 0, 0))]):
        x = rng.standard_normal(shape).astype(np.float32)
        buf = R.interleave(x, shape, fine, coarse)
        out["il%d_x" % i] = x
        out["il%d_fine" % i] = np.array(fine, np.uint32)
        out["il%d_coarse" % i] = np.array(coarse, np.uint32)
        out["il%d_buf" % i] = buf
    out["cases"] = np.array(cases)
    return out


def sinusoid_field(rng, n):
    """Sum of 4 random-phase sinusoids (wavenumbers 1-8, amplitude 1) + N(0, 1e-3^2)."""
    ii = np.indices((n, n, n)).astype(np.float64)
    g = np.zeros((n, n, n))
    for _ in range(4):
        kv = rng.integers(1, 9, 3) * rng.choice([-1, 1], 3)
        g += np.sin(2 * np.pi * (kv[0] * ii[0] + kv[1] * ii[1] + kv[2] * ii[2]) / n + rng.uniform(0, 2 * np.pi))
    g += rng.normal(0.0, 1e-3, g.shape)
    return g.astype(np.float32)


def composed_fixtures(R, rng):
    """ComposedRefactor -> progressive ComposedReconstructor, hierarchical basis."""
    out = {}
    shape, L, B = (33, 33, 33), 3, 32
    g = sinusoid_field(rng, 33)
    vr = float(g.max() - g.min())
    tols = np.array([vr * t for t in (1e-1, 1e-3, 1e-5)])
    out["field"] = g
    out["tols"] = tols
    for enc in ("grouped", "negabinary"):
        with tempfile.TemporaryDirectory() as d:
            outs, ret = R.composed(g, L, B, enc, True, tols, d)
            levels = [np.frombuffer(open(os.path.join(d, "level_%d.bin" % i), "rb").read(), np.uint8)
                      for i in range(L + 1)]
            meta = np.frombuffer(open(os.path.join(d, "metadata.bin"), "rb").read(), np.uint8)
        out[enc + "_levels"] = np.concatenate(levels)
        out[enc + "_level_bytes"] = np.array([len(x) for x in levels], np.int64)
        out[enc + "_metadata"] = meta
        out[enc + "_recon"] = outs
        out[enc + "_retrieved"] = ret
    return out


def qoi_fixtures(R, rng):
    """GE quantities of interest and their error estimates from the reference's
    qoi_utils.hpp (QoI::compute_QoIs and the propagation rules), fp64. Edge
    points: zero velocity (sqrt rule at x == 0), velocities below the bound
    (x <= eb branch), densities whose bound reaches |D| (no bound: 0) and
    negative densities (the other branch of the division rule)."""
    n = 4096
    vx, vy, vz = (rng.normal(0.0, 50.0, n) for _ in range(3))
    p = rng.uniform(0.5e5, 1.5e5, n)
    d = rng.uniform(0.5, 1.5, n)
    vx[:4] = vy[:4] = vz[:4] = 0.0
    vx[4:8], vy[4:8], vz[4:8] = 1e-3, -2e-3, 5e-4
    d[8:12] = [0.05, -0.05, 0.1, -0.5]
    out = {"vx": vx, "vy": vy, "vz": vz, "p": p, "d": d}
    for k, v in zip(("vtot", "temp", "c", "mach", "pt", "mu"), R.qoi_values(vx, vy, vz, p, d)):
        out[k] = v
    out["ebs_v"] = np.array([0.5, 0.25, 1.0])
    out["bound_vtot"] = R.qoi_vtot_bound(vx, vy, vz, out["ebs_v"])
    out["eb_pd"] = np.array([100.0, 0.1])
    out["bound_t"] = R.qoi_t_bound(p, d, 100.0, 0.1)
    return out


def lossless_fixtures(R, rng):
    """AdaptiveLevelCompressor (zstd level 3) on the encoder and per-bit fixture
    levels (read from encoders.npz / perbit.npz): its stopping index, the sizes
    it leaves and every stream's zstd size, for latter indices 26 (default),
    3 and 40."""
    out = {}
    cases = []
    for name in ("encoders", "perbit"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        for c in g["cases"]:
            c = str(c)
            blob, sizes = g[c + "_blob"], g[c + "_sizes"]
            for latter in (26, 3, 40):
                stop, left, zs = R.adaptive_compress(blob, sizes, latter)
                key = "%s_%s_L%d" % (name, c, latter)
                out[key + "_raw"] = sizes
                out[key + "_zstd"] = zs
                out[key + "_left"] = left
                out[key + "_stop"] = np.int32(stop)
                out[key + "_latter"] = np.int32(latter)
                cases.append(key)
    out["cases"] = np.array(cases)
    return out


PB_N = (1, 2, 31, 32, 33, 63, 64, 65, 95, 127, 729, 4184)


def perbit_fixtures(R, rng):
    """PerBitBPEncoder<T, uint32_t> (the GE applications' encoder): streams and
    sizes, and the progressive decode in three steps ([0, s1), [s1, s2),
    [s2, B)) through one decoder object; then a ComposedRefactor ->
    ComposedReconstructor round trip with it (fp64, 60 planes, hierarchical
    basis, SignExclude greedy interpreter, MaxErrorEstimatorHB). fp64 stops at
    63 planes: at 64 the level-max element scales to >= 2^63, whose int64
    conversion in the reference is undefined (it differs between x86 and Arm)."""
    out = {}
    cases = []
    for dt, Bs in ((np.float32, (2, 8, 32)), (np.float64, (2, 33, 60, 63))):
        for n in PB_N:
            for B in Bs:
                scale = float(rng.choice([1e-3, 1.0, 1e3]))
                x = coeff_like(rng, n, dt, scale)
                if n >= 8:
                    x[5] = -np.abs(x).max()                # the level-max element, negative
                    x[6] = np.ldexp(dt(1.0), -40)          # below the last plane
                mx = float(np.max(np.abs(x)))
                e = math.frexp(mx)[1] if mx > 0 else 0
                blob, sizes = R.pb_encode(x, e, B)
                dec = R.perbit_state(dt)
                s1, s2 = max(1, B // 3), max(1, B // 3) + max(1, B // 4)
                s2 = min(s2, B)
                offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
                key = "%s_n%d_B%d" % (np.dtype(dt).name, n, B)
                steps = [(0, s1), (s1, s2), (s2, B)]
                for i, (a, b) in enumerate(steps):
                    out["%s_dec%d" % (key, i)] = dec.decode(blob[offs[a]:offs[b]], sizes[a:b], n, e, a, b - a, 0)
                out[key + "_x"] = x
                out[key + "_exp"] = np.int32(e)
                out[key + "_blob"] = blob
                out[key + "_sizes"] = sizes
                out[key + "_steps"] = np.array(steps, np.int32)
                cases.append(key)
    out["cases"] = np.array(cases)
    shape, L, B = (17, 17, 17), 3, 60
    g = sinusoid_field(rng, 17).astype(np.float64) * 1e3
    vr = float(g.max() - g.min())
    tols = np.array([vr * t for t in (1e-2, 1e-5, 1e-9)])
    with tempfile.TemporaryDirectory() as d:
        outs, ret = R.composed(g, L, B, "perbit", True, tols, d)
        levels = [np.frombuffer(open(os.path.join(d, "level_%d.bin" % i), "rb").read(), np.uint8)
                  for i in range(L + 1)]
        meta = np.frombuffer(open(os.path.join(d, "metadata.bin"), "rb").read(), np.uint8)
    out["composed_field"] = g
    out["composed_tols"] = tols
    out["composed_levels"] = np.concatenate(levels)
    out["composed_level_bytes"] = np.array([len(x) for x in levels], np.int64)
    out["composed_metadata"] = meta
    out["composed_recon"] = outs
    out["composed_retrieved"] = ret
    return out


FIXTURES = (("encoders", encoder_fixtures), ("collectors", collector_fixtures),
            ("interpreters", interpreter_fixtures), ("geometry", geometry_fixtures),
            ("composed", composed_fixtures), ("qoi", qoi_fixtures), ("perbit", perbit_fixtures),
            ("lossless", lossless_fixtures))

OWN_SEED = {"qoi": 20241203, "perbit": 20241204, "lossless": 0}   # fixtures with their own random stream


def main(names=None):
    """Regenerate the named fixture files (all by default)."""
    R = oracle.reference()
    if R is None:
        raise SystemExit("the reference harness is unavailable here; fixtures cannot be regenerated")
    shared = np.random.default_rng(20240611)    # the first five draw from one stream, in order
    for name, fn in FIXTURES:
        rng = np.random.default_rng(OWN_SEED[name]) if name in OWN_SEED else shared
        if names and name not in names:
            if name not in OWN_SEED:
                fn(R, rng)                         # keep the shared stream in step
            continue
        d = fn(R, rng)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **d)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1:] or None)
