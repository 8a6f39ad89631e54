"""Small, self-contained workload for kernel profiling (ncu) and quick timing.

    python -m prodm_gb300.profile_case --shape 257 --levels 7 --reps 3

Runs `reps` refactor + progressive-retrieve steps of a seeded Gaussian random
field (k^-5/3) with the benchmark's component set (NegaBinary, 32 planes,
hierarchical basis, squared-error tables, relative L2 tolerances 1e-2..1e-6)
and prints per-stage CUDA-event times of the last step. With --encoder perbit
the step is the GE applications' configuration instead: a seeded fp64 tanh
shear layer (+1e-6 relative noise), 60 planes, max collector, SignExclude
interpreter with MaxErrorEstimatorHB, relative L-inf tolerances 1e-3..1e-9.
With --basis orthogonal: the orthogonal MGARD basis on the same fp64 shear
layer with the grouped encoder, 60 planes, max collector, SignExclude
interpreter with MaxErrorEstimatorOB and relative L-inf tolerances 1e-3,
1e-6, 1e-9. --shape takes one edge (a cube) or AxBxC. With --batch N: a
batch of N 257^3 and four 129x257x65 spectral fields (slope -2, largest
level counts, 32 planes, negabinary, relative L-inf 1e-3) refactored and
retrieved `reps` times through MDRBatch, with fixed launch shapes (no
autotuning). With --batch-config4: the benchmark's 64-field batch (24 cubes,
24 2-D fields, 16 anisotropic fields; relative L-inf tolerances 1e-5..1e-2)
with the same fixed launch shapes.
"""
import argparse
import math

import torch

from . import api, fields


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="257", help="edge of a cube, or AxBxC")
    ap.add_argument("--levels", type=int, default=None)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--encoder", default="negabinary")
    ap.add_argument("--basis", default="hierarchical")
    ap.add_argument("--lossless", action="store_true",
                    help="after the steps, the lossless stage on the finest level's streams: compress + decompress")
    ap.add_argument("--import-streams", action="store_true",
                    help="per-bit only: export the level files and load them into a second handle (the parse)")
    ap.add_argument("--batch", type=int, default=0,
                    help="N > 0: a batch of N 257^3 and four 129x257x65 fields instead of one field")
    ap.add_argument("--batch-config4", action="store_true", help="the benchmark's 64-field batch")
    a = ap.parse_args()
    if a.batch or a.batch_config4:
        return batch(a.batch, a.reps, a.batch_config4)
    dims = tuple(int(v) for v in a.shape.split("x"))
    shape = dims * 3 if len(dims) == 1 else dims
    if a.basis == "orthogonal":
        L = a.levels if a.levels is not None else api.max_level(shape)
        return orthogonal(shape, L, a.reps)
    L = a.levels if a.levels is not None else min(7, api.max_level(shape))
    if a.encoder == "perbit":
        return perbit(shape, L, a.reps, a.import_streams)
    x = fields.spectral_grf(shape, seed=3)
    norm2 = float((x.double() ** 2).sum().item())
    mdr = api.MDRField(shape, torch.float32, L, 32, a.encoder, a.basis, "squared")
    out = torch.empty_like(x)
    interp = "negabinary" if a.encoder == "negabinary" else "greedy"
    for r in range(a.reps):
        if r == a.reps - 1:
            mdr.set_timing(True)
        mdr.refactor(x)
        mdr.reset()
        for rel in (1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
            mdr.retrieve(rel * rel * norm2, out=out, interpreter=interp, estimator="l2_hb")
    torch.cuda.synchronize()
    err = math.sqrt(float(((out.double() - x.double()) ** 2).sum().item()) / norm2)
    for (kind, level), (ms, n) in sorted(mdr.stage_times().items(), key=lambda kv: -kv[1][0]):
        print("%-10s l%-2d %8.4f ms over %d launches" % (kind, level, ms, n))
    print("final relative L2 error %.3g" % err)
    if a.lossless:
        sizes, _, _ = mdr.level_info()
        blob = mdr.export_level_device(L)
        comp, csz, stop = api.compress_level(blob, sizes[L], 26)
        back, _ = api.decompress_level(comp, csz, 0, len(csz), stop, 26, raw_capacity=blob.numel() + 16)
        torch.cuda.synchronize()
        print("lossless: level %d %d -> %d bytes, stopping index %d, round trip %s"
              % (L, blob.numel(), comp.numel(), stop, bool(torch.equal(back, blob))))


def perbit(shape, L, reps, import_streams=False):
    x = fields.shear_layer(shape, delta=0.05, noise_rel=1e-6, seed=21, dtype=torch.float64, device="cuda")
    vr = float((x.max() - x.min()).item())
    mdr = api.MDRField(shape, torch.float64, L, 60, "perbit", "hierarchical", "max")
    out = torch.empty_like(x)
    for r in range(reps):
        if r == reps - 1:
            mdr.set_timing(True)
        mdr.refactor(x)
        mdr.reset()
        for rel in (1e-3, 1e-5, 1e-7, 1e-9):
            mdr.retrieve(rel * vr, out=out, interpreter="sign_exclude", estimator="max_hb")
    torch.cuda.synchronize()
    for (kind, level), (ms, n) in sorted(mdr.stage_times().items(), key=lambda kv: -kv[1][0]):
        print("%-10s l%-2d %8.4f ms over %d launches" % (kind, level, ms, n))
    print("final max error %.3g of range %.3g" % (float((out - x).abs().max().item()), vr))
    if import_streams:
        files = [mdr.export_level(l) for l in range(L + 1)]
        r = api.MDRField(shape, torch.float64, L, 60, "perbit", "hierarchical", "max")
        r.load_metadata(mdr.metadata())
        for l in range(L + 1):
            r.load_level(l, files[l], 0)
        full = r.retrieve_planes([60] * (L + 1))
        ref = mdr.retrieve_planes([60] * (L + 1))
        torch.cuda.synchronize()
        print("imported streams reconstruct identically: %s" % bool(torch.equal(full, ref)))


def orthogonal(shape, L, reps):
    x = fields.shear_layer(shape, delta=0.05, noise_rel=1e-6, seed=9, dtype=torch.float64, device="cuda")
    vr = float((x.max() - x.min()).item())
    mdr = api.MDRField(shape, torch.float64, L, 60, "grouped", "orthogonal", "max")
    out = torch.empty_like(x)
    for r in range(reps):
        if r == reps - 1:
            mdr.set_timing(True)
        mdr.refactor(x)
        mdr.reset()
        for rel in (1e-3, 1e-6, 1e-9):
            mdr.retrieve(rel * vr, out=out, interpreter="sign_exclude", estimator="max_ob")
    torch.cuda.synchronize()
    for (kind, level), (ms, n) in sorted(mdr.stage_times().items(), key=lambda kv: -kv[1][0]):
        print("%-10s l%-2d %8.4f ms over %d launches" % (kind, level, ms, n))
    print("final max error %.3g of range %.3g" % (float((out - x).abs().max().item()), vr))


def batch(n, reps, config4=False):
    if config4:
        xs, tols, levels = [], [], []
        for i, (shape, slope, rel) in enumerate(fields.batch_specs(seed=7)):
            x = fields.spectral_grf(shape, slope=slope, seed=500 + i)
            xs.append(x)
            tols.append(rel * float(x.max() - x.min()))
            levels.append(fields.batch_level(shape, api.max_level(shape)))
    else:
        shapes = [(257, 257, 257)] * n + [(129, 257, 65)] * 4
        xs = [fields.spectral_grf(s, slope=-2.0, seed=900 + i) for i, s in enumerate(shapes)]
        tols = [1e-3 * float(x.max() - x.min()) for x in xs]
        levels = [fields.batch_level(s, api.max_level(s)) for s in shapes]
    b = api.MDRBatch(xs, levels, 32)
    for stage, shape in (("decompose", (256, 8)), ("encode", (256, 8)), ("recompose", (256, 4)), ("fused", (256, 5))):
        b.set_stage_launch(stage, *shape)
    b.set_tolerances(tols)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for r in range(reps):
        e0.record()
        b.refactor()
        b.reset()
        b.retrieve("negabinary", "max_hb")
        e1.record()
    torch.cuda.synchronize()
    b.status()
    print("batch of %d fields: last refactor + retrieve %.4f ms" % (len(xs), e0.elapsed_time(e1)))


if __name__ == "__main__":
    main()
