"""Benchmark: MDR refactor + progressive retrieve throughput at 513^3 fp32.

One step = refactor of a 513^3 fp32 Gaussian random field (power spectrum
k^-5/3, seeded; 8 levels, 32 bitplanes, NegaBinary encoder, squared-error
tables) followed by retrieval at relative L2 tolerances 1e-2 .. 1e-6
(negabinary greedy interpreter, L2 hierarchical estimator), progressive from
an empty retrieval state.

Algorithmic bytes of a step (the metric's numerator):
  refactor : field read once (N*4) + every stream byte written once
  retrieve : the stream bytes of all retrieved planes + the field written (N*4),
             per tolerance.
value  = bytes of all ranks' steps / max-over-ranks device time (GB/s), inputs
         resident in HBM; every input is larger than L2 (129 MB), no flush.
e2e    = same bytes / time of the reference-facing flow with host buffers:
         H2D field -> refactor -> D2H level files + metadata -> reconstructor
         loads metadata, then per tolerance: interpret, H2D of the newly needed
         level bytes, reconstruct, D2H of the field.

--impl reference: the reference's CPU algorithm on all host threads, each
thread refactoring + retrieving its own 257^3 field with 7 levels (8 levels at
257^3 would leave a 27-value level 0, which the reference's encoders reject),
the same bitplanes, encoder, tables and tolerances: a bounded sample of this
workload, reported on the same config; a one-thread figure of the same sample
is reported beside it.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = (513, 513, 513)
LEVELS = 7              # target level 7 = 8 levels
BITPLANES = 32
REL_TOLS = (1e-2, 1e-3, 1e-4, 1e-5, 1e-6)
CPU_SAMPLE = (257, 257, 257)
CPU_LEVELS = 6          # target level 6 = 7 levels: level 0 = 5^3 values (>= one 32-value block)
METRIC = "refactor & retrieve GB/s at 513^3 fp32 (% HBM roofline), batched vs plain, at stated bound"
WORKLOAD = ("513^3 fp32 Gaussian random field k^-5/3 (seeded), 8 levels, 32 bitplanes, NegaBinaryBPEncoder, "
            "SquaredErrorCollector tables, MGARD hierarchical basis; retrieve at relative L2 1e-2..1e-6 "
            "(progressive, NegaBinary greedy interpreter, L2 hierarchical estimator)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", dest="graph", action="store_false",
                    help="time host launches of the step instead of replaying it as a captured CUDA graph (the "
                         "default: captured without stage events; stage times come from the instrumented pass after "
                         "the timed region)")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-field batched vs per-field-loop measurement")
    ap.add_argument("--no-qoi", action="store_true", help="skip the QoI-guided vs uniform-halving retrieval comparison")
    ap.add_argument("--no-perbit", action="store_true", help="skip the fp64 per-bit encoder measurement")
    ap.add_argument("--no-lossless", action="store_true", help="skip the lossless-stage measurement")
    ap.add_argument("--no-files", action="store_true", help="skip the level-file read / write measurement")
    ap.add_argument("--no-ortho", action="store_true", help="skip the fp64 orthogonal-basis configuration")
    return ap.parse_args()


def replica_throughput(ms_local, step_bytes, steps, world, device):
    """Whole-job throughput of `world` replicas that each processed `steps`
    steps of `step_bytes` in ms_local: the slowest rank's time (max over
    ranks, one all-reduce) against all ranks' bytes. Returns (ms, GB/s)."""
    ms = float(ms_local)
    if world > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    return ms, step_bytes * steps * world / (ms / 1e3) / 1e9


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.time(), line.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = []
        for ts, line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((ts, float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        inside = [r for r in rows if t0 <= r[0] <= t1 + 0.15]
        if not inside and rows:
            inside = sorted(rows, key=lambda r: min(abs(r[0] - t0), abs(r[0] - t1)))[:3]
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[1] for r in inside), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": reasons, "samples": len(inside)}


def config():
    """The workload both arms report (the reference arm times a bounded sample of it)."""
    return {"workload": WORKLOAD, "shape": list(SHAPE), "levels": LEVELS + 1, "bitplanes": BITPLANES,
            "encoder": "negabinary", "basis": "hierarchical", "rel_l2_tolerances": list(REL_TOLS),
            "parallelism": "replicas (one independent field per GPU)",
            "l2_policy": "inputs (540 MB field, 540 MB streams) larger than L2; no flush"}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU baseline: the reference's algorithm on host threads
# ---------------------------------------------------------------------------
def cpu_sample_field(seed):
    import numpy as np
    rng = np.random.default_rng(seed)
    # spectral field of the same slope, host generator (numpy FFT)
    n = CPU_SAMPLE[0]
    white = rng.standard_normal(CPU_SAMPLE).astype(np.float32)
    spec = np.fft.rfftn(white)
    k = [np.fft.fftfreq(n) * n, np.fft.fftfreq(n) * n, np.fft.rfftfreq(n) * n]
    kk = k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2 + k[2][None, None, :] ** 2
    kk[0, 0, 0] = 1.0
    spec *= kk ** (-5.0 / 12.0)
    spec[0, 0, 0] = 0
    x = np.fft.irfftn(spec, s=CPU_SAMPLE, axes=(0, 1, 2)).astype(np.float32)
    x /= x.std()
    return x


def cpu_libraries():
    """(reference harness or None, oracle), loaded once before threads start."""
    import oracle
    return oracle.reference(), oracle.oracle()


def cpu_work(x, libs):
    """One bounded sample: refactor + progressive retrieval at the five
    tolerances, on the reference's own classes when its harness is built
    (oracle/_ref), else on the oracle's restatement. Returns (bytes, kind)."""
    import numpy as np
    L, B = CPU_LEVELS, BITPLANES
    norm2 = float(np.sum(x.astype(np.float64) ** 2))
    tols = [(rel ** 2) * norm2 for rel in REL_TOLS]
    R, O = libs
    if R is not None:
        return R.headline_step(x, L, B, tols), "reference"
    r = O.refactor(x, L, B, "negabinary", True, True)
    nbytes = x.size * 4 + r["blob"].size
    idx = np.zeros(L + 1, np.uint8)
    for tol in tols:
        idx, _ = O.interpret("negabinary", "l2_hb", r["sizes"], r["errs"], tol, idx)
        O.retrieve(x.shape, L, B, r["blob"], r["sizes"], r["bounds"], idx, "negabinary", True)
        nbytes += int(sum(int(r["sizes"][l, :idx[l]].astype(np.int64).sum()) for l in range(L + 1))) + x.size * 4
    return nbytes, "port"


def cpu_baseline(steps, warmup, threads=None):
    threads = threads or os.cpu_count() or 1
    base = cpu_sample_field(100)
    fields = [base] * threads            # read-only input; each refactor works on its own copy
    results = [0] * threads
    kinds = ["port"] * threads
    errors = []
    libs = cpu_libraries()

    def run(t):
        try:
            results[t], kinds[t] = cpu_work(fields[t], libs)
        except Exception as e:   # reported after the join
            errors.append(repr(e))

    total_bytes, total_time = 0, 0.0
    for s in range(warmup + steps):
        ths = [threading.Thread(target=run, args=(t,)) for t in range(threads)]
        t0 = time.perf_counter()
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        dt = time.perf_counter() - t0
        if errors:
            raise RuntimeError("CPU baseline failed: " + errors[0])
        if s >= warmup:
            total_bytes += sum(results)
            total_time += dt
    return total_bytes / total_time / 1e9, threads, total_time / max(steps, 1), kinds[0]


def cpu_sample_text(cores, kind):
    who = ("the reference's own encoder, interleaver, interpreter and estimator classes compiled from its headers"
           if kind == "reference" else "the reference's CPU algorithm as restated by the oracle")
    return ("each step: each of %d host threads refactors its own 257^3 fp32 Gaussian random field (7 levels: 8 "
            "would leave a 27-value level 0, which the reference's encoders reject; 32 planes, NegaBinary, squared "
            "tables) and retrieves it at relative L2 1e-2..1e-6; %s" % (cores, who))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
FUSED_LEVELS = 2   # the library's kFusedLevels


def fused_from(level_dims, L):
    """Lowest level decoded inside its recomposition (the library's rule for
    fp32 negabinary hierarchical handles: the finest level, and the levels
    below it down to FUSED_LEVELS in all while a level's plane has at least
    4096 rows)."""
    rows = [int(d[0]) * int(d[1]) for d in level_dims]
    if rows[L] < 1024:
        return L + 1
    f = L
    while f - 1 >= 1 and L - (f - 1) < FUSED_LEVELS and rows[f - 1] >= 4096:
        f -= 1
    return f


def stage_bytes(mdr, kind, level, step_bytes_info):
    """algorithmic bytes of one launch of a stage: what the stage must read and write."""
    import numpy as np
    ld = mdr.level_dims
    box = lambda l: int(np.prod(ld[l].astype(np.int64)))
    n = int(mdr.level_elements[level])
    sizes = step_bytes_info["sizes"]
    if kind == "decompose":
        return 2 * 4 * box(level)
    if kind == "encode":
        levels = [level]
        if level == step_bytes_info["L"] and step_bytes_info.get("encode_multi"):
            levels = range(0, level + 1)     # one launch encodes every level
        return sum(4 * int(mdr.level_elements[l]) + int(sizes[l].astype(np.int64).sum()) for l in levels)
    ffrom = step_bytes_info.get("fused_from", step_bytes_info["L"] + 1)
    if kind == "decode":
        levels = [level]
        if level == 0 and step_bytes_info.get("decode_multi"):
            # one launch decodes every level the fused kernel does not
            levels = range(0, ffrom)
        return sum(step_bytes_info["decode_bytes"][l] + 4 * int(mdr.level_elements[l]) for l in levels)
    if kind == "recompose":
        if level >= ffrom:
            # fused level: its retrieved planes are read instead of coefficients
            return step_bytes_info["decode_bytes"][level] + 4 * (box(level - 1) + box(level))
        return 4 * (box(level - 1) + n + box(level))
    return 0


def run_ours(args):
    import numpy as np
    import torch
    from prodm_gb300 import api, fields

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)

    x = fields.spectral_grf(SHAPE, slope=-5.0 / 3.0, seed=1234 + rank, dtype=torch.float32, device=dev)
    N = x.numel()
    norm2 = float((x.double() ** 2).sum().item())
    tols = [(r ** 2) * norm2 for r in REL_TOLS]
    mdr = api.MDRField(SHAPE, torch.float32, LEVELS, BITPLANES, "negabinary", "hierarchical", "squared")
    out = torch.empty(SHAPE, dtype=torch.float32, device=dev)

    def step():
        mdr.refactor(x)
        mdr.reset()
        for t in tols:
            mdr.retrieve(t, out=out, interpreter="negabinary", estimator="l2_hb")

    # warm-up, and the per-tolerance retrieved bytes (deterministic)
    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize()
    sizes, bounds, _ = mdr.level_info()
    mdr.refactor(x)
    mdr.reset()
    retrieved, achieved, idxs = [], [], []
    for t in tols:
        mdr.retrieve(t, out=out, interpreter="negabinary", estimator="l2_hb")
        idx = mdr.index()
        idxs.append(idx.tolist())
        retrieved.append(mdr.retrieved_bytes(idx))
        achieved.append(math.sqrt(float(((out.double() - x.double()) ** 2).sum().item()) / norm2))
    refactor_bytes = N * 4 + int(sizes.astype(np.int64).sum())
    retrieve_bytes = [r + N * 4 for r in retrieved]
    step_bytes = refactor_bytes + sum(retrieve_bytes)
    decode_bytes = [sum(int(sizes[l, :idxs[i][l]].astype(np.int64).sum()) for i in range(len(tols))) / len(tols)
                    for l in range(LEVELS + 1)]

    # one step captured as a CUDA graph (the interpreter's plane counts stay on
    # the device, so the whole refactor + retrieve sequence is capturable; the
    # kernels' programmatic launch dependencies become graph edges). Measured
    # at 513^3: 2.843 ms per replayed step against 2.874 ms with host launches.
    graph = None
    launches_per_step = None
    if args.graph:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        l0 = api.kernel_launch_count()
        with torch.cuda.graph(graph):
            step()
        launches_per_step = api.kernel_launch_count() - l0
        graph.replay()
        torch.cuda.synchronize()

    # timed region
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = api.kernel_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    e0.record()
    for i in range(args.steps):
        if graph is not None:
            graph.replay()
        else:
            step()
    e1.record()
    torch.cuda.synchronize()
    t1 = time.time()
    if world > 1:
        dist.barrier()
    launches = (launches_per_step * args.steps) if graph is not None else api.kernel_launch_count() - launches0
    ms = e0.elapsed_time(e1)
    sampler.stop()
    clocks = sampler.summary(t0, t1)
    ms, value = replica_throughput(ms, step_bytes, args.steps, world, dev)

    # per-stage times come from a separate instrumented pass after the timed
    # region (stage events keep kernels from overlapping their neighbours, so
    # they stay out of the headline number)
    stage_steps = min(args.steps, 10)
    mdr.set_timing(True)
    ei0 = torch.cuda.Event(enable_timing=True)
    ei1 = torch.cuda.Event(enable_timing=True)
    ei0.record()
    for _ in range(stage_steps):
        step()
    ei1.record()
    torch.cuda.synchronize()
    ms_instrumented = ei0.elapsed_time(ei1) / stage_steps
    stages = mdr.stage_times()
    mdr.set_timing(False)

    # roofline of the dominant stage
    peak, peak_src = measured_peak()
    info = {"sizes": sizes, "decode_bytes": decode_bytes, "L": LEVELS,
            "fused_from": fused_from(mdr.level_dims, LEVELS) if ("decode", LEVELS) not in stages else LEVELS + 1,
            "decode_multi": ("decode", 1) not in stages, "encode_multi": ("encode", 0) not in stages}
    per_stage = {}
    for (kind, level), (tms, cnt) in stages.items():
        b = stage_bytes(mdr, kind, level, info)
        per_stage["%s_l%d" % (kind, level)] = {"ms_avg": tms / cnt, "launches": cnt, "share": 0.0,
                                               "gbs": (b / (tms / cnt / 1e3) / 1e9) if tms > 0 and b else None,
                                               "bytes": b}
    tot = sum(v["ms_avg"] * v["launches"] for v in per_stage.values()) or 1.0
    for v in per_stage.values():
        v["share"] = v["ms_avg"] * v["launches"] / tot
    dom_name = max(per_stage, key=lambda k: per_stage[k]["ms_avg"] * per_stage[k]["launches"])
    dom = per_stage[dom_name]
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_513.txt")) as f:
            for line in f:
                parts = line.split()
                if len(parts) == 2 and not line.startswith("#") and parts[0] == dom_name:
                    traffic = float(parts[1])
    except OSError:
        pass
    roofline = {"kernel": dom_name, "bound": "hbm", "achieved": dom["gbs"], "peak": peak, "unit": "GB/s",
                "frac": (dom["gbs"] / peak) if dom["gbs"] else None, "traffic": traffic,
                "peak_source": peak_src + " (hbm_gbs, copy bandwidth)",
                "algorithmic_bytes_per_launch": dom["bytes"]}

    batched = run_batched() if (not args.no_batched and world == 1) else None
    qoi_res = run_qoi() if (not args.no_qoi and world == 1) else None
    perbit = run_perbit() if (not args.no_perbit and world == 1) else None
    lossless = run_lossless() if (not args.no_lossless and world == 1) else None
    files = run_files() if (not args.no_files and world == 1) else None
    ortho = run_ortho() if (not args.no_ortho and world == 1) else None

    # end-to-end through the reference-facing flow with host buffers
    e2e = run_e2e(args, mdr, x, tols, refactor_bytes, step_bytes, dev) if args.e2e_steps > 0 else None

    result = None
    if rank == 0:
        result = {
            "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian random field, k^-5/3)",
            "config": config(),
            "run": {"bytes_per_step": step_bytes, "refactor_bytes": refactor_bytes,
                    "retrieve_bytes": retrieve_bytes, "achieved_rel_l2": achieved, "planes_per_level": idxs,
                    "ms_per_step_instrumented": ms_instrumented, "instrumented_steps": stage_steps},
            "roofline": roofline,
            "stages": per_stage,
            "gpu_launches": launches,
            "execution": "CUDA graph replay of one captured step" if graph is not None else "host launches",
            "e2e": e2e,
            "batched": batched,
            "qoi": qoi_res,
            "perbit": perbit,
            "lossless": lossless,
            "files": files,
            "ortho": ortho,
            "clocks": clocks,
        }
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return result


def run_e2e(args, mdr, x, tols, refactor_bytes, step_bytes, dev):
    import numpy as np
    import torch
    from prodm_gb300 import api

    L = LEVELS
    host_field = torch.empty(SHAPE, dtype=torch.float32, pin_memory=True)
    host_field.copy_(x.cpu())
    host_out = torch.empty(SHAPE, dtype=torch.float32, pin_memory=True)
    dfield = torch.empty_like(x)
    # each reconstruction is copied to the host on a side stream while the
    # next one is computed (two device outputs in turn)
    outs = [torch.empty_like(x), torch.empty_like(x)]
    side = torch.cuda.Stream()
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    rec = api.MDRField(SHAPE, torch.float32, L, BITPLANES, "negabinary", "hierarchical", "squared")
    sizes, _, _ = mdr.level_info()
    level_bytes = [int(sizes[l].astype(np.int64).sum()) for l in range(L + 1)]
    host_levels = [torch.empty(b, dtype=torch.uint8, pin_memory=True) for b in level_bytes]
    # the level files go to the host on their own stream while the
    # reconstructor loads what it needs of each level as soon as those bytes
    # have arrived (the host link carries both directions at once): the coarse
    # levels first, then the part of the finest level the first tolerance
    # needs, then the rest of it
    exp_stream = torch.cuda.Stream()
    exported = [torch.cuda.Event() for _ in range(L + 1)]
    head = torch.cuda.Event()
    h2d = d2h = 0

    def needed(idx, l):
        return int(sizes[l, :idx[l]].astype(np.int64).sum())

    def one():
        nonlocal h2d, d2h
        h2d = d2h = 0
        main = torch.cuda.current_stream()
        dfield.copy_(host_field, non_blocking=True)
        h2d += x.numel() * 4
        mdr.refactor(dfield)
        meta = mdr.metadata()
        d2h += len(meta)
        exp_stream.wait_stream(main)
        for l in range(L):                                  # coarse level files -> host
            mdr.export_level_into(l, host_levels[l], exp_stream)
            exported[l].record(exp_stream)
            d2h += level_bytes[l]
        rec.load_metadata(meta)
        rec.interpret(tols[0], interpreter="negabinary", estimator="l2_hb")
        idx = rec.index()
        first = needed(idx, L)                              # finest level file, in two parts
        if 0 < first < level_bytes[L]:
            mdr.export_level_range_into(L, 0, host_levels[L][:first], exp_stream)
            head.record(exp_stream)
            mdr.export_level_range_into(L, first, host_levels[L][first:], exp_stream)
        else:
            mdr.export_level_into(L, host_levels[L], exp_stream)
            head.record(exp_stream)
        exported[L].record(exp_stream)
        d2h += level_bytes[L]
        loaded = [0] * (L + 1)
        for i, t in enumerate(tols):
            if i:
                rec.interpret(t, interpreter="negabinary", estimator="l2_hb")
                idx = rec.index()
            for l in range(L + 1):
                need = needed(idx, l)
                if need > loaded[l]:
                    main.wait_event(head if l == L and need <= first else exported[l])
                    rec.load_level(l, host_levels[l][loaded[l]:need], offset=loaded[l])
                    h2d += need - loaded[l]
                    loaded[l] = need
            k = i & 1
            if i >= 2:
                main.wait_event(copied[k])          # the host copy of outs[k] has finished
            rec.reconstruct(outs[k])
            side.wait_stream(main)
            with torch.cuda.stream(side):
                host_out.copy_(outs[k], non_blocking=True)
                copied[k].record(side)
            d2h += x.numel() * 4
        side.synchronize()
        main.synchronize()
        exp_stream.synchronize()

    one()
    torch.cuda.synchronize()
    n = args.e2e_steps
    t0 = time.perf_counter()
    for _ in range(n):
        one()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / n
    rec.close()
    return {"value": step_bytes / dt / 1e9, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": dt * 1e3, "steps": n,
            "flow": "H2D field, refactor, D2H metadata; D2H level files (own stream, pinned, asynchronous: "
                    "coarse levels, then the finest level's bytes the first tolerance needs, then the rest); "
                    "reconstructor: load metadata, per tolerance interpret -> H2D of the new level bytes (each "
                    "part once it is on the host) -> reconstruct -> D2H field (side stream, overlapping the next "
                    "tolerance)"}


def run_batched(steps=5):
    """64 uneven fp32 fields refactored + retrieved per step: one batched CUDA
    graph (persistent multi-field launches, autotuned launch shape) against
    the plain per-field loop (one device pipeline per field, host launches).
    Both compute identical results; bytes counted as for the single field."""
    import numpy as np
    import torch
    from prodm_gb300 import api, autotune, fields

    specs = fields.batch_specs(seed=7)
    xs, tols, levels = [], [], []
    for i, (shape, slope, rel) in enumerate(specs):
        x = fields.spectral_grf(shape, slope=slope, seed=500 + i)
        xs.append(x)
        tols.append(rel * float(x.max() - x.min()))
        levels.append(fields.batch_level(shape, api.max_level(shape)))
    batch = api.MDRBatch(xs, levels, BITPLANES)
    tuned = autotune.tune(batch, reps=2)
    batch.set_tolerances(tols)

    def bstep():
        batch.refactor()
        batch.reset()
        batch.retrieve("negabinary", "max_hb")

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        bstep()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        bstep()
    g.replay()
    torch.cuda.synchronize()
    nbytes = 0
    for i, x in enumerate(xs):
        idx, sz, _ = batch.field_info(i)
        nbytes += 2 * x.numel() * 4 + int(sz.astype(np.int64).sum())
        nbytes += int(sum(int(sz[l, :idx[l]].astype(np.int64).sum()) for l in range(len(idx))))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1) / steps

    singles = [api.MDRField(x.shape, torch.float32, levels[i], BITPLANES, "negabinary", "hierarchical", "max")
               for i, x in enumerate(xs)]
    outs = [torch.empty_like(x) for x in xs]

    def pstep():
        for i, m in enumerate(singles):
            m.refactor(xs[i])
            m.reset()
            m.retrieve(tols[i], out=outs[i], interpreter="negabinary", estimator="max_hb")

    pstep()
    torch.cuda.synchronize()
    same = all(torch.equal(a, b) for a, b in zip(outs, batch.outs))
    e0.record()
    for _ in range(steps):
        pstep()
    e1.record()
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1) / steps
    for m in singles:
        m.close()
    batch.close()
    return {"fields": len(xs), "bytes_per_step": nbytes, "ms_batched": ms_b, "ms_plain_loop": ms_p,
            "batched_gbs": nbytes / (ms_b / 1e3) / 1e9, "plain_loop_gbs": nbytes / (ms_p / 1e3) / 1e9,
            "speedup": ms_p / ms_b, "identical_results": bool(same),
            "autotuned_launch": {k: {"threads_per_cta": v[0], "ctas_per_sm": v[1]} for k, v in tuned[0].items()
                                 if k != "fused_unit"},
            "autotuned_fused_unit_values": tuned[0].get("fused_unit", (None,))[0],
            "workload": "24 cubes {33,65,129,257}^3, 24 2-D {513,1025,2049}^2, 16 x 129x257x65; spectral slopes "
                        "U[-3,-1]; levels = largest keeping level 0 >= 32 values; 32 planes; negabinary; "
                        "relative L-inf tolerances log-U[1e-5,1e-2]; refactor + retrieve per step"}


def run_qoi(n=257, levels=6, rels=(1e-2, 1e-3, 1e-4)):
    """QoI-bounded retrieval of Vx, Vy, Vz (+ rho): retrieved bytes of the
    QoI-guided per-(field, level) budgets against the reference-style
    uniform-halving loop, for |V| and 1/2 rho |V|^2 at pointwise bounds
    tau = rel * range(QoI)."""
    import torch
    from prodm_gb300 import fields, qoi

    V = [v.cuda() for v in fields.divergence_free_velocity(n, seed=11)]
    rho = fields.lognormal_density(n, seed=12).cuda()
    ge = ge_utilities([v.double() for v in V], rho.double())
    out = {"workload": "Vx, Vy, Vz %d^3 fp32 divergence-free random Fourier modes (|k| <= 16), rho lognormal "
                       "(sigma 0.5); %d levels, 32 planes, grouped encoder, hierarchical basis, L-inf tables" %
                       (n, levels + 1), "cases": [], "ge_utilities": ge}
    for kind in ("vmag", "ke"):
        data = V + ([rho] if kind == "ke" else [])
        q = qoi.qoi_value(kind, [v.double() for v in V], rho.double() if kind == "ke" else None)
        for rel in rels:
            tau = qoi.value_range(q) * rel
            t0 = time.time()
            base = qoi.halving_retrieve(kind, data, tau, rel, levels)
            t1 = time.time()
            ours = qoi.guided_retrieve(kind, data, tau, rel, levels)
            t2 = time.time()
            out["cases"].append({
                "qoi": kind, "rel": rel, "tau": tau,
                "halving": {k: base[k] for k in ("bytes", "bound", "achieved", "iterations", "met")},
                "guided": {k: ours[k] for k in ("bytes", "bound", "achieved", "iterations", "met")},
                "bytes_ratio_guided_over_halving": ours["bytes"] / max(base["bytes"], 1),
                "seconds": {"halving": t1 - t0, "guided": t2 - t1}})
            torch.cuda.empty_cache()
    return out


def run_perbit(shape=(513, 513, 513), levels=7, planes=60, rels=(1e-3, 1e-5, 1e-7, 1e-9), steps=3):
    """The GE applications' encoder (PerBitBPEncoder, fp64, 60 planes, max
    collector, SignExclude interpreter with MaxErrorEstimatorHB) on a 513^3
    fp64 shear layer: the refactor + retrieve step (bytes counted as for the
    headline metric), the per-bit encode / decode kernels against the HBM
    roofline (stage events), export of the reference streams, import of them
    (the plane-by-plane parse), and the oracle's single-thread decode of one
    level beside the device's parse + decode of the same level."""
    import numpy as np
    import torch
    import oracle
    from prodm_gb300 import api, fields

    x = fields.shear_layer(shape, delta=0.05, noise_rel=1e-6, seed=21, dtype=torch.float64, device="cuda")
    N = x.numel()
    vr = float(x.max() - x.min())
    m = api.MDRField(shape, torch.float64, levels, planes, "perbit", "hierarchical", "max")
    out = torch.empty_like(x)

    def step(record=None):
        m.refactor(x)
        m.reset()
        for r in rels:
            m.retrieve(r * vr, out=out, interpreter="sign_exclude", estimator="max_hb")
            if record is not None:
                record.append(m.index().astype(np.int64))

    idxs = []
    step(idxs)
    torch.cuda.synchronize()
    sizes, _, _ = m.level_info()
    sizes = sizes.astype(np.int64)
    stream_bytes = int(sizes.sum())
    retrieved = [int(sum(sizes[l, :ix[l]].sum() for l in range(levels + 1))) for ix in idxs]
    step_bytes = (N * 8 + stream_bytes) + sum(r + N * 8 for r in retrieved)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    err = float((out - x).abs().max())

    # kernel stages (finest level): algorithmic bytes / event time
    m.set_timing(True)
    step()
    torch.cuda.synchronize()
    st = m.stage_times()
    m.set_timing(False)
    lel = api.level_dims(shape, levels)[1]
    n_f = int(lel[levels])
    peak, peak_src = measured_peak()
    stage_ms = {}
    for (kind, _), (t, _) in st.items():
        stage_ms[kind] = stage_ms.get(kind, 0.0) + t
    enc_ms = st[("encode", levels)][0]
    enc_bytes = n_f * 8 + n_f * (planes + 1) // 8
    dec_ms, dec_bytes = st[("decode", levels)][0], sum(n_f * (int(ix[levels]) + 1) // 8 + n_f * 8 for ix in idxs)

    # export: rows -> reference streams on the host
    t0 = time.time()
    files = [m.export_level(l) for l in range(levels + 1)]
    t_exp = time.time() - t0
    meta = m.metadata()
    # import: the reference streams loaded into a fresh handle, parsed plane by plane
    m2 = api.MDRField(shape, torch.float64, levels, planes, "perbit", "hierarchical", "max")
    m2.load_metadata(meta)
    for l in range(levels + 1):
        m2.load_level(l, files[l], 0)
    torch.cuda.synchronize()
    t0 = time.time()
    full = m2.retrieve_planes([planes] * (levels + 1))
    torch.cuda.synchronize()
    t_imp = time.time() - t0
    same = bool(torch.equal(full, m.retrieve_planes([planes] * (levels + 1))))
    m2.close()

    # oracle (single thread) decode of level levels-1 against the device's
    # parse + decode of the same streams through the progressive decoder
    lv = levels - 1
    n_l = int(lel[lv])
    blob = files[lv]
    _, b, _ = m.level_info()
    e = math.frexp(float(b[lv]))[1]                 # the level exponent (ComposedRefactor.hpp:118-123)
    dev = api.ProgressiveDecoder("perbit", torch.float64)
    dblob = torch.from_numpy(blob).cuda()
    torch.cuda.synchronize()
    t0 = time.time()
    dout = dev.decode(dblob, sizes[lv].astype(np.uint32), n_l, e, 0, planes, lv, planes)
    torch.cuda.synchronize()
    t_dev = time.time() - t0
    O = oracle.oracle()
    stt = O.perbit_state(np.float64)
    t0 = time.time()
    cout = stt.decode(blob, sizes[lv].astype(np.uint32), n_l, e, 0, planes, lv)
    t_cpu = time.time() - t0
    dec_same = bool(np.array_equal(dout.cpu().numpy(), cout))
    m.close()
    del x, out, full
    torch.cuda.empty_cache()
    return {
        "workload": "%s fp64 tanh shear layer + 1e-6 relative noise (seeded), %d levels, %d planes, PerBit encoder, "
                    "max collector, SignExclude greedy interpreter + MaxErrorEstimatorHB, relative L-inf %s" %
                    ("x".join(map(str, shape)), levels + 1, planes, list(rels)),
        "step": {"ms": ms, "bytes": step_bytes, "gbs": step_bytes / ms / 1e6, "max_error_at_tightest": err,
                 "tightest_bound": rels[-1] * vr, "planes_per_level": [ix.tolist() for ix in idxs]},
        "stage_ms": stage_ms,
        "encode_finest": {"ms": enc_ms, "bytes": enc_bytes, "gbs": enc_bytes / enc_ms / 1e6,
                          "frac": enc_bytes / enc_ms / 1e6 / peak,
                          "bytes_model": "n*8 read + n*(B+1)/8 rows written"},
        "decode_finest": {"ms": dec_ms, "bytes": dec_bytes, "gbs": dec_bytes / dec_ms / 1e6,
                          "frac": dec_bytes / dec_ms / 1e6 / peak,
                          "bytes_model": "per retrieval n*(planes+1)/8 rows read + n*8 written"},
        "peak": {"gbs": peak, "source": peak_src},
        "export": {"stream_bytes": stream_bytes, "seconds": t_exp, "gbs": stream_bytes / t_exp / 1e9,
                   "flow": "pack kernels + D2H into pageable host memory"},
        "import": {"stream_bytes": stream_bytes, "seconds": t_imp, "gbs": stream_bytes / t_imp / 1e9,
                   "identical_to_device_refactor": same,
                   "flow": "all levels' reference streams resident; parse (one CTA per level, plane pipeline) + "
                           "decode + recompose of all planes"},
        "level_decode_vs_cpu": {"level": lv, "elements": n_l, "stream_bytes": int(sizes[lv].sum()),
                                "device_seconds": t_dev, "cpu_oracle_seconds": t_cpu, "cores": 1,
                                "identical": dec_same, "speedup": t_cpu / t_dev},
    }


def run_ortho(shape=(1025, 1025, 513), levels=8, planes=60, rels=(1e-3, 1e-4, 1e-5, 1e-6, 1e-7, 1e-8, 1e-9),
              steps=2):
    """The double-precision configuration: a 1025x1025x513 fp64 tanh shear
    layer + 1e-6 relative noise, 9 levels, 60 planes, grouped encoder, max
    collector, MGARD orthogonal basis (FP64 mass-matrix correction solves),
    SignExclude interpreter with MaxErrorEstimatorOB, relative L-inf bounds
    1e-3..1e-9 of the value range, progressive. Step bytes as the headline's
    (field read + streams written; per tolerance the retrieved streams + the
    field written); per-stage event times from a separate instrumented pass."""
    import numpy as np
    import torch
    from prodm_gb300 import api, fields

    x = fields.shear_layer(shape, delta=0.05, noise_rel=1e-6, seed=9, dtype=torch.float64, device="cuda")
    N = x.numel()
    vr = float(x.max() - x.min())
    m = api.MDRField(shape, torch.float64, levels, planes, "grouped", "orthogonal", "max")
    out = torch.empty_like(x)

    def step(record=None):
        m.refactor(x)
        m.reset()
        for r in rels:
            m.retrieve(r * vr, out=out, interpreter="sign_exclude", estimator="max_ob")
            if record is not None:
                record.append(m.index().astype(np.int64))

    idxs = []
    step(idxs)
    torch.cuda.synchronize()
    errs_ok = bool(float((out - x).abs().max()) <= rels[-1] * vr)
    sizes, _, _ = m.level_info()
    sizes = sizes.astype(np.int64)
    stream_bytes = int(sizes.sum())
    retrieved = [int(sum(sizes[l, :ix[l]].sum() for l in range(levels + 1))) for ix in idxs]
    step_bytes = (N * 8 + stream_bytes) + sum(r + N * 8 for r in retrieved)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    m.set_timing(True)
    step()
    torch.cuda.synchronize()
    st = m.stage_times()
    m.set_timing(False)
    peak, peak_src = measured_peak()
    ld, lel = api.level_dims(shape, levels)
    box = [int(np.prod(ld[l].astype(np.int64))) for l in range(levels + 1)]
    stages = {}
    for (kind, level), (t, cnt) in sorted(st.items(), key=lambda kv: -kv[1][0])[:12]:
        b = None
        if kind == "decompose":     # level box read + written, the correction's boxes
            b = 2 * 8 * box[level]
        stages["%s_l%d" % (kind, level)] = {"ms": t / cnt, "launches": cnt,
                                            "gbs": (b / (t / cnt) / 1e6) if b else None,
                                            "frac": (b / (t / cnt) / 1e6 / peak) if b else None}
    m.close()
    del x, out
    torch.cuda.empty_cache()
    return {
        "workload": "%s fp64 tanh shear layer + 1e-6 relative noise (seeded), %d levels, %d planes, grouped encoder, "
                    "max collector, orthogonal basis, SignExclude greedy interpreter + MaxErrorEstimatorOB, relative "
                    "L-inf %s" % ("x".join(map(str, shape)), levels + 1, planes, list(rels)),
        "step": {"ms": ms, "bytes": step_bytes, "gbs": step_bytes / ms / 1e6, "frac": step_bytes / ms / 1e6 / peak,
                 "tightest_bound_met": errs_ok, "planes_per_level": [ix.tolist() for ix in idxs]},
        "stages": stages,
        "peak": {"gbs": peak, "source": peak_src},
    }


def run_lossless(reps=3):
    """The lossless stage (AdaptiveLevelCompressor's rule, ZCB codec) on the
    headline workload's streams: stored / raw sizes and stopping indices per
    level, the retrieved bytes at each tolerance with and without the stage,
    and the codec's throughput on the finest level's streams (raw bytes per
    second through prodm_lossless_compress_level / _decompress_level, each
    call including its host synchronisation)."""
    import numpy as np
    import torch
    from prodm_gb300 import api, fields

    x = fields.spectral_grf(SHAPE, slope=-5.0 / 3.0, seed=1234, device="cuda")
    norm2 = float((x.double() ** 2).sum())
    m = api.MDRField(SHAPE, torch.float32, LEVELS, BITPLANES, "negabinary", "hierarchical", "squared")
    m.refactor(x)
    raw, _, _ = m.level_info()
    out = torch.empty_like(x)

    def retrieved(sizes):
        m.reset()
        res = []
        for rel in REL_TOLS:
            m.retrieve(rel * rel * norm2, out=out, interpreter="negabinary", estimator="l2_hb")
            idx = m.index()
            res.append(int(sum(int(sizes[l, :idx[l]].astype(np.int64).sum()) for l in range(LEVELS + 1))))
        return res

    raw_ret = retrieved(raw)
    m.set_lossless(26)
    stored, _, _ = m.level_info()
    stored_ret = retrieved(stored)
    m.set_lossless(None)
    blob = m.export_level_device(LEVELS)
    sizes = raw[LEVELS]
    nbytes = int(sizes.astype(np.int64).sum())
    torch.cuda.synchronize()
    t0 = time.time()
    for _ in range(reps):
        comp, csz, stop = api.compress_level(blob, sizes, 26)
    torch.cuda.synchronize()
    t_c = (time.time() - t0) / reps
    t0 = time.time()
    for _ in range(reps):
        back, _ = api.decompress_level(comp, csz, 0, BITPLANES, stop, 26, raw_capacity=nbytes + 16)
    torch.cuda.synchronize()
    t_d = (time.time() - t0) / reps
    same = bool(torch.equal(back, blob))
    # CPU beside it: the oracle's single-thread ZCB compression of planes 0-3
    import oracle
    O = oracle.oracle()
    host = blob.cpu().numpy()
    offs = np.concatenate([[0], np.cumsum(sizes.astype(np.int64))])
    t0 = time.time()
    for p in range(4):
        O.zcb_compress(host[offs[p]:offs[p + 1]])
    t_cpu = time.time() - t0
    cpu_bytes = int(offs[4])
    # the reference's own AdaptiveLevelCompressor (zstd level 3, latter index
    # 26) on the same streams, and what its interpreter would retrieve with
    # those stored sizes (the oracle interpreter, pinned to the reference's)
    zstd = {"available": False}
    import importlib
    ob = importlib.import_module("oracle.build_oracle")
    R = oracle.reference()
    if R is not None and ob.zstd_library():
        _, _, errs = m.level_info()
        zs = np.zeros_like(raw)
        zstop = []
        t0 = time.time()
        for l in range(LEVELS + 1):
            stp, kept, _ = R.adaptive_compress(m.export_level(l), raw[l].astype(np.uint32), 26)
            zs[l] = kept
            zstop.append(int(stp))
        t_z = time.time() - t0
        idx = np.zeros(LEVELS + 1, np.uint8)
        zret = []
        for rel in REL_TOLS:
            idx, _ = O.interpret("negabinary", "l2_hb", zs.astype(np.uint32), errs, rel * rel * norm2, idx)
            zret.append(int(sum(int(zs[l, :idx[l]].astype(np.int64).sum()) for l in range(LEVELS + 1))))
        zl = zs.astype(np.int64).sum(axis=1)
        zstd = {"available": True, "stored_bytes_per_level": zl.tolist(), "stopping_indices": zstop,
                "ratio": float(raw.astype(np.int64).sum() / zl.sum()), "retrieved_bytes": zret,
                "cpu_seconds_all_levels": t_z, "cores": 1,
                "codec": "reference AdaptiveLevelCompressor + ZSTD (level 3), system libzstd"}
    m.close()
    del x, out, blob, comp, back
    torch.cuda.empty_cache()
    rs, ss = raw.astype(np.int64).sum(axis=1), stored.astype(np.int64).sum(axis=1)
    return {"workload": WORKLOAD + "; lossless stage AdaptiveLevelCompressor rule (latter index 26), ZCB codec",
            "raw_bytes_per_level": rs.tolist(), "stored_bytes_per_level": ss.tolist(),
            "ratio": float(rs.sum() / ss.sum()),
            "retrieved_bytes_raw": raw_ret, "retrieved_bytes_stored": stored_ret,
            "reference_zstd": zstd,
            "finest_level": {"raw_bytes": nbytes, "stopping_index": stop, "stored_bytes": int(csz.astype(np.int64).sum()),
                             "compress_seconds": t_c, "compress_gbs": nbytes / t_c / 1e9,
                             "decompress_seconds": t_d, "decompress_gbs": nbytes / t_d / 1e9,
                             "round_trip_identical": same},
            "cpu_baseline": {"kind": "port", "cores": 1, "sample": "oracle ZCB compression of planes 0-3 of the "
                             "finest level (%d bytes)" % cpu_bytes, "value": cpu_bytes / t_cpu / 1e9, "unit": "GB/s"}}


def run_files():
    """Level files of the headline workload written and read back: every level
    file written by prodm_mdr_write_level_file, then loaded into a second
    handle by prodm_mdr_load_level_file (cuFile where it registers the file,
    else pinned staging) into a RAM-backed directory, so that the numbers are
    the path's, not a disk's; the loaded handle's retrieval equals the
    device-resident one."""
    import shutil
    import tempfile
    import torch
    from prodm_gb300 import api, fields

    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    d = tempfile.mkdtemp(prefix="prodm_files_", dir=base)
    try:
        x = fields.spectral_grf(SHAPE, slope=-5.0 / 3.0, seed=1234, device="cuda")
        m = api.MDRField(SHAPE, torch.float32, LEVELS, BITPLANES, "negabinary", "hierarchical", "squared")
        m.refactor(x)
        paths = [os.path.join(d, "level_%d.bin" % l) for l in range(LEVELS + 1)]
        t0 = time.time()
        for l, pth in enumerate(paths):
            m.write_level_file(l, pth)
        t_w = time.time() - t0
        nbytes = sum(os.path.getsize(pth) for pth in paths)
        # the file path's one-time set-up (cuFile's driver, staging buffers) on a
        # throw-away handle first
        w = api.MDRField(SHAPE, torch.float32, LEVELS, BITPLANES, "negabinary", "hierarchical", "squared")
        w.load_metadata(m.metadata())
        w.load_level_file(0, paths[0])
        w.close()
        r = api.MDRField(SHAPE, torch.float32, LEVELS, BITPLANES, "negabinary", "hierarchical", "squared")
        r.load_metadata(m.metadata())
        torch.cuda.synchronize()
        t0 = time.time()
        for l, pth in enumerate(paths):
            r.load_level_file(l, pth)
        torch.cuda.synchronize()
        t_r = time.time() - t0
        norm2 = float((x.double() ** 2).sum())
        tol = REL_TOLS[-1] ** 2 * norm2
        same = bool(torch.equal(m.retrieve(tol, interpreter="negabinary", estimator="l2_hb"),
                                r.retrieve(tol, interpreter="negabinary", estimator="l2_hb")))
        mode = r.file_read_mode()
        t0 = time.time()   # CPU beside it: the files read into host memory (ConcatLevelFileRetriever's fread)
        host_bytes = 0
        for pth in paths:
            with open(pth, "rb") as f:
                host_bytes += len(f.read())
        t_h = time.time() - t0
        m.close()
        r.close()
        del x
        torch.cuda.empty_cache()
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {"workload": WORKLOAD + "; all level files written, then read into a second handle",
            "directory": "RAM-backed (/dev/shm)" if base else "temporary directory", "bytes": nbytes,
            "write_seconds": t_w, "write_gbs": nbytes / t_w / 1e9,
            "read_seconds": t_r, "read_gbs": nbytes / t_r / 1e9,
            "read_path": {1: "cuFile (GPUDirect Storage)", 0: "pread into pinned staging + async copies"}.get(mode, "none"),
            "retrieval_identical": same,
            "cpu_baseline": {"kind": "reference-style", "cores": 1, "sample": "every level file read into host "
                             "memory", "value": host_bytes / t_h / 1e9, "unit": "GB/s"}}


def ge_utilities(V, rho, reps=5):
    """GE quantities of interest on the device (prodm_qoi_ge_values /
    prodm_qoi_ge_bounds) on fp64 fields: V_TOT, T, C, Mach, PT, mu and the V_TOT
    / T error estimates; algorithmic bytes (fields read + results written) per
    CUDA-event time, beside the oracle's single-thread evaluation of a sample."""
    import numpy as np
    import torch
    import oracle
    from prodm_gb300 import api

    N = V[0].numel()
    vx, vy, vz = (v.reshape(-1) for v in V)
    p = (1e5 * (1.0 + 0.1 * rho)).reshape(-1)      # pressure-like field around 1 bar
    d = rho.reshape(-1)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    api.qoi_ge_values(vx, vy, vz, p, d)
    api.qoi_ge_bounds([vx, vy, vz], (0.01, 0.01, 0.01), p, d, 10.0, 1e-4)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        api.qoi_ge_values(vx, vy, vz, p, d)
    ev[1].record()
    for _ in range(reps):
        api.qoi_ge_bounds([vx, vy, vz], (0.01, 0.01, 0.01), p, d, 10.0, 1e-4)
    ev[2].record()
    torch.cuda.synchronize()
    t_v = ev[0].elapsed_time(ev[1]) / reps / 1e3
    t_b = ev[1].elapsed_time(ev[2]) / reps / 1e3
    k = min(N, 1 << 21)
    h = [t[:k].cpu().numpy() for t in (vx, vy, vz, p, d)]
    O = oracle.oracle()
    t0 = time.time()
    O.qoi_values(*h)
    t_c = time.time() - t0
    peak, src = measured_peak()
    bv, bb = 11 * 8 * N, 7 * 8 * N
    return {"points": N, "values_ms": t_v * 1e3, "values_gbs": bv / t_v / 1e9, "values_frac": bv / t_v / 1e9 / peak,
            "bounds_ms": t_b * 1e3, "bounds_gbs": bb / t_b / 1e9, "bounds_frac": bb / t_b / 1e9 / peak,
            "bytes_model": "values: 5 fields read + 6 written; bounds: 5 read + 2 written (8 bytes each)",
            "cpu_baseline": {"kind": "port", "cores": 1, "sample": "oracle qoi_values on %d points" % k,
                             "points_per_s": k / t_c, "device_points_per_s": N / t_v}}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        value, cores, sec, kind = cpu_baseline(args.steps, args.warmup)
        one, _, one_sec, _ = cpu_baseline(1, 0, threads=1)
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian random field)",
            "config": config(),
            "cpu_baseline": {"value": value, "unit": "GB/s", "cores": cores, "kind": kind,
                             "sample": cpu_sample_text(cores, kind),
                             "one_core": {"value": one, "unit": "GB/s", "cores": 1, "seconds_per_field": one_sec}},
            "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return 0
    res = run_ours(args)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            value, cores, sec, kind = cpu_baseline(1, 0)
            one, _, one_sec, _ = cpu_baseline(1, 0, threads=1)
            res["cpu_baseline"] = {"value": value, "unit": "GB/s", "cores": cores, "kind": kind,
                                   "sample": cpu_sample_text(cores, kind),
                                   "one_core": {"value": one, "unit": "GB/s", "cores": 1,
                                                "seconds_per_field": one_sec}}
        print(json.dumps(res))
    return 0


if __name__ == "__main__":
    sys.exit(main())
