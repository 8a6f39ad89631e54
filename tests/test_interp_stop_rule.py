"""The interpreter's stop rule (csrc/interpret.cu, fixed-point pass) as a
host model: the estimate the reference updates pop by pop in double
(acc -= ev[cur]; acc += ev[next]; stop at the first acc < tol) is decided from
exact prefix sums in fixed point plus a bound on the double rounding; where
the model declares a pop certain, the decision must equal the sequential
double arithmetic's, and undecided cases go to the sequential walk.

The model restates the kernel's arithmetic: units of 2^elsb with elsb = the
largest exponent + 1 + 12 - 125, truncation toward zero, the bound
2^28 * sum(|R'| >> 80 + 1 + |R| >> 80 + 1) + 2p + 4."""
import struct

import numpy as np


def fixed_units(x, elsb):
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    ev, m, e = (b >> 52) & 0x7FF, b & ((1 << 52) - 1), -1074
    if ev:
        m |= 1 << 52
        e = ev - 1075
    sh = e - elsb
    v = (m << sh) if sh >= 0 else (0 if sh <= -64 else m >> -sh)
    return -v if b >> 63 else v


def exp_field(x):
    return (struct.unpack("<Q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def model(acc0, tol, subs, adds, ties):
    n = len(subs)
    maxev = max([exp_field(acc0), exp_field(tol)] + [exp_field(v) for v in subs + adds])
    elsb = (maxev - 1022 + 1) + 12 - 125
    R, S, fm, fa, ft = fixed_units(acc0, elsb), 0, n, n, n
    tf = fixed_units(tol, elsb)
    for p in range(n):
        Rp = R - fixed_units(subs[p], elsb)
        R = Rp + fixed_units(adds[p], elsb)
        S += (abs(Rp) >> 80) + 1 + (abs(R) >> 80) + 1
        e = (S << 28) + 2 * p + 4
        if ties[p] and ft == n:
            ft = p
        if R + e < tf:
            fm = min(fm, p)
        elif not (R - e >= tf + 1):
            fa = min(fa, p)
    if (ft <= fm and ft <= fa) or fm < fa:
        if ft <= fm and ft <= fa and ft < n:
            return ("bail", None)
        return ("stop", fm + 1 if fm < n else n)
    return ("sequential", None)


def sequential(acc0, tol, subs, adds, ties):
    acc = acc0
    for p in range(len(subs)):
        if ties[p]:
            return ("bail", None)
        acc = acc - subs[p]
        acc = acc + adds[p]
        if acc < tol:
            return ("stop", p + 1)
    return ("stop", len(subs))


def cases(rng, count, near):
    for _ in range(count):
        n = int(rng.integers(1, 120))
        scale = 10.0 ** rng.uniform(-30, 30)
        subs = list(rng.uniform(0.1, 1, n) * scale * np.exp(-rng.uniform(0, 0.3) * np.arange(n)))
        adds = [s * rng.uniform(0, 0.9) for s in subs]
        acc0 = float(sum(subs) * rng.uniform(1, 3))
        if near:   # tolerances at, or within rounding of, one of the estimates
            acc, vals = acc0, []
            for a, b in zip(subs, adds):
                acc = acc - a
                acc = acc + b
                vals.append(acc)
            tol = vals[int(rng.integers(0, n))] * (1 + rng.choice([0.0, 1e-17, -1e-17, 1e-15, -1e-15, 1e-9]))
        else:
            tol = acc0 * 10 ** rng.uniform(-14, 0)
        ties = [False] * n
        if rng.uniform() < 0.1:
            ties[int(rng.integers(0, n))] = True
        if tol > 0:
            yield acc0, tol, subs, adds, ties


def test_certain_decisions_equal_the_sequential_walk():
    rng = np.random.default_rng(7)
    for near in (False, True):
        undecided = 0
        for c in cases(rng, 1500, near):
            got = model(*c)
            if got[0] == "sequential":
                undecided += 1
                continue
            assert got == sequential(*c)
        if not near:   # random tolerances are decided without the sequential walk
            assert undecided == 0
