"""Seeded synthetic fields with the shapes and statistics of the benchmark
configurations (no dataset is needed or reproduced).

* sinusoids      -- sum of 4 random-phase sinusoids, integer wavenumbers 1-8,
                    amplitude 1, plus N(0, sigma^2) noise        (65^3 CPU case)
* spectral_grf   -- Gaussian random field with power spectrum k^slope
                    (FFT of white noise times k^(slope/2))       (513^3 headline)
* shear_layer    -- tanh((y - y0) / delta) plus white noise of a given
                    relative amplitude                           (fp64 case)
* divergence_free_velocity / lognormal_density               (QoI case)

Generators run on the GPU with torch when a device is present (the 513^3 FFT
takes seconds on the host) and fall back to numpy on the host otherwise.
"""
import math

import numpy as np
import torch


def _dev(device):
    if device is not None:
        return torch.device(device)
    return torch.device("cuda" if torch.cuda.is_available() else "cpu")


def sinusoids(shape, seed=0, n_waves=4, kmin=1, kmax=8, noise=1e-3, dtype=torch.float32, device=None):
    rng = np.random.default_rng(seed)
    dev = _dev(device)
    grids = torch.meshgrid(*[torch.arange(n, dtype=torch.float64, device=dev) for n in shape], indexing="ij")
    g = torch.zeros(shape, dtype=torch.float64, device=dev)
    for _ in range(n_waves):
        kv = rng.integers(kmin, kmax + 1, len(shape)) * rng.choice([-1, 1], len(shape))
        ph = rng.uniform(0, 2 * math.pi)
        arg = sum(2 * math.pi * float(kv[i]) * grids[i] / shape[i] for i in range(len(shape)))
        g += torch.sin(arg + ph)
    gen = torch.Generator(device=dev).manual_seed(int(seed) + 7)
    g += noise * torch.randn(shape, dtype=torch.float64, device=dev, generator=gen)
    return g.to(dtype)


def spectral_grf(shape, slope=-5.0 / 3.0, seed=0, dtype=torch.float32, device=None):
    """Gaussian random field whose power spectrum falls as k^slope, unit variance."""
    dev = _dev(device)
    gen = torch.Generator(device=dev).manual_seed(int(seed))
    white = torch.randn(shape, dtype=torch.float32, device=dev, generator=gen)
    spec = torch.fft.rfftn(white)
    ks = []
    for i, n in enumerate(shape):
        if i == len(shape) - 1:
            k = torch.fft.rfftfreq(n, device=dev) * n
        else:
            k = torch.fft.fftfreq(n, device=dev) * n
        view = [1] * len(shape)
        view[i] = -1
        ks.append((k.to(torch.float32) ** 2).view(view))
    kk = ks[0]
    for k in ks[1:]:
        kk = kk + k
    kmag = torch.sqrt(kk)
    kmag[(0,) * len(shape)] = 1.0
    amp = kmag ** (slope / 2.0)
    amp[(0,) * len(shape)] = 0.0
    spec = spec * amp
    del kk, kmag, amp
    f = torch.fft.irfftn(spec, s=shape)
    f = f / f.std()
    return f.to(dtype).contiguous()


def shear_layer(shape, delta=0.05, noise_rel=1e-6, seed=0, dtype=torch.float64, device=None):
    dev = _dev(device)
    ny = shape[-2] if len(shape) >= 2 else shape[0]
    y = torch.linspace(0.0, 1.0, ny, dtype=torch.float64, device=dev)
    prof = torch.tanh((y - 0.5) / delta)
    view = [1] * len(shape)
    view[-2 if len(shape) >= 2 else 0] = -1
    f = prof.view(view).expand(shape).clone()
    gen = torch.Generator(device=dev).manual_seed(int(seed))
    f += noise_rel * 2.0 * torch.randn(shape, dtype=torch.float64, device=dev, generator=gen)
    return f.to(dtype).contiguous()


def divergence_free_velocity(n, kmax=16, n_modes=64, seed=0, dtype=torch.float32, device=None):
    """Sum of random Fourier modes with |k| <= kmax, each projected orthogonal to k."""
    rng = np.random.default_rng(seed)
    dev = _dev(device)
    x = torch.arange(n, dtype=torch.float64, device=dev) / n
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    V = [torch.zeros((n, n, n), dtype=torch.float64, device=dev) for _ in range(3)]
    m = 0
    while m < n_modes:
        k = rng.integers(-kmax, kmax + 1, 3)
        kn = float(np.linalg.norm(k))
        if kn == 0 or kn > kmax:
            continue
        a = rng.standard_normal(3)
        a -= k * (a @ k) / (kn * kn)
        a /= max(np.linalg.norm(a), 1e-12)
        a *= kn ** (-5.0 / 6.0)
        ph = rng.uniform(0, 2 * math.pi)
        s = torch.sin(2 * math.pi * (k[0] * X + k[1] * Y + k[2] * Z) + ph)
        for c in range(3):
            V[c] += float(a[c]) * s
        m += 1
    return [v.to(dtype).contiguous() for v in V]


def lognormal_density(n, sigma=0.5, seed=0, dtype=torch.float32, device=None):
    g = spectral_grf((n, n, n), slope=-3.0, seed=seed, dtype=torch.float32, device=device)
    return torch.exp(sigma * g.to(torch.float64)).to(dtype).contiguous()


def batch_level(shape, max_level):
    """Largest level count the reference accepts that keeps level 0 at >= 32
    values (its block encoders need one full block, see the encoder loops)."""
    L = max_level
    while L > 0:
        box = list(shape)
        for _ in range(L):
            box = [(n >> 1) + 1 for n in box]
        if int(np.prod(box)) >= 32:
            return L
        L -= 1
    return 0


def batch_specs(seed=0):
    """The 64-field batch: 24 cubes with sides from {33, 65, 129, 257}, 24 2-D
    fields with sides from {513, 1025, 2049}, 16 anisotropic 129 x 257 x 65
    fields; spectral slopes uniform in [-3, -1]; relative L-inf tolerances
    log-uniform in [1e-5, 1e-2]."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(24):
        n = int(rng.choice([33, 65, 129, 257]))
        specs.append((n, n, n))
    for _ in range(24):
        n = int(rng.choice([513, 1025, 2049]))
        specs.append((n, n))
    for _ in range(16):
        specs.append((129, 257, 65))
    slopes = rng.uniform(-3.0, -1.0, len(specs))
    rel = 10.0 ** rng.uniform(-5.0, -2.0, len(specs))
    return [(s, float(a), float(t)) for s, a, t in zip(specs, slopes, rel)]
