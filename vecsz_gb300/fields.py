"""Seeded synthetic fields with the shapes and statistics of the benchmark workloads.

The reference benchmarks on CESM / Hurricane / NYX files that are not available; these generators
stand in for them:
  bump_field_2d   sum of 64 Gaussian bumps (centres uniform, sigma U[20, 400] px, amplitudes N(0,1))
                  plus U(0, 1e-5) noise, min-max scaled to [0, 1]          (1800 x 3600 CESM-like)
  grf_3d          Gaussian random field, amplitude ~ k^(-11/6) (power ~ k^(-11/3)), random phases,
                  standardised, exponentiated so max/min ~ 1e4              (512^3 NYX-like)
  adversarial_3d  grf_3d + 5% Cauchy spikes (scale 100 std) + 8 planar steps (256 x 384 x 384)
Each has a numpy version (small fields, CPU) and a torch version (any size, on the GPU).
Shapes are numpy order (z, y, x); the reference's dims are the reverse (x, y, z).
"""
from __future__ import annotations

import math

import numpy as np


def bump_field_2d(ny: int, nx: int, seed: int = 0, nbumps: int = 64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    cy = rng.uniform(0, ny, nbumps)
    cx = rng.uniform(0, nx, nbumps)
    sig = rng.uniform(20, 400, nbumps)
    amp = rng.standard_normal(nbumps)
    yy = np.arange(ny, dtype=np.float64)[:, None]
    xx = np.arange(nx, dtype=np.float64)[None, :]
    f = np.zeros((ny, nx), np.float64)
    for i in range(nbumps):
        f += amp[i] * np.exp(-((yy - cy[i]) ** 2 + (xx - cx[i]) ** 2) / (2 * sig[i] ** 2))
    f += rng.uniform(0, 1e-5, (ny, nx))
    f = (f - f.min()) / (f.max() - f.min())
    return f.astype(np.float32)


def _grf_spectrum_np(shape, rng, slope=-11.0 / 6.0):
    nz, ny, nx = shape
    kz = np.fft.fftfreq(nz)[:, None, None]
    ky = np.fft.fftfreq(ny)[None, :, None]
    kx = np.fft.rfftfreq(nx)[None, None, :]
    k = np.sqrt(kz ** 2 + ky ** 2 + kx ** 2)
    k[0, 0, 0] = 1.0
    amp = k ** slope
    amp[0, 0, 0] = 0.0
    ph = rng.standard_normal(amp.shape) + 1j * rng.standard_normal(amp.shape)
    return amp * ph


def grf_3d(nz: int, ny: int, nx: int, seed: int = 0, decades: float = 4.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    g = np.fft.irfftn(_grf_spectrum_np((nz, ny, nx), rng), s=(nz, ny, nx), axes=(0, 1, 2))
    g = (g - g.mean()) / g.std()
    a = decades * math.log(10.0) / (g.max() - g.min())
    return np.exp(a * g).astype(np.float32)


def adversarial_3d(nz: int, ny: int, nx: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed + 7)
    f = grf_3d(nz, ny, nx, seed).astype(np.float64)
    std = f.std()
    n = f.size
    idx = rng.choice(n, int(0.05 * n), replace=False)
    f.reshape(-1)[idx] = rng.standard_cauchy(len(idx)) * 100 * std
    for _ in range(8):
        nrm = rng.standard_normal(3)
        nrm /= np.linalg.norm(nrm)
        off = rng.uniform(-0.3, 0.3)
        z, y, x = np.meshgrid(np.linspace(-0.5, 0.5, nz), np.linspace(-0.5, 0.5, ny), np.linspace(-0.5, 0.5, nx),
                              indexing="ij")
        f += (nrm[0] * z + nrm[1] * y + nrm[2] * x > off) * rng.standard_normal() * std
    return f.astype(np.float32)


# ------------------------------------------------------------------------------------------------
# torch versions (GPU, large fields); the same recipes with torch's generator
# ------------------------------------------------------------------------------------------------

def bump_field_2d_torch(ny, nx, seed=0, nbumps=64, device="cuda"):
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    cy = torch.rand(nbumps, generator=g, dtype=torch.float64) * ny
    cx = torch.rand(nbumps, generator=g, dtype=torch.float64) * nx
    sig = 20 + torch.rand(nbumps, generator=g, dtype=torch.float64) * 380
    amp = torch.randn(nbumps, generator=g, dtype=torch.float64)
    yy = torch.arange(ny, dtype=torch.float64, device=device)[:, None]
    xx = torch.arange(nx, dtype=torch.float64, device=device)[None, :]
    f = torch.zeros((ny, nx), dtype=torch.float64, device=device)
    for i in range(nbumps):
        f += amp[i].item() * torch.exp(-((yy - cy[i].item()) ** 2 + (xx - cx[i].item()) ** 2) / (2 * sig[i].item() ** 2))
    noise = torch.rand((ny, nx), generator=g, dtype=torch.float64).to(device) * 1e-5
    f += noise
    f = (f - f.min()) / (f.max() - f.min())
    return f.float().contiguous()


def grf_3d_torch(nz, ny, nx, seed=0, decades=4.0, device="cuda"):
    import torch
    gen = torch.Generator(device=device).manual_seed(seed)
    kz = torch.fft.fftfreq(nz, device=device)[:, None, None]
    ky = torch.fft.fftfreq(ny, device=device)[None, :, None]
    kx = torch.fft.rfftfreq(nx, device=device)[None, None, :]
    k = torch.sqrt(kz ** 2 + ky ** 2 + kx ** 2)
    k[0, 0, 0] = 1.0
    amp = k ** (-11.0 / 6.0)
    amp[0, 0, 0] = 0.0
    re = torch.randn(amp.shape, generator=gen, device=device)
    im = torch.randn(amp.shape, generator=gen, device=device)
    spec = torch.complex(amp * re, amp * im)
    del re, im, k
    g = torch.fft.irfftn(spec, s=(nz, ny, nx))
    del spec
    g = (g - g.mean()) / g.std()
    a = decades * math.log(10.0) / float(g.max() - g.min())
    return torch.exp(a * g).float().contiguous()


def adversarial_3d_torch(nz, ny, nx, seed=0, device="cuda"):
    import torch
    f = grf_3d_torch(nz, ny, nx, seed, device=device).double()
    gen = torch.Generator(device=device).manual_seed(seed + 7)
    std = float(f.std())
    n = f.numel()
    idx = torch.randperm(n, generator=gen, device=device)[: int(0.05 * n)]
    u = torch.rand(idx.numel(), generator=gen, device=device, dtype=torch.float64)
    f.view(-1)[idx] = torch.tan(math.pi * (u - 0.5)) * 100 * std
    for _ in range(8):
        nrm = torch.randn(3, generator=gen, device=device, dtype=torch.float64)
        nrm = nrm / nrm.norm()
        off = float(torch.rand(1, generator=gen, device=device)) * 0.6 - 0.3
        amp = float(torch.randn(1, generator=gen, device=device)) * std
        z = torch.linspace(-0.5, 0.5, nz, device=device, dtype=torch.float64)[:, None, None]
        y = torch.linspace(-0.5, 0.5, ny, device=device, dtype=torch.float64)[None, :, None]
        x = torch.linspace(-0.5, 0.5, nx, device=device, dtype=torch.float64)[None, None, :]
        f += ((nrm[0] * z + nrm[1] * y + nrm[2] * x) > off).double() * amp
    return f.float().contiguous()


# ------------------------------------------------------------------------------------------------
# Mixed field sets for the batched path: 1D/2D/3D at 20/40/40 %, element counts log-uniform in
# [16K, 16M] factored into random aspect ratios, each field the k^-11/3 random field or the smooth
# bump field, with its own r2r error bound log-uniform in [1e-5, 1e-2].
# ------------------------------------------------------------------------------------------------

def _factor(n: int, nd: int, rng) -> tuple:
    """dims (x fastest) of about n elements with random aspect ratios."""
    if nd == 1:
        return (n,)
    if nd == 2:
        u = rng.uniform(0.25, 0.75)
        d0 = max(1, int(round(n ** u)))
        return (d0, max(1, int(round(n / d0))))
    w = rng.uniform(0.5, 1.5, 3)
    w = w / w.sum()
    d0 = max(1, int(round(n ** w[0])))
    d1 = max(1, int(round(n ** w[1])))
    return (d0, d1, max(1, int(round(n / (d0 * d1)))))


def batch_field_specs(n_fields: int = 1000, seed: int = 0, n_min: int = 1 << 14, n_max: int = 1 << 24) -> list:
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n_fields):
        nd = int(rng.choice([1, 2, 3], p=[0.2, 0.4, 0.4]))
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        dims = _factor(n, nd, rng)
        kind = "bump" if (nd == 2 and rng.random() < 0.5) else "grf"
        specs.append({"ndim": nd, "dims": dims, "kind": kind, "eb": float(10 ** rng.uniform(-5, -2)),
                      "seed": seed * 100003 + i})
    return specs


def grf_torch(shape, seed=0, decades=4.0, device="cuda"):
    """k^-11/3 random field of any dimensionality (numpy-order shape), exponentiated to span
    `decades` decades."""
    import torch
    gen = torch.Generator(device=device).manual_seed(seed)
    shape = tuple(int(v) for v in shape)
    ks = []
    for ax, m in enumerate(shape):
        f = torch.fft.rfftfreq(m, device=device) if ax == len(shape) - 1 else torch.fft.fftfreq(m, device=device)
        view = [1] * len(shape)
        view[ax] = -1
        ks.append(f.view(view) ** 2)
    k2 = ks[0]
    for t in ks[1:]:
        k2 = k2 + t
    k = torch.sqrt(k2)
    k.view(-1)[0] = 1.0
    amp = k ** (-11.0 / 6.0)
    amp.view(-1)[0] = 0.0
    spec = torch.complex(amp * torch.randn(amp.shape, generator=gen, device=device),
                         amp * torch.randn(amp.shape, generator=gen, device=device))
    g = torch.fft.irfftn(spec, s=shape)
    del spec, amp, k
    sd = g.std()
    g = (g - g.mean()) / (sd if float(sd) > 0 else 1.0)
    span = float(g.max() - g.min())
    a = decades * math.log(10.0) / (span if span > 0 else 1.0)
    return torch.exp(a * g).float().contiguous()


def bump_field_2d_torch32(ny, nx, seed=0, nbumps=64, device="cuda"):
    """bump_field_2d in float32 on the device (for large mixed sets)."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    cy = (torch.rand(nbumps, generator=g) * ny).tolist()
    cx = (torch.rand(nbumps, generator=g) * nx).tolist()
    sig = (20 + torch.rand(nbumps, generator=g) * 380).tolist()
    amp = torch.randn(nbumps, generator=g).tolist()
    yy = torch.arange(ny, dtype=torch.float32, device=device)[:, None]
    xx = torch.arange(nx, dtype=torch.float32, device=device)[None, :]
    f = torch.zeros((ny, nx), dtype=torch.float32, device=device)
    for i in range(nbumps):
        f += amp[i] * torch.exp(-((yy - cy[i]) ** 2 + (xx - cx[i]) ** 2) / (2 * sig[i] ** 2))
    f += torch.rand((ny, nx), generator=torch.Generator(device=device).manual_seed(seed), device=device) * 1e-5
    lo, hi = f.min(), f.max()
    return ((f - lo) / (hi - lo if float(hi - lo) > 0 else 1.0)).contiguous()


def batch_field_torch(spec, device="cuda"):
    dims = spec["dims"]
    shape = tuple(reversed(dims))
    if spec["kind"] == "bump":
        return bump_field_2d_torch32(shape[0], shape[1], seed=spec["seed"], device=device).reshape(-1)
    return grf_torch(shape, seed=spec["seed"], device=device).reshape(-1)
