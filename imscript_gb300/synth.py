"""Seeded synthetic hole-filling workloads (no external dataset).

The five workloads follow the shapes, sizes and value distributions the
simpois benchmarks are stated on; every random stream derives from one
``numpy.random.default_rng(seed)``.

* smooth field: a sum of isotropic Gaussians (sigma ~ U[10, 80] px,
  amplitude ~ U[-1, 1], centres uniform) plus white noise of variance 0.01;
* holes: random disks (radius ~ U[4, 30] px) drawn until the hole fraction
  is reached, irregular blobs (a disk level set perturbed by smoothed noise),
  a square plus thin scratches;
* guidance: forward-difference gradient G of an independent field, and its
  backward-difference divergence f = div G, which equals the clamped 5-point
  Laplacian of that field, so that Poisson filling reproduces it.

Images are planar float32 (pd, h, w); holes are NaN.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def gaussian_field(rng, h, w, n_gauss, noise_var=0.01):
    """Sum of ``n_gauss`` isotropic Gaussians plus N(0, noise_var) noise, float32."""
    sig = rng.uniform(10, 80, n_gauss)
    amp = rng.uniform(-1, 1, n_gauss)
    cx = rng.uniform(0, w, n_gauss)
    cy = rng.uniform(0, h, n_gauss)
    xs = np.arange(w, dtype=np.float64)
    ys = np.arange(h, dtype=np.float64)
    # separable: field = sum_k amp_k * gy_k(y) gx_k(x) = GY @ diag(amp) @ GX^T
    gx = np.exp(-((xs[None, :] - cx[:, None]) ** 2) / (2 * sig[:, None] ** 2))
    gy = np.exp(-((ys[None, :] - cy[:, None]) ** 2) / (2 * sig[:, None] ** 2))
    f = (gy.T * amp[None, :]) @ gx
    f += rng.normal(0.0, math.sqrt(noise_var), (h, w))
    return f.astype(np.float32)


def disk_mask(rng, h, w, frac, rmin=4.0, rmax=30.0, min_disks=1):
    """Union of random disks, radius ~ U[rmin, rmax], until ``frac`` is covered."""
    m = np.zeros((h, w), bool)
    target = frac * h * w
    nd = 0
    yy = np.arange(h)[:, None]
    xx = np.arange(w)[None, :]
    while nd < min_disks or m.sum() < target:
        r = rng.uniform(rmin, rmax)
        cx = rng.uniform(0, w)
        cy = rng.uniform(0, h)
        y0, y1 = max(0, int(cy - r)), min(h, int(cy + r) + 2)
        x0, x1 = max(0, int(cx - r)), min(w, int(cx + r) + 2)
        sub = (yy[y0:y1] - cy) ** 2 + (xx[:, x0:x1] - cx) ** 2 <= r * r
        m[y0:y1, x0:x1] |= sub
        nd += 1
        if nd > 100000:
            break
    return m


def _smooth_noise(rng, h, w, sigma):
    """Gaussian-filtered white noise (FFT), unit standard deviation."""
    n = rng.standard_normal((h, w))
    ky = np.fft.fftfreq(h)[:, None]
    kx = np.fft.rfftfreq(w)[None, :]
    filt = np.exp(-2 * (math.pi * sigma) ** 2 * (kx ** 2 + ky ** 2))
    s = np.fft.irfft2(np.fft.rfft2(n) * filt, s=(h, w))
    s -= s.mean()
    return s / (s.std() + 1e-30)


def blob_mask(rng, h, w, frac, nblobs=6, roughness=0.35):
    """``nblobs`` irregular blobs covering ``frac``: thresholded smoothed noise
    around random centres, the common radius found by bisection."""
    noise = _smooth_noise(rng, h, w, sigma=max(h, w) / 48.0)
    cx = rng.uniform(0.15 * w, 0.85 * w, nblobs)
    cy = rng.uniform(0.15 * h, 0.85 * h, nblobs)
    rel = rng.uniform(0.7, 1.3, nblobs)
    yy = np.arange(h, dtype=np.float32)[:, None]
    xx = np.arange(w, dtype=np.float32)[None, :]
    dist = np.full((h, w), np.inf, np.float32)
    for k in range(nblobs):
        d = np.sqrt((xx - cx[k]) ** 2 + (yy - cy[k]) ** 2) / rel[k]
        dist = np.minimum(dist, d)
    lo, hi = 0.0, float(max(h, w))
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        cov = ((dist / mid + roughness * noise) < 1.0).mean()
        lo, hi = (mid, hi) if cov < frac else (lo, mid)
    return (dist / hi + roughness * noise) < 1.0


def scratch_mask(rng, h, w, n, lmin=50, lmax=600, width=3):
    """``n`` straight scratches ``width`` px wide, length ~ U[lmin, lmax]."""
    m = np.zeros((h, w), bool)
    for _ in range(n):
        L = rng.uniform(lmin, lmax)
        th = rng.uniform(0, math.pi)
        x0, y0 = rng.uniform(0, w), rng.uniform(0, h)
        t = np.arange(0, L, 0.5)
        xs = x0 + t * math.cos(th)
        ys = y0 + t * math.sin(th)
        for o in range(width):
            ox = -math.sin(th) * (o - (width - 1) / 2)
            oy = math.cos(th) * (o - (width - 1) / 2)
            xi = np.round(xs + ox).astype(int)
            yi = np.round(ys + oy).astype(int)
            ok = (xi >= 0) & (xi < w) & (yi >= 0) & (yi < h)
            m[yi[ok], xi[ok]] = True
    return m


def guidance(field2):
    """Forward-difference gradient of ``field2`` and its backward divergence.

    Returns (gx, gy, f) where f = div G equals the clamped 5-point Laplacian of
    ``field2`` (Neumann at the image border)."""
    F = field2.astype(np.float64)
    gx = np.zeros_like(F)
    gy = np.zeros_like(F)
    gx[:, :-1] = F[:, 1:] - F[:, :-1]
    gy[:-1, :] = F[1:, :] - F[:-1, :]
    f = gx.copy()
    f[:, 1:] -= gx[:, :-1]
    f += gy
    f[1:, :] -= gy[:-1, :]
    return gx.astype(np.float32), gy.astype(np.float32), f.astype(np.float32)


@dataclass
class Instance:
    """One hole-filling problem: planar input with NaN holes, optional data term."""
    g: np.ndarray                    # (pd, h, w) float32, NaN = unknown
    f: np.ndarray | None = None      # (pd, h, w) float32 or None
    tstep: float = 0.25              # > 0: Laplace/Poisson; < 0: biharmonic
    rtol: float = 1e-6
    meta: dict = field(default_factory=dict)

    @property
    def unknowns(self) -> int:
        return int(np.isnan(self.g).sum())


def config0(seed=0, size=512):
    """Laplace, 512x512x1, 32 Gaussians, 20% as disks of radius U[4,30]."""
    rng = np.random.default_rng(seed)
    img = gaussian_field(rng, size, size, 32)
    m = disk_mask(rng, size, size, 0.20, min_disks=40)
    img[m] = np.nan
    return Instance(img[None], None, 0.25, 1e-6, {"name": "laplace-512x512x1"})


def config1(seed=0, size=2048, channels=3, rtol=1e-6):
    """Poisson with guidance, 2048x2048x3: 128 Gaussians per channel, guidance
    from an independent field, 6 blobs covering 15%."""
    rng = np.random.default_rng(seed)
    g = np.stack([gaussian_field(rng, size, size, 128) for _ in range(channels)])
    f = np.stack([guidance(gaussian_field(rng, size, size, 128))[2] for _ in range(channels)])
    m = blob_mask(rng, size, size, 0.15)
    g[:, m] = np.nan
    return Instance(g, f, 0.25, rtol, {"name": f"poisson-guided-{size}x{size}x{channels}"})


def config2(seed=0, size=4096, hole=1024, n_scratch=200):
    """Biharmonic, 4096x4096x1: 256 Gaussians, one 1024^2 square + 200 scratches."""
    rng = np.random.default_rng(seed)
    img = gaussian_field(rng, size, size, 256)
    m = scratch_mask(rng, size, size, n_scratch)
    y0 = (size - hole) // 2
    x0 = (size - hole) // 2
    m[y0:y0 + hole, x0:x0 + hole] = True
    img[m] = np.nan
    return Instance(img[None], None, -0.08, 1e-6, {"name": f"biharmonic-{size}x{size}x1"})


def config3(seed=0, n=256, smin=64, smax=1024):
    """256 uneven instances: sides log-uniform in [64,1024], 1 or 3 channels,
    hole fraction U[5%,60%] as disks, half Laplace, half guided Poisson."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        h = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
        w = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
        pd = 1 if rng.random() < 0.5 else 3
        frac = rng.uniform(0.05, 0.60)
        ng = max(4, int(32 * h * w / 512 ** 2))
        g = np.stack([gaussian_field(rng, h, w, ng) for _ in range(pd)])
        m = disk_mask(rng, h, w, frac)
        g[:, m] = np.nan
        f = None
        if rng.random() < 0.5:
            f = np.stack([guidance(gaussian_field(rng, h, w, ng))[2] for _ in range(pd)])
        out.append(Instance(g, f, 0.25, 1e-6, {"name": f"inst{k}-{w}x{h}x{pd}"}))
    return out


def config4(seed=0, n=32, size=1024):
    """32 single-channel 1024^2 guided Poisson fills plus target fields."""
    rng = np.random.default_rng(seed)
    insts, targets, guid = [], [], []
    for k in range(n):
        g = gaussian_field(rng, size, size, 128)
        gx, gy, f = guidance(gaussian_field(rng, size, size, 128))
        m = blob_mask(rng, size, size, 0.15)
        g[m] = np.nan
        insts.append(Instance(g[None], f[None], 0.25, 1e-6, {"name": f"diff{k}"}))
        targets.append(gaussian_field(rng, size, size, 128))
        guid.append((gx, gy))
    return insts, targets, guid
