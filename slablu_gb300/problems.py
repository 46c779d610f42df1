"""Seeded synthetic problems of the benchmark configurations.

No public dataset is involved; every field is generated from a seed.
Wavenumbers follow the reference driver: kh = (nwaves + 0.03) 2 pi + 1.8 with
nwaves = n / ppw (argparse_driver.py:86-90).

  config1  p=12, n=400 (40 x 40 leaves): constant Helmholtz, Dirichlet data
           Re sum_{k<8} exp(i kh d_k . x), seeded directions.
  config2  16,384 leaves (128 x 128 tiling), p=22: c = -kh^2 b,
           b = 1 + 0.5 sum of 32 Gaussian bumps (width 0.02, seeded centres).
  config3  p=22, n=2000 (100 x 100 leaves, N = 4,404,000): lattice of narrow
           Gaussian bumps (spacing 0.04, width 0.005, amplitude 1, seeded
           offset), c = -kh^2 (1 - b) as the reference's crystal fields,
           Dirichlet u = 1.
  config4  256 right-hand sides on the config3 factors: i.i.d. N(0,1) at the
           Dirichlet nodes, smoothed by a width-8 moving average along the
           boundary ordering.
  config5  p=16, n=1008 (72 x 72 leaves, N = 1,163,232; n = 1000 would give a
           prime 71 x 71 leaf grid, which the reference's slab partition turns
           into one-leaf slabs): c = -kh^2 b, b = 1 + 0.3 g with g a seeded
           Gaussian random field of correlation length 0.05, kh for 20
           wavelengths across the domain (kh = (20 + 0.03) 2 pi + 1.8, the
           driver's formula with nwaves = 20), Dirichlet u = 1; loss
           ||P u(b) - d||^2 with P the
           values at 4,096 seeded interior leaf nodes and d = P u(b') for a
           perturbed field b' = b + 0.05 g'.
"""
import math

import numpy as np
import torch


def kh_for(n, ppw):
    return (int(n / ppw) + 0.03) * 2 * math.pi + 1.8


def leaf_half_width(n, p):
    return 1 / (2 * (n / (p - 2)))


def plane_wave_dirichlet(kh, seed=0, nwaves=8):
    g = torch.Generator().manual_seed(seed)
    theta = torch.rand(nwaves, generator=g, dtype=torch.float64) * 2 * math.pi
    d = torch.stack((torch.cos(theta), torch.sin(theta)), 1)

    def uu(xx):
        xx = torch.as_tensor(xx, dtype=torch.float64)
        ph = kh * (xx.to(d.device) @ d.T)
        return torch.cos(ph).sum(1, keepdim=True)
    return uu


def bumps32_b(xx, seed=0, nb=32, width=0.02, amp=0.5):
    rng = np.random.default_rng(seed)
    cen = torch.as_tensor(rng.random((nb, 2)), dtype=torch.float64, device=xx.device)
    d2 = ((xx[:, None, :] - cen[None]) ** 2).sum(-1)
    return 1.0 + amp * torch.exp(-d2 / (2 * width ** 2)).sum(1)


def lattice_b(xx, seed=0, spacing=0.04, width=0.005, amp=1.0):
    """Sum of Gaussian bumps on a square lattice with a seeded offset.

    Only the nearest lattice sites matter (exp(-(0.02/0.005)^2/2) ~ 3e-4 at half
    a spacing), so each point sums the 3 x 3 sites around it."""
    rng = np.random.default_rng(seed)
    off = torch.as_tensor(rng.random(2) * spacing, dtype=torch.float64, device=xx.device)
    rel = (xx - off) / spacing
    base = torch.floor(rel)
    b = torch.zeros(xx.shape[0], dtype=torch.float64, device=xx.device)
    for dx in (-1, 0, 1, 2):
        for dy in (-1, 0, 1, 2):
            site = (base + torch.tensor([dx, dy], dtype=torch.float64, device=xx.device)) * spacing + off
            d2 = ((xx - site) ** 2).sum(1)
            b += amp * torch.exp(-d2 / (2 * width ** 2))
    return b


def config1(seed=0):
    p, n = 12, 400
    kh = kh_for(n, 10)
    return dict(p=p, n=n, kh=kh, a=leaf_half_width(n, p),
                c=lambda xx: -(kh ** 2) * torch.ones(xx.shape[0], dtype=torch.float64, device=xx.device),
                uu_dir=plane_wave_dirichlet(kh, seed))


def config2(seed=0):
    p, nside = 22, 128
    n = nside * (p - 2)
    kh = kh_for(n, 10)
    return dict(p=p, n=n, nside=nside, kh=kh, a=leaf_half_width(n, p),
                c=lambda xx: -(kh ** 2) * bumps32_b(xx, seed))


def config3(seed=0):
    p, n = 22, 2000
    kh = kh_for(n, 10)
    return dict(p=p, n=n, kh=kh, a=leaf_half_width(n, p),
                c=lambda xx: -(kh ** 2) * (1 - lattice_b(xx, seed)),
                uu_dir=lambda xx: torch.ones(xx.shape[0], 1, dtype=torch.float64))


def config4_rhs(nbnd, nrhs=256, seed=0, width=8):
    """(nbnd, nrhs) smoothed Gaussian boundary data (moving average of `width`)."""
    g = torch.Generator().manual_seed(seed)
    z = torch.randn(nrhs, 1, nbnd + width - 1, generator=g, dtype=torch.float64)
    k = torch.ones(1, 1, width, dtype=torch.float64) / width
    return torch.nn.functional.conv1d(z, k)[:, 0, :].T.contiguous()


def grf(xx, seed=0, ell=0.05, nfeat=1024):
    """Seeded Gaussian random field of unit variance with the squared-exponential
    covariance exp(-|x - y|^2 / (2 ell^2)), sampled by random Fourier features
    (Rahimi and Recht): g(x) = sqrt(2/M) sum_m cos(w_m . x + phi_m) with
    w_m ~ N(0, I / ell^2) and phi_m ~ U[0, 2 pi).  Defined at any point, so the
    leaf nodes of any grid see the same field."""
    g = torch.Generator().manual_seed(seed)
    w = torch.randn(nfeat, 2, generator=g, dtype=torch.float64) / ell
    ph = torch.rand(nfeat, generator=g, dtype=torch.float64) * 2 * math.pi
    xx = torch.as_tensor(xx, dtype=torch.float64)
    w, ph = w.to(xx.device), ph.to(xx.device)
    out = torch.zeros(xx.shape[0], dtype=torch.float64, device=xx.device)
    for i0 in range(0, xx.shape[0], 1 << 18):  # chunks keep the (points x features) product small
        x = xx[i0:i0 + (1 << 18)]
        out[i0:i0 + x.shape[0]] = torch.cos(x @ w.T + ph).sum(1)
    return out * math.sqrt(2.0 / nfeat)


def config5(seed=0, n=1008, nwaves=20):
    p = 16
    kh = (nwaves + 0.03) * 2 * math.pi + 1.8
    return dict(p=p, n=n, kh=kh, a=leaf_half_width(n, p), nprobe=4096,
                b=lambda xx: 1.0 + 0.3 * grf(xx, seed),
                b_perturbed=lambda xx: 1.0 + 0.3 * grf(xx, seed) + 0.05 * grf(xx, seed + 100),
                c_of_b=lambda b: -(kh ** 2) * b,
                uu_dir=lambda xx: torch.ones(xx.shape[0], 1, dtype=torch.float64))


def probe_nodes(xx, nprobe=4096, seed=0, margin=1e-12):
    """Indices of `nprobe` distinct seeded leaf nodes strictly inside the unit square."""
    xx = np.asarray(xx)
    inside = np.where((xx[:, 0] > margin) & (xx[:, 0] < 1 - margin) & (xx[:, 1] > margin) &
                      (xx[:, 1] < 1 - margin))[0]
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(inside, size=nprobe, replace=False))
