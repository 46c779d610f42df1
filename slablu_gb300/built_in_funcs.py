"""Coefficient fields and boundary data of the reference's driver.

Same formulas as src_disc/built_in_funcs.py (functions of an (N, 2) torch
tensor of points); ``c(x) = bfield(x, kh)`` is the zeroth-order coefficient
of the Helmholtz operator -Lap u + c u.
"""
import numpy as np
import torch
from scipy.special import hankel1


def _bumps(xx, centres, width, mag=1.0):
    b = torch.zeros(xx.shape[0], device=xx.device, dtype=torch.float64)
    for (x, y) in centres:
        b += mag * torch.exp(-width * ((xx[:, 0] - x) ** 2 + (xx[:, 1] - y) ** 2))
    return b


def uu_dir_func_greens(xx, kh, center=(-0.1, +0.5)):
    """Re[(i/4) H0^(1)(kh |x - center|)] (log for kh = 0), built_in_funcs.py:59-70."""
    x = xx.detach().cpu().numpy() if isinstance(xx, torch.Tensor) else np.asarray(xx)
    d2 = (x[:, 0] - center[0]) ** 2 + (x[:, 1] - center[1]) ** 2
    if kh == 0:
        u = (1 / np.pi) * np.log(d2)
    else:
        u = np.real((1j / 4) * hankel1(0, kh * np.sqrt(d2)))
    return torch.as_tensor(u, dtype=torch.float64)[:, None]


def uu_dir_pulse(xx, kh):
    u = torch.zeros(xx.shape[0], 1, dtype=torch.float64, device=xx.device)
    left = xx[:, 0] == 0
    u[left, 0] = torch.exp(-200 * (xx[left, 1] - 0.5) ** 2)
    return u


def bfield_constant(xx, kh):
    return -(kh ** 2) * torch.ones(xx.shape[0], device=xx.device, dtype=torch.float64)


def bfield_bumpy(xx, kh):
    s = torch.sin(4 * np.pi * xx[:, 0]) * torch.sin(4 * np.pi * xx[:, 1])
    return -(kh ** 2) * (1 - s ** 2)


def bfield_gaussian_bumps(xx, kh):
    b = _bumps(xx, [(0.5, 0.5), (0.25, 0.5)], 2000.0)
    return -(kh ** 2) * (1 - b)


def bfield_crystal(xx, kh, crystal_start=0.2, crystal_end=0.8, dist=0.05):
    cen = [(x, y) for x in np.arange(crystal_start, crystal_end + dist, dist)
           for y in np.arange(crystal_start, crystal_end, dist)]
    b = _bumps(xx, cen, 1500.0)
    return -(kh ** 2) * (1 - b / torch.max(b))


def bfield_crystal_waveguide(xx, kh):
    dist = 0.04
    x0 = y0 = 0.1 + 0.5 * dist
    x1 = 0.50
    x2 = y2 = x1 + 2.5 * dist
    x3 = y3 = 0.9
    cen = [(x, y) for x in np.arange(x0, x1, dist) for y in np.arange(y0, x1, dist)]
    cen += [(x, y) for x in np.arange(x2, x3, dist) for y in np.arange(y0, y2 - 0.5 * dist, dist)]
    cen += [(x, y) for x in np.arange(x0, x3, dist) for y in np.arange(y2, y3, dist)]
    b = _bumps(xx, cen, 2500.0, mag=0.930655)
    return -(kh ** 2) * (1 - b)


def bfield_cavity_scattering(xx, kh):
    r2 = (xx[:, 0] - 0.5) ** 2 + (xx[:, 1] - 0.5) ** 2
    phi = torch.atan2(xx[:, 1] - 0.5, xx[:, 0] - 0.5)
    b = (1 - torch.sin(0.5 * phi) ** 200) * torch.exp(-1000 * (0.1 - r2) ** 2)
    return -(kh ** 2) * (1 - b)


BFIELDS = {
    'bfield_constant': bfield_constant,
    'bfield_bumpy': bfield_bumpy,
    'bfield_gaussian_bumps': bfield_gaussian_bumps,
    'bfield_cavity': bfield_cavity_scattering,
    'bfield_crystal': bfield_crystal,
    'bfield_crystal_waveguide': bfield_crystal_waveguide,
}
