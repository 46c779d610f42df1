"""Partial differential operator container (src_disc/pdo.py:6-12, 24-33) and
the parameter maps of curved domains (:36-333).

-c11 u_xx - c22 u_yy - 2 c12 u_xy + c1 u_x + c2 u_y + c u = f, each
coefficient a callable of an (N, 2) torch tensor of points, or None.
"""
import numpy as np
import torch


class PDO_2d:
    def __init__(self, c11, c22, c12=None, c1=None, c2=None, c=None):
        self.c11, self.c22 = c11, c22
        self.c12 = c12
        self.c1, self.c2 = c1, c2
        self.c = c


def ones(xxloc):
    return torch.ones(xxloc.shape[0], device=xxloc.device, dtype=torch.float64)


def const(c=1):
    return lambda xxloc: c * torch.ones(xxloc.shape[0], device=xxloc.device, dtype=torch.float64)


# ---------------------------------------------------------------------------
# Curved domains by a parameter map (src_disc/pdo.py:36-333).  A domain Psi is
# the image of a rectangle Omega under z = z(x); with y = y(z) the inverse map,
# -Lap_z u + c u = 0 on Psi becomes on Omega
#   -(|grad y1|^2) u_11 - (|grad y2|^2) u_22 - 2 (grad y1 . grad y2) u_12
#   - (Lap y1) u_1 - (Lap y2) u_2 + c(z(x)) u = 0,
# i.e. c11 = |grad y1|^2, c22 = |grad y2|^2, c12 = grad y1 . grad y2,
# c1 = -Lap y1, c2 = -Lap y2, with the derivatives of y taken at z(x).  Each
# geometry supplies z and the first and second derivatives of y; a term the
# reference leaves out is None (its annulus drops Lap y1, which is zero there).
# ---------------------------------------------------------------------------

def _sum_terms(terms, sign):
    terms = [t for t in terms if t is not None]
    if not terms:
        return None

    def f(zz):
        out = 0
        for t in terms:
            out = out + t(zz) if sign > 0 else out - t(zz)
        return out
    return f


def _mapped_pdo(kh, bfield, z, y1_d=(None, None), y2_d=(None, None), y1_dd=(None, None), y2_dd=(None, None)):
    def pmap(xx):
        z1, z2 = z(xx)
        return torch.stack((z1, z2), dim=1)

    def on_domain(f):
        return None if f is None else (lambda xx: f(pmap(xx)))

    sq = lambda g: None if g is None else (lambda zz: g(zz) ** 2)
    dot = lambda g, h: None if (g is None or h is None) else (lambda zz: g(zz) * h(zz))
    op = PDO_2d(c11=on_domain(_sum_terms([sq(y1_d[0]), sq(y1_d[1])], 1)),
                c22=on_domain(_sum_terms([sq(y2_d[0]), sq(y2_d[1])], 1)),
                c12=on_domain(_sum_terms([dot(y1_d[0], y2_d[0]), dot(y1_d[1], y2_d[1])], 1)),
                c1=on_domain(_sum_terms(list(y1_dd), -1)),
                c2=on_domain(_sum_terms(list(y2_dd), -1)),
                c=lambda xx: bfield(pmap(xx), kh))
    return op, pmap


def _radius(zz):
    return (zz[:, 0] ** 2 + zz[:, 1] ** 2) ** 0.5


def _annulus(kh, bfield):
    """r = 1 + x2, theta = x1 pi / 3 (pdo.py:189-215)."""
    t = 1 / (np.pi / 3)
    r = _radius
    z = lambda xx: ((1 + 1 * xx[:, 1]) * torch.cos(xx[:, 0] / t), (1 + 1 * xx[:, 1]) * torch.sin(xx[:, 0] / t))
    return _mapped_pdo(
        kh, bfield, z,
        y1_d=(lambda zz: -t * (zz[:, 1] / r(zz) ** 2), lambda zz: +t * (zz[:, 0] / r(zz) ** 2)),
        y2_d=(lambda zz: zz[:, 0] / r(zz), lambda zz: zz[:, 1] / r(zz)),
        y2_dd=(lambda zz: zz[:, 1] ** 2 / r(zz) ** 3, lambda zz: zz[:, 0] ** 2 / r(zz) ** 3))


def _curvy_annulus(kh, bfield):
    """r = 1 + 0.2 cos(5 theta) + x2, theta = x1 pi / 3 (pdo.py:217-282)."""
    t, ph, amp = 1 / (np.pi / 3), 5, 0.2
    r = _radius
    th = lambda zz: torch.arctan2(zz[:, 1], zz[:, 0])
    rad = lambda xx: 1 + amp * torch.cos(ph * xx[:, 0] / t) + xx[:, 1]

    def y2_d1(zz):
        return zz[:, 0] / r(zz) - amp * ph * (zz[:, 1] * (torch.sin(ph * th(zz)) / r(zz) ** 2))

    def y2_d2(zz):
        return zz[:, 1] / r(zz) + (amp * ph * zz[:, 0]) * (torch.sin(ph * th(zz)) / r(zz) ** 2)

    def y2_d1d1(zz):
        a1, a2 = zz[:, 0] * torch.sin(ph * th(zz)), zz[:, 1] * torch.cos(ph * th(zz))
        return zz[:, 1] ** 2 / r(zz) ** 3 + amp * ph * ((zz[:, 1] * (2 * a1 + ph * a2)) / r(zz) ** 4)

    def y2_d2d2(zz):
        a1, a2 = zz[:, 0] * torch.cos(ph * th(zz)), zz[:, 1] * torch.sin(ph * th(zz))
        return zz[:, 0] ** 2 / r(zz) ** 3 + amp * ph * ((zz[:, 0] * (ph * a1 - 2 * a2)) / r(zz) ** 4)

    z = lambda xx: (rad(xx) * torch.cos(xx[:, 0] / t), rad(xx) * torch.sin(xx[:, 0] / t))
    return _mapped_pdo(
        kh, bfield, z,
        y1_d=(lambda zz: -t * (zz[:, 1] / r(zz) ** 2), lambda zz: +t * (zz[:, 0] / r(zz) ** 2)),
        y2_d=(y2_d1, y2_d2),
        y1_dd=(lambda zz: +2 * t * ((zz[:, 0] * zz[:, 1]) / r(zz) ** 4),
               lambda zz: -2 * t * ((zz[:, 0] * zz[:, 1]) / r(zz) ** 4)),
        y2_dd=(y2_d1d1, y2_d2d2))


def _sinusoidal(kh, bfield):
    """The strip under x2 = 1 / (1 - 0.25 sin(6 x1)) (pdo.py:166-187)."""
    psi = lambda s: 1 - 0.25 * torch.sin(6 * s)
    z = lambda xx: (xx[:, 0], xx[:, 1] / psi(xx[:, 0]))
    return _mapped_pdo(
        kh, bfield, z,
        y1_d=(lambda zz: torch.ones(zz.shape[0], dtype=zz.dtype, device=zz.device), None),
        y2_d=(lambda zz: zz[:, 1] * (-0.25 * 6 * torch.cos(6 * zz[:, 0])), lambda zz: psi(zz[:, 0])),
        y2_dd=(lambda zz: zz[:, 1] * (0.25 * 36 * torch.sin(6 * zz[:, 0])), None))


def get_param_map_and_pdo(geom, bfield, kh):
    """(op, param_map, inv_param_map) as src_disc/pdo.py:321-333.  'square' is the
    identity map; 'annulus', 'curvy_annulus' and 'sinusoidal' / 'curved' give
    operators with a mixed derivative (c12), for which Domain_Solver runs the
    reference's c12 leaf branch (the annulus's map is orthogonal, so its c12 is
    zero to rounding)."""
    if geom == 'square':
        ident = lambda xx: xx.clone()
        return PDO_2d(const(1), const(1), c=lambda xx: bfield(xx, kh)), ident, ident
    table = {'annulus': _annulus, 'curvy_annulus': _curvy_annulus, 'sinusoidal': _sinusoidal,
             'curved': _sinusoidal}
    if geom not in table:
        raise ValueError(f'geom {geom} not available')
    op, pmap = table[geom](kh, bfield)
    return op, pmap, _INVERSE[geom]


def _inv_annulus(zz):
    t = 1 / (np.pi / 3)
    return torch.stack((t * torch.atan2(zz[:, 1], zz[:, 0]), _radius(zz) - 1), dim=1)


def _inv_curvy(zz):
    t = 1 / (np.pi / 3)
    th = torch.arctan2(zz[:, 1], zz[:, 0])
    return torch.stack((t * th, _radius(zz) - 0.2 * torch.cos(5 * th) - 1), dim=1)


def _inv_sinusoidal(zz):
    return torch.stack((zz[:, 0], zz[:, 1] * (1 - 0.25 * torch.sin(6 * zz[:, 0]))), dim=1)


_INVERSE = {'annulus': _inv_annulus, 'curvy_annulus': _inv_curvy, 'sinusoidal': _inv_sinusoidal,
            'curved': _inv_sinusoidal}
