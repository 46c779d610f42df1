"""Oracle: coefficient fields and Dirichlet data (test infrastructure only).

Restates src_disc/built_in_funcs.py:59-70 (uu_dir_func_greens),
:79-80 (bfield_constant) and :208-217 (bfield_gaussian_bumps), and the
parameter maps of curved domains in src_disc/pdo.py (:36-161 pdo_param and the
c*_func helpers; get_param_helper :164-319: 'sinusoidal' / 'curved'
:166-187, 'annulus' :189-215, 'curvy_annulus' :217-282) in NumPy.
"""
import numpy as np
from scipy.special import hankel1


def uu_dir_greens(xx, kh, center=(-0.1, 0.5)):
    d0 = xx[:, 0] - center[0]
    d1 = xx[:, 1] - center[1]
    r2 = d0 * d0 + d1 * d1
    if kh == 0:
        return ((1 / np.pi) * np.log(r2))[:, None]
    return np.real((1j / 4) * hankel1(0, kh * np.sqrt(r2)))[:, None]


def bfield_constant(xx, kh):
    return -(kh ** 2) * np.ones(xx.shape[0])


def bfield_gaussian_bumps(xx, kh):
    r0 = (xx[:, 0] - 0.5) ** 2 + (xx[:, 1] - 0.5) ** 2
    r1 = (xx[:, 0] - 0.25) ** 2 + (xx[:, 1] - 0.5) ** 2
    b = np.exp(-2000 * r0) + np.exp(-2000 * r1)
    return -(kh ** 2) * (1 - b)


def helmholtz_pdo(cfun):
    """c11 = c22 = 1, c = cfun(xx) (argparse_driver.py:115-118)."""
    one = lambda xx: np.ones(xx.shape[0])
    return {'c11': one, 'c22': one, 'c': cfun}


def _pdo_param(kh, bfield, z1, z2, y1_d1=None, y1_d2=None, y2_d1=None, y2_d2=None,
               y1_d1d1=None, y1_d2d2=None, y2_d1d1=None, y2_d2d2=None):
    """Coefficients on the reference rectangle of Helmholtz on a mapped domain
    (pdo.py:36-161).  z maps the rectangle to the domain; the y_* are the
    derivatives of the inverse map, evaluated at mapped points.  Each
    coefficient is summed from zero in the reference's term order:
      c11 = y1_d1^2 + y1_d2^2,  c22 = y2_d1^2 + y2_d2^2,
      c1 = -y1_d1d1 - y1_d2d2,  c2 = -y2_d1d1 - y2_d2d2,
      c12 = y1_d1 y2_d1 + y1_d2 y2_d2,  c = bfield(z(x), kh);
    a coefficient whose terms are all absent is absent (None).  Returns (pdo
    dict of coefficient callables, parameter map rectangle -> domain)."""

    def param_map(xx):
        return np.stack((z1(xx), z2(xx)), axis=1)

    def combine(terms, sign):
        terms = [t for t in terms if t is not None]
        if not terms:
            return None

        def f(xx):
            yy = param_map(xx)
            out = 0
            for t in terms:
                out = out + t(yy) if sign > 0 else out - t(yy)
            return out
        return f

    sq = lambda g: None if g is None else (lambda yy: g(yy) ** 2)
    both = lambda g, h: None if (g is None or h is None) else (lambda yy: g(yy) * h(yy))
    pdo = {
        'c11': combine([sq(y1_d1), sq(y1_d2)], 1),
        'c22': combine([sq(y2_d1), sq(y2_d2)], 1),
        'c1': combine([y1_d1d1, y1_d2d2], -1),
        'c2': combine([y2_d1d1, y2_d2d2], -1),
        'c12': combine([both(y1_d1, y2_d1), both(y1_d2, y2_d2)], 1),
        'c': lambda xx: bfield(param_map(xx), kh),
    }
    return {k: v for k, v in pdo.items() if v is not None}, param_map


def annulus_pdo(kh, bfield):
    """Helmholtz on the annulus 1 <= r <= 2, 0 <= theta <= 2 pi / 6 * x1-range,
    pulled back to the rectangle (pdo.py:189-215).  The reference drops the
    second derivatives of y1 (y1_d1d1 = y1_d2d2 = None), so c1 is absent."""
    ct = 1 / (np.pi / 3)
    r = lambda zz: (zz[:, 0] ** 2 + zz[:, 1] ** 2) ** 0.5
    return _pdo_param(
        kh, bfield,
        z1=lambda xx: (1 + 1 * xx[:, 1]) * np.cos(xx[:, 0] / ct),
        z2=lambda xx: (1 + 1 * xx[:, 1]) * np.sin(xx[:, 0] / ct),
        y1_d1=lambda zz: -ct * (zz[:, 1] / r(zz) ** 2),
        y1_d2=lambda zz: +ct * (zz[:, 0] / r(zz) ** 2),
        y2_d1=lambda zz: zz[:, 0] / r(zz),
        y2_d2=lambda zz: zz[:, 1] / r(zz),
        y2_d1d1=lambda zz: zz[:, 1] ** 2 / r(zz) ** 3,
        y2_d2d2=lambda zz: zz[:, 0] ** 2 / r(zz) ** 3)


def curvy_annulus_pdo(kh, bfield):
    """Helmholtz on the annulus with a wavy inner and outer boundary,
    r = 1 + 0.2 cos(5 theta) + x2, theta = x1 pi / 3 (pdo.py:217-282).  With x1 in
    [0, 6] the rectangle wraps once around the origin, and its left and right
    edges are the same curve (the periodic case of the reference's tests)."""
    ct, ph, amp = 1 / (np.pi / 3), 5, 0.2
    r = lambda zz: (zz[:, 0] ** 2 + zz[:, 1] ** 2) ** 0.5
    rad = lambda xx: 1 + amp * np.cos(ph * xx[:, 0] / ct) + xx[:, 1]
    th = lambda zz: np.arctan2(zz[:, 1], zz[:, 0])

    def y2_d1(zz):
        out = zz[:, 0] / r(zz)
        t = np.sin(ph * th(zz)) / r(zz) ** 2
        return out - amp * ph * (zz[:, 1] * t)

    def y2_d2(zz):
        out = zz[:, 1] / r(zz)
        t = np.sin(ph * th(zz)) / r(zz) ** 2
        return out + (amp * ph * zz[:, 0]) * t

    def y2_d1d1(zz):
        out = zz[:, 1] ** 2 / r(zz) ** 3
        t1 = zz[:, 0] * np.sin(ph * th(zz))
        t2 = zz[:, 1] * np.cos(ph * th(zz))
        return out + amp * ph * ((zz[:, 1] * (2 * t1 + ph * t2)) / r(zz) ** 4)

    def y2_d2d2(zz):
        out = zz[:, 0] ** 2 / r(zz) ** 3
        t1 = zz[:, 0] * np.cos(ph * th(zz))
        t2 = zz[:, 1] * np.sin(ph * th(zz))
        return out + amp * ph * ((zz[:, 0] * (ph * t1 - 2 * t2)) / r(zz) ** 4)

    return _pdo_param(
        kh, bfield,
        z1=lambda xx: rad(xx) * np.cos(xx[:, 0] / ct),
        z2=lambda xx: rad(xx) * np.sin(xx[:, 0] / ct),
        y1_d1=lambda zz: -ct * (zz[:, 1] / r(zz) ** 2),
        y1_d2=lambda zz: +ct * (zz[:, 0] / r(zz) ** 2),
        y1_d1d1=lambda zz: +2 * ct * ((zz[:, 0] * zz[:, 1]) / r(zz) ** 4),
        y1_d2d2=lambda zz: -2 * ct * ((zz[:, 0] * zz[:, 1]) / r(zz) ** 4),
        y2_d1=y2_d1, y2_d2=y2_d2, y2_d1d1=y2_d1d1, y2_d2d2=y2_d2d2)


def sinusoidal_pdo(kh, bfield):
    """Helmholtz on the strip under the curve x2 = 1 / (1 - 0.25 sin(6 x1)), pulled
    back to the rectangle (pdo.py:166-187; the driver's 'curved' domain)."""
    mag = 0.25
    psi = lambda z: 1 - mag * np.sin(6 * z)
    dpsi = lambda z: -mag * 6 * np.cos(6 * z)
    ddpsi = lambda z: mag * 36 * np.sin(6 * z)
    return _pdo_param(
        kh, bfield,
        z1=lambda xx: xx[:, 0],
        z2=lambda xx: xx[:, 1] / psi(xx[:, 0]),
        y1_d1=lambda zz: np.ones(zz.shape[0]),
        y2_d1=lambda zz: zz[:, 1] * dpsi(zz[:, 0]),
        y2_d2=lambda zz: psi(zz[:, 0]),
        y2_d1d1=lambda zz: zz[:, 1] * ddpsi(zz[:, 0]))


def param_pdo(geom, kh, bfield):
    """pdo.get_param_map_and_pdo for the curved domains: (pdo dict, parameter map)."""
    table = {'annulus': annulus_pdo, 'curvy_annulus': curvy_annulus_pdo,
             'sinusoidal': sinusoidal_pdo, 'curved': sinusoidal_pdo}
    if geom not in table:
        raise ValueError(f'geom {geom} not available')
    return table[geom](kh, bfield)
