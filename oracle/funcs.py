"""Oracle: coefficient fields and Dirichlet data (test infrastructure only).

Restates src_disc/built_in_funcs.py:59-70 (uu_dir_func_greens),
:79-80 (bfield_constant) and :208-217 (bfield_gaussian_bumps), and the annulus
parameter map of src_disc/pdo.py (:44-159 pdo_param and the c*_func helpers,
:196-215 the 'annulus' branch of get_param_helper) in NumPy.
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


def annulus_pdo(kh, bfield):
    """Helmholtz on the annulus, pulled back to the unit square (pdo.py:196-215).

    Returns (pdo dict of coefficient callables on the square, parameter map
    square -> annulus).  The reference drops the second derivatives of y1
    (y1_d1d1 = y1_d2d2 = None), so c1 is absent."""
    ct = 1 / (np.pi / 3)

    def param_map(xx):
        rad = 1 + 1 * xx[:, 1]
        return np.stack((rad * np.cos(xx[:, 0] / ct), rad * np.sin(xx[:, 0] / ct)), axis=1)

    r = lambda zz: (zz[:, 0] ** 2 + zz[:, 1] ** 2) ** 0.5
    y1_d1 = lambda zz: -ct * (zz[:, 1] / r(zz) ** 2)
    y1_d2 = lambda zz: +ct * (zz[:, 0] / r(zz) ** 2)
    y2_d1 = lambda zz: zz[:, 0] / r(zz)
    y2_d2 = lambda zz: zz[:, 1] / r(zz)
    y2_d1d1 = lambda zz: zz[:, 1] ** 2 / r(zz) ** 3
    y2_d2d2 = lambda zz: zz[:, 0] ** 2 / r(zz) ** 3

    def c11(xx):
        yy = param_map(xx)
        return (0 + y1_d1(yy) ** 2) + y1_d2(yy) ** 2

    def c22(xx):
        yy = param_map(xx)
        return (0 + y2_d1(yy) ** 2) + y2_d2(yy) ** 2

    def c2(xx):
        yy = param_map(xx)
        return (0 - y2_d1d1(yy)) - y2_d2d2(yy)

    def c12(xx):
        yy = param_map(xx)
        return (0 + y1_d1(yy) * y2_d1(yy)) + y1_d2(yy) * y2_d2(yy)

    def c(xx):
        return bfield(param_map(xx), kh)

    return {'c11': c11, 'c22': c22, 'c12': c12, 'c2': c2, 'c': c}, param_map
