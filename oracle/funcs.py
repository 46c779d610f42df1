"""Oracle: coefficient fields and Dirichlet data (test infrastructure only).

Restates src_disc/built_in_funcs.py:59-70 (uu_dir_func_greens),
:79-80 (bfield_constant) and :208-217 (bfield_gaussian_bumps) in NumPy.
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
