"""Partial differential operator container (src_disc/pdo.py:6-12, 31-38).

-c11 u_xx - c22 u_yy - 2 c12 u_xy + c1 u_x + c2 u_y + c u = f, each
coefficient a callable of an (N, 2) torch tensor of points, or None.
"""
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
