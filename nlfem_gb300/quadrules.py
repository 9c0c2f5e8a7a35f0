"""Quadrature rules used by the assembly.

The triangle rules are the published symmetric rules of Dunavant (1985) and the 11-point
tetrahedral rule of Keast (1986). They are written here from the published formulas/tables,
with the same point order the reference configurations use
(examples/test2D/conf/testConfFractional.py:27-77 lists the 7- and 16-point rules with truncated
digits). Weights are scaled to the reference element's volume (1/2 for the triangle, 1/6 for the
tetrahedron), as the reference expects (checks.cpp:25-34).

``tensorgauss`` builds the deg^4 Gauss-Legendre tensor rule on [-1, 1]^4 that the singular
close-pair (Duffy) quadrature consumes; it follows cython/nlfem.pyx:108-126 (points in C order
of the multi-index, last index fastest; weight = product of the 1-D weights).
"""
import numpy as np

__all__ = ["dunavant7", "dunavant16", "keast11", "centroid1", "tensorgauss"]


def centroid1():
    """One-point centroid rule on the reference triangle."""
    return np.array([[1.0 / 3.0, 1.0 / 3.0]]), np.array([0.5])


def dunavant7():
    """7-point, degree-5 rule (Radon / Dunavant #5) in closed form."""
    s15 = np.sqrt(15.0)
    a = (6.0 - s15) / 21.0
    b = (6.0 + s15) / 21.0
    wa = (155.0 - s15) / 1200.0
    wb = (155.0 + s15) / 1200.0
    P = np.array([
        [1.0 / 3.0, 1.0 / 3.0],
        [b, b], [b, 1.0 - 2.0 * b], [1.0 - 2.0 * b, b],
        [a, a], [a, 1.0 - 2.0 * a], [1.0 - 2.0 * a, a],
    ])
    w = 0.5 * np.array([9.0 / 40.0, wb, wb, wb, wa, wa, wa])
    return P, w


def dunavant16():
    """16-point, degree-8 rule (Dunavant #8)."""
    a1, w1 = 0.459292588292723, 0.095091634267285
    a2, w2 = 0.170569307751760, 0.103217370534718
    a3, w3 = 0.050547228317031, 0.032458497623198
    b, c, w4 = 0.263112829634638, 0.728492392955404, 0.027230314174435
    d = 1.0 - b - c
    P = np.array([
        [1.0 / 3.0, 1.0 / 3.0],
        [a1, a1], [a1, 1 - 2 * a1], [1 - 2 * a1, a1],
        [a2, a2], [a2, 1 - 2 * a2], [1 - 2 * a2, a2],
        [a3, a3], [a3, 1 - 2 * a3], [1 - 2 * a3, a3],
        [b, c], [c, d], [d, b], [c, b], [b, d], [d, c],
    ])
    w = 0.5 * np.array([0.144315607677787, w1, w1, w1, w2, w2, w2, w3, w3, w3,
                        w4, w4, w4, w4, w4, w4])
    return P, w


def keast11():
    """11-point, degree-4 tetrahedral rule (Keast 1986); weights sum to 1/6, one is negative."""
    r = np.sqrt(5.0 / 14.0)
    c = (1.0 + r) / 4.0
    d = (1.0 - r) / 4.0
    a, b = 1.0 / 14.0, 11.0 / 14.0
    pts = [[0.25, 0.25, 0.25]]
    w = [-74.0 / 5625.0]
    for p in ([b, a, a], [a, b, a], [a, a, b], [a, a, a]):
        pts.append(p)
        w.append(343.0 / 45000.0)
    for p in ([c, c, d], [c, d, c], [c, d, d], [d, c, c], [d, c, d], [d, d, c]):
        pts.append(p)
        w.append(56.0 / 2250.0)
    return np.array(pts), np.array(w)


class tensorgauss:
    """deg^dim tensor Gauss-Legendre rule on [-1, 1]^dim (cython/nlfem.pyx:108-126)."""

    def __init__(self, deg, dim=4):
        self.deg = int(deg)
        self.dim = int(dim)
        p, w = np.polynomial.legendre.leggauss(self.deg)
        self.N = self.deg ** self.dim
        idx = np.indices([self.deg] * self.dim).reshape(self.dim, -1).T  # C order, last fastest
        self.points = p[idx]
        self.weights = np.ones(self.N)
        for j in range(self.dim):
            self.weights = self.weights * w[idx[:, j]]
