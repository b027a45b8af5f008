"""CPU restatement of the contact-interaction propagator table -- TEST
INFRASTRUCTURE ONLY (the golden fixtures and the bench's CPU baseline use it;
the engine builds its table on the device and never calls this).

prop_rel_interpolate_terms (src/propagator.jl:36-73 of oameye/PIMC.jl)
integrates, for every (r1, r2) of the grid r_i = 1e-20 + i (range - 1e-20)/(n - 1),

    T(r1, r2) = (1/2pi) int_0^inf k exp(-tau k^2) [ -t^2/(1+t^2) J0(k r1) J0(k r2)
                 - t/(1+t^2) (J0(k r1) Y0(k r2) + J0(k r2) Y0(k r1))
                 + t^2/(1+t^2) Y0(k r1) Y0(k r2) ] dk,
    t(k) = 1 / ((2/pi)(gamma + log(k/2)) - 4/g0)

(Gautier et al., supplementary S28) with adaptive Gauss-Kronrod quadrature
(QuadGK, rtol 1e-11).  Here the same formula is integrated adaptively with
scipy's QUADPACK, panel by panel: graded panels near k = 0, then panels of a
quarter period of the Bessel products, up to sqrt(50/tau) where the Gaussian
factor is below 2e-22.
"""
import math
import warnings

import numpy as np
from scipy import integrate, special

EULER_GAMMA = 0.57721566490153286


def grid(range_, n):
    """the reference's radii: range(1e-20, range_, n)"""
    return 1e-20 + np.arange(n) * ((range_ - 1e-20) / (n - 1))


def integrand(k, r1, r2, g0, tau):
    t = 1.0 / ((2.0 / math.pi) * (EULER_GAMMA + math.log(k / 2.0)) - 4.0 / g0)
    wa = t * t / (1.0 + t * t)
    wb = t / (1.0 + t * t)
    j1, j2 = special.j0(k * r1), special.j0(k * r2)
    y1, y2 = special.y0(k * r1), special.y0(k * r2)
    return k * math.exp(-tau * k * k) * (-wa * j1 * j2 - wb * (j1 * y2 + j2 * y1) + wa * y1 * y2)


def entry(r1, r2, g0, tau):
    """T(r1, r2) by adaptive quadrature"""
    kmax = math.sqrt(50.0 / tau)
    edges = [0.0, 1e-14, 1e-12, 1e-10, 1e-8, 1e-6, 1e-4, 1e-3, 1e-2, 0.1, 0.5]
    width = min(0.5, math.pi / (2.0 * (r1 + r2) + 1e-300))
    k = 0.5
    while k < kmax:
        k = min(kmax, k + width)
        edges.append(k)
    total = 0.0
    with warnings.catch_warnings():
        # tiny entries reach the roundoff floor before epsrel
        warnings.simplefilter("ignore", integrate.IntegrationWarning)
        for a, b in zip(edges[:-1], edges[1:]):
            v, _ = integrate.quad(integrand, a, b, args=(r1, r2, g0, tau), epsabs=1e-20,
                                  epsrel=1e-14, limit=200)
            total += v
    return total / (2.0 * math.pi)
