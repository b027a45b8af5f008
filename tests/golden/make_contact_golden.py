"""Generates tests/golden/contact_table.json: entries of the contact-interaction
propagator table (prop_rel_interpolate_terms, src/propagator.jl:36-73 of
oameye/PIMC.jl) evaluated independently of the engine with scipy's adaptive
quadrature and scipy's Bessel functions.

The reference integrates, for every (r1, r2) on the grid
r_i = 1e-20 + i (range - 1e-20)/(n - 1),

    T(r1, r2) = (1/2pi) int_0^inf k exp(-tau k^2) [ -t^2/(1+t^2) J0(k r1) J0(k r2)
                 - t/(1+t^2) (J0(k r1) Y0(k r2) + J0(k r2) Y0(k r1))
                 + t^2/(1+t^2) Y0(k r1) Y0(k r2) ] dk,
    t(k) = 1 / ((2/pi)(gamma + log(k/2)) - 4/g0)

(Gautier et al., supplementary S28), with QuadGK at rtol 1e-11.  This script
restates that formula, integrates it panel by panel (graded panels near
k = 0, quarter-period panels of the Bessel products above) to
sqrt(50/tau), where the Gaussian factor is below 2e-22, and records the
values.  The reference's stored tables (JLD2 files under Store/) are not part
of its repository, so these entries pin the engine's device table instead.

The configurations are the reference's own: g0 = 1.16, tau = 0.01, range 6
(the table its periodic Levy test loads), and g0 = 2 and 20 at
tau = 1/(T M) = 1/(0.2 * 200), range ceil(sqrt(8^2 + 8^2)) = 12
(examples/density_SRL_lattice.jl).

Run from the repository root: python tests/golden/make_contact_golden.py
"""
import json
import math
import os

import numpy as np
from scipy import integrate, special

EULER_GAMMA = 0.57721566490153286
HERE = os.path.dirname(os.path.abspath(__file__))

CONFIGS = [
    dict(g0=1.16, tau=0.01, range=6.0, n=600),
    dict(g0=2.0, tau=1.0 / (0.2 * 200), range=12.0, n=600),
    dict(g0=20.0, tau=1.0 / (0.2 * 200), range=12.0, n=600),
]

# (i1, i2) grid indices: the diagonal, near-diagonal, off-diagonal and far
# corners of the table
INDEX_PAIRS = [
    (0, 0), (1, 1), (5, 5), (50, 50), (300, 300), (599, 599),
    (10, 12), (40, 45), (100, 103), (20, 21),
    (0, 10), (5, 40), (0, 3), (200, 260), (100, 300), (0, 599),
]


def integrand(k, r1, r2, g0, tau):
    t = 1.0 / ((2.0 / math.pi) * (EULER_GAMMA + math.log(k / 2.0)) - 4.0 / g0)
    wa = t * t / (1.0 + t * t)
    wb = t / (1.0 + t * t)
    j1, j2 = special.j0(k * r1), special.j0(k * r2)
    y1, y2 = special.y0(k * r1), special.y0(k * r2)
    return k * math.exp(-tau * k * k) * (-wa * j1 * j2 - wb * (j1 * y2 + j2 * y1) + wa * y1 * y2)


def entry(r1, r2, g0, tau):
    kmax = math.sqrt(50.0 / tau)
    edges = [0.0, 1e-14, 1e-12, 1e-10, 1e-8, 1e-6, 1e-4, 1e-3, 1e-2, 0.1, 0.5]
    width = min(0.5, math.pi / (2.0 * (r1 + r2) + 1e-300))
    k = 0.5
    while k < kmax:
        k = min(kmax, k + width)
        edges.append(k)
    total = 0.0
    for a, b in zip(edges[:-1], edges[1:]):
        v, _ = integrate.quad(integrand, a, b, args=(r1, r2, g0, tau), epsabs=1e-20,
                              epsrel=1e-14, limit=200)
        total += v
    return total / (2.0 * math.pi)


def main():
    out = {"generator": "tests/golden/make_contact_golden.py", "configs": []}
    for c in CONFIGS:
        n, rng = c["n"], c["range"]
        grid = 1e-20 + np.arange(n) * ((rng - 1e-20) / (n - 1))
        ents = []
        for i1, i2 in INDEX_PAIRS:
            v = entry(float(grid[i1]), float(grid[i2]), c["g0"], c["tau"])
            ents.append([i1, i2, v])
            print(c["g0"], i1, i2, v, flush=True)
        out["configs"].append(dict(c, entries=ents))
    with open(os.path.join(HERE, "contact_table.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
