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

(Gautier et al., supplementary S28), with QuadGK at rtol 1e-11.  The values
come from oracle/contact_table.py, which integrates that formula adaptively
with scipy's QUADPACK (the device uses a fixed composite Gauss-Legendre
rule).  The reference's stored tables (JLD2 files under Store/) are not part
of its repository, so these entries pin the engine's device table instead.

The configurations are the reference's own: g0 = 1.16, tau = 0.01, range 6
(the table its periodic Levy test loads), and g0 = 2 and 20 at
tau = 1/(T M) = 1/(0.2 * 200), range ceil(sqrt(8^2 + 8^2)) = 12
(examples/density_SRL_lattice.jl).

Run from the repository root: python tests/golden/make_contact_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.contact_table import entry, grid  # noqa: E402

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


def main():
    out = {"generator": "tests/golden/make_contact_golden.py", "configs": []}
    for c in CONFIGS:
        r = grid(c["range"], c["n"])
        ents = []
        for i1, i2 in INDEX_PAIRS:
            v = entry(float(r[i1]), float(r[i2]), c["g0"], c["tau"])
            ents.append([i1, i2, v])
            print(c["g0"], i1, i2, v, flush=True)
        out["configs"].append(dict(c, entries=ents))
    with open(os.path.join(HERE, "contact_table.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
