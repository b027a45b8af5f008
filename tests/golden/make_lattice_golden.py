"""Generates tests/golden/lattice_angles.json: the named beam-angle sets of
the reference's optical-lattice potentials (the l25 and l65 arrays of
examples/tools/potentialtools.jl in oameye/PIMC.jl), read from that file, so
that the engine's construction of them (directions of the integer points on
the circles x^2 + y^2 = 25 and 65) is checked against the reference's numbers.

Run with the path of a checkout of the reference project:

    python tests/golden/make_lattice_golden.py <reference checkout>
"""
import argparse
import json
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
REL = os.path.join("examples", "tools", "potentialtools.jl")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference", help="root of a checkout of oameye/PIMC.jl")
    args = ap.parse_args()
    text = open(os.path.join(args.reference, REL)).read()
    out = {"generator": "tests/golden/make_lattice_golden.py",
           "source": "examples/tools/potentialtools.jl (top-level l25 and l65)"}
    for name in ("l25", "l65"):
        m = re.search(r"^" + name + r"\s*=\s*\[([^\]]*)\]", text, re.M)
        vals = [float(v) for v in re.split(r"[,\s]+", m.group(1).strip()) if v]
        out[name] = vals
    with open(os.path.join(HERE, "lattice_angles.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
