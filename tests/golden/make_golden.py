"""Generate tests/golden/golden.json: the reference's own known answers.

* the N=1 2D harmonic thermal energy hard-coded in
  examples/energy_2d_harmonically_trapped_bose_gas.jl:28 (coth(1/2));
* exact canonical energies from the Z_N recursion of
  examples/tools/energytools.jl:3-21 (continuum, z(beta) of the oscillator),
  and the same recursion with the M-slice primitive-action single-particle
  partition function (what the primitive thermodynamic estimator averages to);
* the periodic free Bose gas (winding-0 sector and full lattice sum).
The recursion is restated here with mpmath (ForwardDiff becomes a central
difference at 60 digits).  Run: python tests/golden/make_golden.py
"""
import json
import os

import mpmath as mp

mp.mp.dps = 60


def Z_rec(N, z1, beta):
    Z = [mp.mpf(1)]
    for n in range(1, N + 1):
        Z.append(sum(z1(k * beta) * Z[n - k] for k in range(1, n + 1)) / n)
    return Z[N]


def energy(N, z1, beta):
    h = mp.mpf("1e-20")
    f = lambda b: mp.log(Z_rec(N, z1, b))
    return -(f(beta + h) - f(beta - h)) / (2 * h)


def z_ho(d):
    # (exp(-beta/2)/(1-exp(-beta)))^d  (energytools.jl:3-5)
    return lambda b: (mp.exp(-b / 2) / (1 - mp.exp(-b))) ** d


def energy_primitive(N, beta, M, d=2):
    """exact average of the primitive thermodynamic estimator for N bosons in
    the d-dimensional oscillator (omega = 1, lambda = 1/2) with M slices: a
    k-cycle is a closed Gaussian chain of kM beads, tau = beta/M, whose
    circulant determinant gives z_k = (2 sinh(kM theta/2))^-d with
    cosh(theta) = 1 + tau^2/2; E = -d ln Z_N / d beta at fixed M"""
    def lnZ(b):
        tau = b / M
        th = mp.acosh(1 + tau ** 2 / 2)
        z = lambda k: (1 / (2 * mp.sinh(k * M * th / 2))) ** d
        Z = [mp.mpf(1)]
        for n in range(1, N + 1):
            Z.append(sum(z(k) * Z[n - k] for k in range(1, n + 1)) / n)
        return mp.log(Z[N])
    h = mp.mpf("1e-20")
    return -(lnZ(beta + h) - lnZ(beta - h)) / (2 * h)


def free_periodic(N, beta, side, lam, d=2, kmax=60):
    """ideal bosons on a periodic square of side `side`: z(b) = (sum_n
    exp(-b lam (2 pi n / side)^2))^d; winding-0 keeps only the Gaussian
    integral of the unwrapped free propagator, z0 = (side/sqrt(4 pi lam b))^d"""
    def z_full(b):
        s = mp.nsum(lambda n: mp.exp(-b * lam * (2 * mp.pi * n / side) ** 2), [-mp.inf, mp.inf])
        return s ** d

    def z_w0(b):
        return (side / mp.sqrt(4 * mp.pi * lam * b)) ** d
    return energy(N, z_full, beta), energy(N, z_w0, beta)


def main():
    out = {}
    out["E_N1_d2_beta1_reference_constant"] = 2.1639534137386534
    out["E_N1_d2_beta1"] = float(energy(1, z_ho(2), mp.mpf(1)))
    out["E_C1_exact"] = float(energy(10, z_ho(2), mp.mpf(1)))
    out["E_C1_boltzmannon"] = float(10 * energy(1, z_ho(2), mp.mpf(1)))
    out["E_C1_primitive_M20"] = float(energy_primitive(10, mp.mpf(1), 20))
    out["E_N1_primitive_M20"] = float(energy_primitive(1, mp.mpf(1), 20))
    out["E_N2_primitive_M8"] = float(energy_primitive(2, mp.mpf(1), 8))
    out["E_N4_primitive_M8"] = float(energy_primitive(4, mp.mpf(1), 8))
    full, w0 = free_periodic(64, mp.mpf(2), mp.mpf(20), mp.mpf("0.5"))
    out["E_C2_lattice_sum"] = float(full)
    out["E_C2_winding0"] = float(w0)
    for N in (1, 2, 3, 5):
        out[f"E_N{N}_d2_beta1"] = float(energy(N, z_ho(2), mp.mpf(1)))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
