"""The reference package's user API (oameye/PIMC.jl) over the GB300 engine.

Mirrors the names, keyword arguments and fields a PIMC.jl user touches:

    System(potential; dV, dim, M, N, mu, L, T, lambda, interactions, propint,
           g, r_a, length_measurement_cycle, measure_scheme)   src/system.jl:129-167
    ReshapeLinear / ReshapeSwapLinear (s, slices; ...)          src/updates/reshape.jl:7-29,99-121
    SingleCenterOfMass / PolymerCenterOfMass (s, step; ...)     src/updates/com.jl:7-28,112-133
    run!(s, n, updates; Zmeasurements)  -> run(...)             src/simulation.jl:29-42
    apply!(s, f) -> apply(...), acceptance(q)                   src/simulation.jl:1-27
    Density(s; nbins), Energy(s, n)                             src/measurement.jl:31-122

Julia closures cannot cross the C ABI, so ``potential``, ``dV`` and
``propint`` must be engine-known callables (Harmonic, SquareLattice, sums of
them, GaussianPair); anything else raises -- there is no CPU fallback.
Slices and particle indices are 0-based here.
"""
from __future__ import annotations

import math
from collections import deque

import numpy as np

from .engine import (ACCEPT, SEM_PHYSICAL, SEM_REFERENCE, SKIP, ChainParams, Engine,
                     Mix, PimcError, contact_table, julia_float, write_density_csv)


# --------------------------------------------------------------- potentials
class Harmonic:
    """V(r) = omega^2 |r|^2 / 2; callable like the reference's closures."""

    def __init__(self, omega: float = 1.0):
        self.omega = float(omega)

    def __call__(self, r):
        r = np.asarray(r, dtype=float)
        return 0.5 * self.omega ** 2 * float(np.dot(r, r))

    def grad(self, r):
        return self.omega ** 2 * np.asarray(r, dtype=float)


class SquareLattice:
    """V(r) = V0 sum_d sin^2(pi r_d / a)."""

    def __init__(self, V0: float, a: float = 1.0):
        self.V0, self.a = float(V0), float(a)

    def __call__(self, r):
        r = np.asarray(r, dtype=float)
        return self.V0 * float(np.sum(np.sin(np.pi * r / self.a) ** 2))

    def grad(self, r):
        r = np.asarray(r, dtype=float)
        return self.V0 * (np.pi / self.a) * np.sin(2 * np.pi * r / self.a)


class OpticalLattice:
    """depth * normalized_intensity(r, angles, scale; helical) of
    examples/tools/potentialtools.jl:1-16: K plane waves along (sin a, cos a),
    phases 2 pi scale (r . (sin a, cos a)) (+ a when helical), the squared
    modulus of their mean.  Two-dimensional, at most 16 beams."""

    def __init__(self, angles, scale: float, depth: float, helical: bool = False):
        self.angles = [float(a) for a in angles]
        if not 0 < len(self.angles) <= 16:
            raise PimcError("an optical lattice has between 1 and 16 beams")
        self.scale, self.depth, self.helical = float(scale), float(depth), bool(helical)

    def _phases(self, r):
        a = np.asarray(self.angles)
        ph = 2 * np.pi * (r[0] * np.sin(a) + r[1] * np.cos(a)) * self.scale
        return a, ph + a if self.helical else ph

    def __call__(self, r):
        _, ph = self._phases(r)
        return self.depth * (np.mean(np.sin(ph)) ** 2 + np.mean(np.cos(ph)) ** 2)

    def grad(self, r):
        a, ph = self._phases(r)
        s, c = np.mean(np.sin(ph)), np.mean(np.cos(ph))
        w = 2 * np.pi * self.scale
        d = np.stack([np.sin(a), np.cos(a)])  # dphi/dr per beam, over w
        return self.depth * 2 * w * (s * (d @ np.cos(ph)) - c * (d @ np.sin(ph))) / len(a)

    def __add__(self, other):
        return PotentialSum(self, other)


def lattice_angles(sym: str):
    """the beam sets of generate_V (potentialtools.jl:18-39): "l25" and "l65"
    point the beams at the integer points of the circles x^2 + y^2 = 25 and 65
    (12 and 16 beams), a = atan2(x, y) so that (sin a, cos a) = (x, y)/R;
    "cubic" is 2 pi k / 4, k = 0..3"""
    if sym == "cubic":
        return [2 * math.pi * k / 4 for k in range(4)]
    r2 = {"l25": 25, "l65": 65}.get(sym)
    if r2 is None:
        raise PimcError(f"unknown lattice {sym!r} (l25, l65, cubic, harmonic)")
    return sorted(math.atan2(x, y) for x in range(-9, 10) for y in range(-9, 10)
                  if x * x + y * y == r2)


def generate_V(*args, attractive: bool = True, helical: bool = False):
    """generate_V(scale, depth, sym; attractive) or generate_V(angles, scale,
    depth; helical) (potentialtools.jl:18-39); sym "harmonic" gives the unit
    trap 0.5 |r|^2"""
    if len(args) == 3 and isinstance(args[2], str):
        scale, depth, sym = args
        if sym == "harmonic":
            return Harmonic(1.0)
        return OpticalLattice(lattice_angles(sym), scale, -depth if attractive else depth)
    angles, scale, depth = args
    return OpticalLattice(angles, scale, depth, helical)


class PotentialSum:
    def __init__(self, *terms):
        self.terms = terms

    def __call__(self, r):
        return sum(t(r) for t in self.terms)

    def grad(self, r):
        return sum(t.grad(r) for t in self.terms)

    def __add__(self, other):
        return PotentialSum(*self.terms, other)


Harmonic.__add__ = lambda self, o: PotentialSum(self, o)
SquareLattice.__add__ = lambda self, o: PotentialSum(self, o)


class Zero:
    def __call__(self, r):
        return 0.0

    def grad(self, r):
        return np.zeros_like(np.asarray(r, dtype=float))


class GaussianPair:
    """Pair propagator of v(r) = g exp(-r^2 / 2 sigma^2) in primitive form:
    propint(r1, r2, tau) = exp(-tau/2 (v(|r1|) + v(|r2|)))."""

    def __init__(self, g: float, sigma: float):
        self.g, self.sigma = float(g), float(sigma)

    def v(self, r):
        return self.g * math.exp(-r * r / (2 * self.sigma ** 2))

    def __call__(self, r1, r2, tau):
        return math.exp(-0.5 * tau * (self.v(float(np.linalg.norm(r1))) + self.v(float(np.linalg.norm(r2)))))


class ContactPropagator:
    """build_prop_int(L, g0, tau) (src/propagator.jl:35-89): the contact
    interaction's propagator prop_int(r1, r2, tau) = 1 + T(|r1|, |r2|) /
    prop_rel0(r1, r2, tau), T bilinear in a table over [1e-20, L]^2 whose n x n
    Bessel integrals are computed on the device.  As the pair propagator of a
    System it runs on the device; calling it evaluates the same formula on
    the host (the reference's determine_nnrange calls it at set-up)."""

    def __init__(self, L: float, g0: float, τ: float, n: int = 600, table=None):
        self.range, self.g0, self.tau, self.n = float(L), float(g0), float(τ), int(n)
        if table is None:
            table = contact_table(self.g0, self.tau, self.range, self.n)
        self.table = np.ascontiguousarray(table, dtype=np.float64)
        if self.table.shape != (self.n, self.n):
            raise PimcError("the contact table must be n x n")
        self._h = (self.range - 1e-20) / (self.n - 1)

    def terms(self, r1: float, r2: float) -> float:
        """T(r1, r2) by the linear B-spline of the table (radii clamped)"""
        def cell(r):
            r = min(max(r, 1e-20), self.range)
            p = (r - 1e-20) / self._h
            f = min(math.floor(p), self.n - 2)
            return f, p - f
        i, wx = cell(float(r1))
        j, wy = cell(float(r2))
        t = self.table
        c0 = (1.0 - wy) * t[i, j] + wy * t[i, j + 1]
        c1 = (1.0 - wy) * t[i + 1, j] + wy * t[i + 1, j + 1]
        return (1.0 - wx) * c0 + wx * c1

    def __call__(self, r1_rel, r2_rel, τ):
        r1 = np.asarray(r1_rel, dtype=np.float64)
        r2 = np.asarray(r2_rel, dtype=np.float64)
        d = r1 - r2
        rel0 = math.exp(-float(np.dot(d, d)) / (4 * τ)) / (4 * math.pi * τ)
        return 1.0 + self.terms(float(np.linalg.norm(r1)), float(np.linalg.norm(r2))) / rel0


def build_prop_int(L: float, g0: float, τ: float, n: int = 600) -> ContactPropagator:
    """build_prop_int (src/propagator.jl:79-89); L is the table's range"""
    return ContactPropagator(L, g0, τ, n)


def determine_nnrange(propint, τ: float, a: float, b: float) -> float:
    """determine_nnrange (src/system.jl:10-15): the radius r > r_min where
    propint([r], [r], tau) = 0.999, r_min the minimiser of that curve.  The
    minimiser is taken on the table's grid (the reference runs Nelder-Mead
    from a); the root is bisected to the last bit, as Roots.Bisection does."""
    f = lambda r: propint([r], [r], τ) - 0.999
    grid = np.linspace(a, b, 4097)
    vals = np.array([f(r) for r in grid])
    lo = float(grid[int(np.argmin(vals))])
    hi = float(b)
    flo, fhi = f(lo), f(hi)
    if flo * fhi > 0:
        raise PimcError("determine_nnrange: propint - 0.999 has no sign change on (r_min, b)")
    while True:
        mid = 0.5 * (lo + hi)
        if mid <= lo or mid >= hi:
            break
        fm = f(mid)
        if fm == 0.0:
            return mid
        if (fm < 0) == (flo < 0):
            lo, flo = mid, fm
        else:
            hi = mid
    return lo if abs(flo) <= abs(f(hi)) else hi


def _potential_terms(potential):
    omega, V0, a, beams = 0.0, 0.0, 1.0, None
    terms = potential.terms if isinstance(potential, PotentialSum) else (potential,)
    for t in terms:
        if isinstance(t, Harmonic):
            omega = t.omega
        elif isinstance(t, SquareLattice):
            V0, a = t.V0, t.a
        elif isinstance(t, OpticalLattice):
            if beams is not None:
                raise PimcError("one optical lattice per potential")
            beams = t
        elif isinstance(t, Zero) or t is None:
            pass
        else:
            raise PimcError("potential must be Harmonic, SquareLattice, OpticalLattice, Zero or a "
                            "sum of them; arbitrary closures cannot run on the device")
    return omega, V0, a, beams


# --------------------------------------------------------------- world view
class Particle:
    """One path: r (M x dim), cached link actions V (M), next (0-based)."""

    def __init__(self, r, V, nxt):
        self.r, self.V, self.next = r, V, int(nxt)


class System:
    def __init__(self, potential=None, dV=None, dim: int = 2, M: int = 100, N: int = 2,
                 μ: float = 0.0, L: float = 4.0, T: float = 1.0, λ: float = 1.0,
                 interactions: bool = False, propint=None, g: float = 0.0, ra: float = 0.0,
                 length_measurement_cycle: int = 10, measure_scheme: str = "c",
                 semantics: int = SEM_REFERENCE, seed: int = 20261203, **kw):
        λ = kw.pop("lam", λ)
        μ = kw.pop("mu", μ)
        ra = kw.pop("r_a", ra)
        if kw:
            raise TypeError(f"unknown keyword arguments {sorted(kw)}")
        potential = Zero() if potential is None else potential
        omega, V0, a, beams = _potential_terms(potential)
        if beams is not None and dim != 2:
            raise PimcError("the optical lattice is two-dimensional")
        if dV is not None and not (dV is potential or getattr(dV, "__self__", None) is potential
                                   or dV in ("grad", np.asarray) or callable(dV)):
            raise PimcError("dV must be the potential's gradient")
        pair_g, pair_sigma = 0.0, 1.0
        contact = None
        if interactions:
            if isinstance(propint, GaussianPair):
                pair_g, pair_sigma = propint.g, propint.sigma
                if ra == 0.0:
                    raise PimcError("pass ra (the neighbour range) with a GaussianPair")
            elif isinstance(propint, ContactPropagator):
                contact = propint
                if ra == 0.0:
                    # init_int (src/system.jl:17-34)
                    ra = determine_nnrange(propint, 1.0 / (T * M), 1e-20, L)
            else:
                raise PimcError("interactions=True needs propint=GaussianPair(g, sigma) or "
                                "build_prop_int(L, g0, tau)")
        self.dim, self.M, self.N, self.Ninit = dim, M, N, N
        self.μ, self.λ, self.L = μ, λ, L
        self.vol = (2 * L) ** dim
        self.β = 1.0 / T
        self.τ = self.β / M
        # hard-core radius of the contact model (src/system.jl:151)
        self.a = math.exp(-2 * math.pi / g) if (interactions and g > 0) else 0.0
        self.ctr = 10_000
        self.V, self.dV, self.propint = potential, (dV or getattr(potential, "grad", None)), propint
        self.measure_scheme = measure_scheme
        self.N_MC = {N: 0}
        self.Nctr = {N: 0}
        self.Ncycle = length_measurement_cycle
        self.semantics = semantics
        self.rₐ = ra if ra > 0 else L / 4.0
        self.nbins = int(math.floor(2 * L / self.rₐ))
        self.rng = np.random.default_rng(seed)
        self._cp = ChainParams(dim=dim, N=N, M=M, L=L, T=T, lam=λ, mu=μ, harmonic_omega=omega,
                               lattice_V0=V0, lattice_a=a, interactions=interactions,
                               pair_g=pair_g, pair_sigma=pair_sigma, r_a=ra,
                               hardcore_a=self.a, semantics=semantics, seed=seed)
        self._contact = contact
        self._beams = beams
        self.engine = Engine(self._cp)
        self._attach()
        self._eser_seen = 0

    def _attach(self):
        """the parts of the potential that are set after creation"""
        if self._contact is not None:
            self.engine.set_contact_table(self._contact.table, self._contact.range)
        if self._beams is not None:
            b = self._beams
            self.engine.set_beams(b.angles, b.scale, b.depth, b.helical)

    # System() already ran init_world on the device
    @property
    def world(self):
        x = self.engine.get_beads()
        V = self.engine.get_links()
        nx = self.engine.get_next()
        return [Particle(x[:, n, :].T.copy(), V[n].copy(), nx[n]) for n in range(self.N)]

    def set_world(self, x, nxt=None):
        self.engine.set_beads(x)
        if nxt is not None:
            self.engine.set_next(nxt)

    def _ensure_engine(self, density_nbins: int, energy_capacity: int):
        cp = self._cp
        if cp.density_nbins == density_nbins and cp.energy_capacity >= energy_capacity:
            return
        x, V, nx = self.engine.get_beads(), self.engine.get_links(), self.engine.get_next()
        cp.density_nbins = density_nbins
        cp.energy_capacity = max(cp.energy_capacity, energy_capacity)
        self.engine.close()
        self.engine = Engine(cp)
        self._attach()
        self.engine.set_raw(x, V, nx)
        self._eser_seen = 0


# --------------------------------------------------------------- updates
class Counter:
    """Rolling acceptance queue (src/updates/helper.jl:6-11)."""

    def __init__(self, range: int = 100_000, adj: int = 10):
        self.queue, self.tries, self.range, self.adj = deque(), 0, range, adj


class Step:
    def __init__(self, size, minstep, maxstep, minacc, maxacc):
        self.size, self.minstep, self.maxstep = size, minstep, maxstep
        self.minacc, self.maxacc = minacc, maxacc


class NumbOfSlices:
    def __init__(self, m, minslices, maxslices, minacc, maxacc):
        self.m, self.minslices, self.maxslices = m, minslices, maxslices
        self.minacc, self.maxacc = minacc, maxacc


def acceptance(q) -> float:
    """sum(q)/length(q) (src/simulation.jl:1); NaN for an empty queue."""
    return sum(q) / len(q) if len(q) else float("nan")


def queue_(c: Counter, acc: bool):
    c.tries += 1
    c.queue.append(1 if acc else 0)
    if len(c.queue) > c.range:
        c.queue.popleft()


def adjust_(var, acc: float):
    if isinstance(var, Step):
        if acc < var.minacc:
            var.size *= 0.9
        elif acc > var.maxacc:
            var.size *= 1.1
        var.size = min(var.maxstep, max(var.minstep, var.size))
    else:
        if acc < var.minacc:
            var.m -= 1
        elif acc > var.maxacc:
            var.m += 1
        var.m = min(var.maxslices, max(var.minslices, var.m))


class _Update:
    counter: Counter
    counter_var: Counter


class ReshapeLinear(_Update):
    def __init__(self, s: System, slices: int, minslices=2, maxslices=None, minacc=0.6, maxacc=0.8,
                 adj=10, range=10_000):
        maxslices = s.M - 2 if maxslices is None else maxslices
        self.counter = Counter()
        self.var = NumbOfSlices(min(slices, maxslices), minslices, maxslices, minacc, maxacc)
        self.counter_var = Counter(adj=adj, range=range)

    def __call__(self, s: System) -> bool:
        """One staging attempt on the device with host-drawn random numbers
        (src/updates/reshape.jl:31-91)."""
        n = int(s.rng.integers(0, s.N))
        j0 = int(s.rng.integers(0, s.M))
        m = min(self.var.maxslices, int(s.rng.integers(2, self.var.m + 1)))
        res = _attempt_with_draws(s, lambda nr, un: s.engine.attempt_staging(n, j0, m, nr, un)[0],
                                  (m - 1) * s.dim)
        acc = res == ACCEPT
        queue_(self.counter_var, acc)
        return acc


class ReshapeSwapLinear(_Update):
    def __init__(self, s: System, slices: int, minslices=2, maxslices=None, minacc=0.6, maxacc=0.8,
                 adj=10, range=10_000):
        maxslices = s.M - 2 if maxslices is None else maxslices
        self.counter = Counter()
        self.var = NumbOfSlices(min(slices, maxslices), minslices, maxslices, minacc, maxacc)
        self.counter_var = Counter(adj=adj, range=range)

    def __call__(self, s: System) -> bool:
        """One permutation attempt (src/updates/reshape.jl:123-283)."""
        if s.N <= 1:
            return False
        j0 = int(s.rng.integers(0, s.M))
        m = min(self.var.maxslices, int(s.rng.integers(2, self.var.m + 1)))
        n1 = int(s.rng.integers(0, s.N))
        up = float(s.rng.random())
        res = _attempt_with_draws(
            s, lambda nr, un: s.engine.attempt_swap(j0, m, n1, up, nr, un)[0], 2 * (m - 1) * s.dim)
        if res == SKIP:
            return False
        acc = res == ACCEPT
        queue_(self.counter_var, acc)
        return acc


class SingleCenterOfMass(_Update):
    def __init__(self, s: System, step: float, minstep=1e-1, maxstep=None, minacc=0.4, maxacc=0.6,
                 adj=10, range=10_000):
        maxstep = s.L / 2 if maxstep is None else maxstep
        self.counter = Counter()
        self.var = Step(step, minstep, maxstep, minacc, maxacc)
        self.counter_var = Counter(adj=adj, range=range)

    def __call__(self, s: System) -> bool:
        """Rigid shift of one non-permuting path (src/updates/com.jl:136-224)."""
        nx = s.engine.get_next()
        singles = [i for i in range(s.N) if nx[i] == i]
        if not singles:
            return False
        n = singles[int(s.rng.integers(0, len(singles)))]
        res = _attempt_with_draws(s, lambda nr, un: s.engine.attempt_com(n, self.var.size, un), 0,
                                  n_uni=s.dim + 1)
        acc = res == ACCEPT
        queue_(self.counter_var, acc)
        return acc


class PolymerCenterOfMass(_Update):
    def __init__(self, s: System, step: float, minstep=1e-1, maxstep=None, minacc=0.4, maxacc=0.6,
                 adj=10, range=10_000):
        maxstep = s.L / 2 if maxstep is None else maxstep
        self.counter = Counter()
        self.var = Step(step, minstep, maxstep, minacc, maxacc)
        self.counter_var = Counter(adj=adj, range=range)

    def __call__(self, s: System) -> bool:
        """Rigid shift of a whole permutation cycle (src/updates/com.jl:31-104)."""
        n = int(s.rng.integers(0, s.N))
        res = _attempt_with_draws(s, lambda nr, un: s.engine.attempt_polymer_com(n, self.var.size, un),
                                  0, n_uni=s.dim + 1)
        acc = res == ACCEPT
        queue_(self.counter_var, acc)
        return acc


def _attempt_with_draws(s: System, call, n_norm: int, n_uni: int = 1):
    """Run one attempt with host-drawn normals/uniforms, growing the arrays when
    the hard-core retries need more."""
    scale = 1
    while True:
        nr = s.rng.standard_normal(max(n_norm * scale, 0))
        un = s.rng.random(n_uni * scale)
        try:
            return call(nr, un)
        except PimcError as e:
            if "draws" not in str(e) or scale > 1 << 20:
                raise
            scale *= 4


# --------------------------------------------------------------- measurements
class Density:
    """Cartesian density histogram (src/measurement.jl:31-55)."""

    def __init__(self, s: System, nbins: int = 500):
        self.nbins = nbins
        self.bin = (2 * s.L) / nbins
        self.dens = np.zeros((nbins,) * s.dim)
        self.ndata = 0

    def __call__(self, s: System):
        s._ensure_engine(self.nbins, s._cp.energy_capacity)
        s.engine.reset_measurements()
        s.engine.measure()
        self._pull(s)

    def _pull(self, s: System):
        hist, nd = s.engine.density()
        h = hist.reshape((self.nbins,) * s.dim, order="F")
        self.dens = self.dens + h
        self.ndata += nd


class Energy:
    """Thermodynamic and virial energy series keyed by N (src/measurement.jl:78-122)."""

    def __init__(self, s: System, n: int = 20_000):
        self.capacity = n
        self.energy = {0: []}
        self.energy_virial = {0: []}

    def _add(self, s: System, rows):
        phys = s.semantics == SEM_PHYSICAL
        e = rows[:, 0] + (rows[:, 2] if phys else 0.0)
        ev = rows[:, 1] + (rows[:, 3] if phys else 0.0)
        self.energy.setdefault(s.N, []).extend(e.tolist())
        self.energy_virial.setdefault(s.N, []).extend(ev.tolist())
        if len(self.energy[s.N]) > self.capacity:
            raise PimcError("Energy storage is full (the reference errors here too)")


class RadialDistribution:
    """Pair radial distribution g(r) (the TODO of src/measurement.jl:125):
    every measurement bins, at every slice, each unordered pair's
    minimum-image distance into nbins bins over [0, rmax)."""

    def __init__(self, s: System, nbins: int = 100, rmax: float | None = None):
        self.nbins = int(nbins)
        self.rmax = float(s.L if rmax is None else rmax)
        self.bin = self.rmax / self.nbins
        self.hist = np.zeros(self.nbins)
        self.ndata = 0       # measurements
        self._dim, self._L, self._M, self._N = s.dim, s.L, s.M, s.N

    def _pull(self, s: System):
        h, nm = s.engine.radial()
        self.hist = self.hist + h
        self.ndata += nm

    def r(self):
        return (np.arange(self.nbins) + 0.5) * self.bin

    def g(self):
        """counts over the ideal-gas expectation: pairs per slice
        N(N-1)/2 times the shell's share of the box (2L)^dim"""
        e = np.arange(self.nbins + 1) * self.bin
        shell = np.pi * (e[1:] ** 2 - e[:-1] ** 2) if self._dim == 2 else 2.0 * (e[1:] - e[:-1])
        pairs = self.ndata * self._M * self._N * (self._N - 1) / 2
        with np.errstate(invalid="ignore", divide="ignore"):
            return self.hist / (pairs * shell / (2 * self._L) ** self._dim)


class Superfluid:
    """Superfluid-fraction estimators (the TODO of src/measurement.jl:126):
    the winding estimator rho_s/rho = <W^2> / (2 dim lambda beta N) for a
    periodic box, and the area estimator rho_s/rho = 2 <A_z^2> / (lambda beta
    <sum r^2 / M>) about the trap centre (Sindzingre, Klein and Ceperley, PRL
    63, 1601 (1989)), from per-measurement series keyed by N."""

    def __init__(self, s: System, n: int = 20_000):
        self.capacity = n
        self.W2 = {0: []}
        self.area = {0: []}
        self.I = {0: []}
        self._lam, self._beta, self._dim = s.λ, s.β, s.dim

    def _add(self, s: System, rows):
        self.W2.setdefault(s.N, []).extend(rows[:, 4].tolist())
        self.area.setdefault(s.N, []).extend(rows[:, 5].tolist())
        self.I.setdefault(s.N, []).extend(rows[:, 6].tolist())
        if len(self.W2[s.N]) > self.capacity:
            raise PimcError("Superfluid storage is full")

    def winding_fraction(self, N: int) -> float:
        return float(np.mean(self.W2[N])) / (2 * self._dim * self._lam * self._beta * N)

    def area_fraction(self, N: int) -> float:
        a = np.asarray(self.area[N])
        return 2.0 * float(np.mean(a * a)) / (self._lam * self._beta * float(np.mean(self.I[N])))


# --------------------------------------------------------------- files
def save_paths(s: System, path: str = "paths.csv"):
    """save_paths (examples/tools/savetools.jl:30-34): the paths table
    written from the device state"""
    s.engine.write_paths_csv(path)


def density_filename(s: System, g, name, V) -> str:
    """the reference's save_density file name,
    density<name>M<M>beta<beta>N<N>g<g>V<V>.csv (savetools.jl:55)"""
    fmt = lambda v: julia_float(v) if isinstance(v, float) else str(v)
    return f"density{name}M{s.M}beta{fmt(s.β)}N{s.N}g{fmt(g)}V{fmt(V)}.csv"


def save_density(s: System, d: Density, g, name, V, directory: str = "."):
    """save_density (savetools.jl:37-65): the normalised histogram with its
    position column, under the reference's file name; returns the path"""
    import os
    path = os.path.join(directory, density_filename(s, g, name, V))
    write_density_csv(path, s.dim, d.nbins, s.L, d.dens, d.ndata)
    return path


def save_checkpoint(s: System, path: str):
    """every chain's state (beads, links, permutation, counters, adaptive
    variables, generator position, series) in a checksummed file"""
    s.engine.save_checkpoint(path)


def load_checkpoint(s: System, path: str):
    s.engine.load_checkpoint(path)


# --------------------------------------------------------------- driver
def _mix_for(s: System, n: int, updates):
    """Map run!(s, n, updates) onto sweeps of the engine (one staging phase per
    sweep; swaps and centre-of-mass moves in the proportions 1/every)."""
    w = {}
    objs = {}
    for every, u in updates:
        key = type(u).__name__
        w[key] = w.get(key, 0.0) + 1.0 / every
        objs[key] = u
    wsum = sum(w.values())
    N, M = s.N, s.M
    st = objs.get("ReshapeLinear")
    sw = objs.get("ReshapeSwapLinear")
    cm = objs.get("SingleCenterOfMass")
    pc = objs.get("PolymerCenterOfMass")
    ell = st.var.m if st else 2
    k = math.ceil(M / ell)
    if st:
        per_sweep = N * k * wsum / w["ReshapeLinear"]
    else:
        per_sweep = N * wsum / max(w.values())
    sweeps = max(1, round(n / per_sweep))
    unit = per_sweep / wsum

    def frac(key):
        return w.get(key, 0.0) * unit

    mix = Mix(
        staging_phases=1 if st else 0,
        stage_slices=st.var.m if st else 2, stage_min=st.var.minslices if st else 2,
        stage_max=min(st.var.maxslices, 64) if st else 2,
        stage_minacc=st.var.minacc if st else 0.6, stage_maxacc=st.var.maxacc if st else 0.8,
        swaps_per_sweep=int(round(frac("ReshapeSwapLinear"))) if (sw and N > 1) else 0,
        swap_slices=sw.var.m if sw else 2, swap_min=sw.var.minslices if sw else 2,
        swap_max=min(sw.var.maxslices, 64) if sw else 2,
        swap_minacc=sw.var.minacc if sw else 0.6, swap_maxacc=sw.var.maxacc if sw else 0.8,
        com_phases=max(1, int(round(frac("SingleCenterOfMass") / N))) if cm else 0,
        com_step=cm.var.size if cm else 1.0, com_minstep=cm.var.minstep if cm else 0.1,
        com_maxstep=cm.var.maxstep if cm else 1.0, com_minacc=cm.var.minacc if cm else 0.4,
        com_maxacc=cm.var.maxacc if cm else 0.6,
        polymer_com_phases=max(1, int(round(frac("PolymerCenterOfMass") / N))) if pc else 0,
        pcom_step=pc.var.size if pc else 1.0, pcom_minstep=pc.var.minstep if pc else 0.1,
        pcom_maxstep=pc.var.maxstep if pc else 1.0, pcom_minacc=pc.var.minacc if pc else 0.4,
        pcom_maxacc=pc.var.maxacc if pc else 0.6,
        adapt=1, measure_every=0)
    return mix, sweeps, per_sweep, objs


def run(s: System, n: int, updates, Zmeasurements=()):
    """run!(s, n, updates; Zmeasurements) on the device: n move attempts are
    mapped to sweeps (per sweep N*ceil(M/l) staging windows, swaps and CoM
    moves in the 1/every proportions); measurements every
    length_measurement_cycle attempts become one every ceil(Ncycle/per_sweep)
    sweeps."""
    s.ctr = 10_000 if not Zmeasurements else 1_000
    mix, sweeps, per_sweep, objs = _mix_for(s, n, updates)
    dens = [z for z in Zmeasurements if isinstance(z, Density)]
    ens = [z for z in Zmeasurements if isinstance(z, (Energy, Superfluid))]
    rdfs = [z for z in Zmeasurements if isinstance(z, RadialDistribution)]
    if Zmeasurements:
        mix.measure_every = max(1, round(s.Ncycle / per_sweep))
        nb = dens[0].nbins if dens else 0
        cap = s._eser_seen + sweeps // mix.measure_every + 1 if ens else 0
        s._ensure_engine(nb, cap)
        s.engine.reset_measurements()
        s._eser_seen = 0
        s.engine.set_radial(rdfs[0].nbins if rdfs else 0, rdfs[0].rmax if rdfs else 0.0)
    before = s.engine.stats()
    s.engine.set_mix(mix)
    s.engine.run(sweeps)
    after = s.engine.stats()
    # mirror the engine's counters and adaptive variables into the updates
    kinds = {"ReshapeLinear": 0, "ReshapeSwapLinear": 1, "SingleCenterOfMass": 2,
             "PolymerCenterOfMass": 3}
    for key, u in objs.items():
        q = kinds[key]
        att = after.attempts[q] - before.attempts[q]
        acc = after.accepts[q] - before.accepts[q]
        u.counter.tries += att
        u.counter_var.tries += att
        u.counter_var.queue.extend([1] * acc + [0] * (att - acc))
        while len(u.counter_var.queue) > u.counter_var.range:
            u.counter_var.queue.popleft()
        if q == 0:
            u.var.m = after.stage_slices
        elif q == 1:
            u.var.m = after.swap_slices
        elif q == 2:
            u.var.size = after.com_step
        else:
            u.var.size = after.pcom_step
    if Zmeasurements:
        nmeas = after.measurements - before.measurements
        s.N_MC[s.N] = s.N_MC.get(s.N, 0) + nmeas
        rows = s.engine.observables()
        for e in ens:
            e._add(s, rows[s._eser_seen:])
        s._eser_seen = len(rows)
        for d in dens:
            d._pull(s)
        for r in rdfs:
            r._pull(s)
    return None


def apply(s: System, f):
    """apply!(s, f) (src/simulation.jl:19-27): one attempt, queue, adjust."""
    if isinstance(f, (list, tuple)):
        for g in f:
            g(s)
        return None
    acc = f(s)
    queue_(f.counter, acc)
    if f.counter_var.tries % f.counter_var.adj == 0:
        adjust_(f.var, acceptance(f.counter_var.queue))
    return None


__all__ = ["System", "Particle", "Harmonic", "SquareLattice", "PotentialSum", "Zero",
           "GaussianPair", "ReshapeLinear", "ReshapeSwapLinear", "SingleCenterOfMass",
           "PolymerCenterOfMass", "Counter", "Step", "NumbOfSlices", "acceptance", "run", "apply",
           "Density", "Energy", "SEM_REFERENCE", "SEM_PHYSICAL"]
