"""The adjoint at the differentiated configuration (C5) and batched.

C5: 2D square optical lattice V0 (sin^2(pi x / a) + sin^2(pi y / a)), a = 1,
V0 = 4, plus the trap omega = 0.1 and the Gaussian pair g = 1, sigma = 0.3;
N = 1024, beta = 4, M = 64, box [-16, 16)^2, neighbour range r_a = 0.9
(cell 0.914), physical rules.  The adjoint returns dS/dr for every bead and
dS/d(V0, omega, g) of the potential action S = -sum lnV - sum lnU; both are
checked against central differences with h = 1e-5 within 1e-6 relative.

A bead's derivative is the derivative of the action terms that contain the
bead (the rest of S does not move with it).  Those terms are restated here
in numpy from the reference's formulas (src/propagator.jl:26-28 lnV,
src/system.jl:26-28 lnU with the Gaussian propagator, the neighbour set of
src/nearest_neighbours.jl:131-154: partners within 2L/nbins of a link's
first bead), so the difference quotient is free of the rounding of a
65536-term total.  The parameter derivatives difference the engine's own
total action (pimc_eval_action), whose size keeps the quotient well within
the tolerance.

pimc_batch_adjoint must give every chain of a batch what pimc_adjoint gives
it alone.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H = 1e-5
RTOL = 1e-6


def c5_params(**kw):
    from pimc.engine import ChainParams
    base = dict(dim=2, N=1024, M=64, L=16.0, T=0.25, lam=0.5, harmonic_omega=0.1, lattice_V0=4.0,
                lattice_a=1.0, interactions=True, pair_g=1.0, pair_sigma=0.3, r_a=0.9,
                semantics=1, seed=20261203)
    base.update(kw)
    return ChainParams(**base)


def _mi(d, L):
    return d - 2 * L * np.round(d / (2 * L))


class LocalAction:
    """the action terms containing bead (n, j) of a chain, as a function of
    that bead's position"""

    def __init__(self, p, x, nxt):
        self.p, self.x, self.nxt = p, x, nxt
        self.inv = np.argsort(nxt)
        self.tau = 1.0 / (p.T * p.M)
        nb = int(np.floor(2 * p.L / p.r_a))
        self.rc = 2 * p.L / nb
        self.c = 1.0 / (2 * p.pair_sigma ** 2)

    def vext(self, r, V0=None, om=None):
        p = self.p
        V0 = p.lattice_V0 if V0 is None else V0
        om = p.harmonic_omega if om is None else om
        k = np.pi / p.lattice_a
        return 0.5 * om ** 2 * (r[0] ** 2 + r[1] ** 2) + V0 * (np.sin(k * r[0]) ** 2 + np.sin(k * r[1]) ** 2)

    def vpair(self, r2):
        return self.p.pair_g * np.exp(-r2 * self.c)

    def __call__(self, n, j, r):
        p, x, L, M = self.p, self.x, self.p.L, self.p.M
        s = self.tau * self.vext(r)  # both links at the bead: 2 * tau/2 * V(r)
        # links starting at slice j: pairs (n, b) with |r - x_b(j)| <= rc
        d = _mi(r[:, None] - x[:, :, j], L)
        d2 = (d ** 2).sum(axis=0)
        mask = d2 <= self.rc ** 2
        mask[n] = False
        s += 0.5 * self.tau * self.vpair(d2[mask]).sum()
        # links ending at slice j: the predecessor bead p0 = (n or inv[n], j-1)
        # and partners b0 within rc of it at j-1; their next beads at j
        jp = j - 1 if j > 0 else M - 1
        p0 = n if j > 0 else self.inv[n]
        d0 = _mi(x[:, p0, jp][:, None] - x[:, :, jp], L)
        m0 = (d0 ** 2).sum(axis=0) <= self.rc ** 2
        m0[p0] = False
        b0 = np.nonzero(m0)[0]
        bn = b0 if j > 0 else self.nxt[b0]
        e = _mi(r[:, None] - x[:, bn, j], L)
        s += 0.5 * self.tau * self.vpair((e ** 2).sum(axis=0)).sum()
        return s


def _c5_engine():
    from pimc.engine import Engine, Mix
    e = Engine(c5_params())
    e.set_mix(Mix(stage_slices=16, stage_max=16, stage_minacc=0.0, stage_maxacc=1.0,
                  swaps_per_sweep=1024, swap_slices=16, swap_max=16, swap_minacc=0.0,
                  swap_maxacc=1.0, com_step=1.0, com_maxstep=8.0, measure_every=0))
    e.run(12)  # permuted cycles, beads off their initial loops
    return e


def test_c5_adjoint_matches_central_differences():
    e = _c5_engine()
    p = e.params[0]
    x, nxt = e.get_beads(), e.get_next()
    g, th, ex = e.adjoint()
    loc = LocalAction(p, x, nxt)
    rng = np.random.default_rng(5)
    beads = [(int(rng.integers(p.N)), int(rng.integers(p.M))) for _ in range(24)]
    beads += [(int(rng.integers(p.N)), 0) for _ in range(4)] + [(int(rng.integers(p.N)), p.M - 1)
                                                                 for _ in range(4)]
    checked = 0
    for n, j in beads:
        for d in range(2):
            rp, rm = x[:, n, j].copy(), x[:, n, j].copy()
            rp[d] += H
            rm[d] -= H
            fd = (loc(n, j, rp) - loc(n, j, rm)) / (2 * H)
            assert abs(g[d, n, j] - fd) <= RTOL * max(abs(fd), 1e-3), (d, n, j, g[d, n, j], fd)
            checked += 1
    assert checked == 64
    # the parameter derivatives from the engine's total potential action
    base = (p.lattice_V0, p.harmonic_omega, p.pair_g)

    def s_pot():
        a = e.eval_action()
        return -(a[1] + a[2])

    for q in range(3):
        vp, vm = list(base), list(base)
        vp[q] += H
        vm[q] -= H
        e.set_potential(*vp)
        sp = s_pot()
        e.set_potential(*vm)
        sm = s_pot()
        fd = (sp - sm) / (2 * H)
        assert abs(th[q] - fd) <= RTOL * abs(fd), (q, th[q], fd)
    e.set_potential(*base)
    S = s_pot()
    assert abs((ex[0] + ex[1]) - S) <= 1e-10 * abs(S)
    e.close()


def test_batch_adjoint_equals_per_chain_adjoint():
    from pimc.engine import Engine, Mix
    rng = np.random.default_rng(12)
    ps = []
    for i in range(20):
        ps.append(c5_params(N=int(rng.integers(4, 200)), M=int(rng.choice([8, 16, 32, 64])),
                            L=6.0, T=float(1 / rng.uniform(0.5, 4)), harmonic_omega=float(rng.uniform(0, 1)),
                            lattice_V0=float(rng.choice([0.0, 2.0])), pair_g=float(rng.uniform(0, 2)),
                            interactions=bool(i % 4 != 3), r_a=1.0, semantics=int(i % 2), seed=700 + i))
    e = Engine(ps)
    for i, q in enumerate(ps):
        e.set_mix(Mix(stage_slices=min(8, q.M // 2), stage_max=min(8, q.M // 2), swaps_per_sweep=q.N,
                      swap_slices=min(8, q.M // 2), swap_max=min(8, q.M // 2), com_maxstep=2.0),
                  chain=i)
    e.run_batched(4)
    for rep in range(2):  # the pool is made on the first call and reused
        gb, thb, exb = e.batch_adjoint(want_beads=True)
        for c in range(len(ps)):
            g, th, ex = e.adjoint(c)
            # the batched kernel adds each pair's force once, in another
            # order: components that cancel to near zero keep an absolute
            # error of order the rounding of the terms they came from
            np.testing.assert_allclose(gb[c], g, rtol=1e-12, atol=1e-12 * np.abs(g).max())
            np.testing.assert_allclose(thb[c], th, rtol=1e-12, atol=1e-300)
            np.testing.assert_allclose(exb[c], ex, rtol=1e-12, atol=1e-12 * np.abs(ex).max())
    assert e.last_run_launches() == 4 and e.last_run_ms() > 0
    _, th2, _ = e.batch_adjoint(want_beads=False)
    np.testing.assert_array_equal(th2, thb)
    e.close()
