"""The optical-lattice potentials of examples/tools/potentialtools.jl as an
engine potential (pimc_set_beams).

- Action values, staging weights, injected-draw moves and the energy
  estimators (whose virial term uses the potential's gradient) agree with
  the oracle given the same beams, in both semantics and helical or not.
- The adjoint's per-bead dS/dr with the lattice matches central differences.
- The API's generate_V(scale, depth, :l25) runs through System and run!.
"""
import numpy as np
import pytest

from common import random_config

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def lattice_pair(oracle_mod, sem, helical, seed=3, interactions=False):
    import pimc
    from pimc.engine import ChainParams, Engine
    ang = pimc.lattice_angles("l25")
    scale, depth = 0.6, -3.0
    ek = dict(dim=2, N=10, M=16, L=4.0, T=1.0, lam=0.5, harmonic_omega=0.5, semantics=sem,
              energy_capacity=4)
    ok = dict(dim=2, N=10, M=16, L=4.0, T=1.0, lam=0.5, hcoef=0.125, semantics=sem,
              beams=(ang, scale, depth, helical))
    if interactions:
        ek.update(interactions=True, pair_g=1.0, pair_sigma=0.5, r_a=1.0)
        ok.update(interactions=True, pair_g=1.0, pair_sigma=0.5, r_a=1.0)
    e = Engine(ChainParams(**ek))
    e.set_beams(ang, scale, depth, helical)
    o = oracle_mod.Oracle(oracle_mod.make_params(**ok))
    rng = np.random.default_rng(seed)
    x, nxt = random_config(rng, 2, 10, 16, 4.0, 1.2, True)
    e.set_beads(x)
    e.set_next(nxt)
    o.set_state(x, nxt)
    return e, o, rng


@pytest.mark.parametrize("sem", [0, 1])
@pytest.mark.parametrize("helical", [False, True])
def test_lattice_action_and_estimators(sem, helical, oracle_mod, engine_lib):
    e, o, _ = lattice_pair(oracle_mod, sem, helical, interactions=sem == 1)
    ge, go = e.eval_action(), o.eval_action()
    assert np.all(np.abs(ge - go) <= RTOL * np.maximum(np.abs(go), 1.0)), (ge, go)
    x, V, _ = o.get_state()
    np.testing.assert_allclose(e.get_links(), V, rtol=1e-12, atol=1e-12)
    e.measure()
    got, want = e.energies()[0], o.energy()
    assert np.all(np.abs(got - want) <= 1e-11 * np.maximum(np.abs(want), 1.0)), (got, want)


@pytest.mark.parametrize("sem", [0, 1])
def test_lattice_moves(sem, oracle_mod, engine_lib):
    e, o, rng = lattice_pair(oracle_mod, sem, False, seed=7, interactions=True)
    N, M = 10, 16
    outcomes = set()
    for it in range(200):
        if it % 3:
            n, j0, m = int(rng.integers(N)), int(rng.integers(M)), int(rng.integers(2, M - 1))
            nr, u = rng.standard_normal((m - 1) * 2), rng.random(1)
            re, pe = e.attempt_staging(n, j0, m, nr, u)
            ro, po = o.staging(n, j0, m, oracle_mod.Draw(nr, u))
            np.testing.assert_allclose(pe, po, rtol=0, atol=1e-12)
        else:
            nx = o.get_state()[2]
            singles = [i for i in range(N) if nx[i] == i]
            if not singles:
                continue
            n = int(rng.choice(singles))
            u = rng.random(3)
            re = e.attempt_com(n, 0.5, u)
            ro = o.com(n, 0.5, oracle_mod.Draw([], u))
        assert re == ro, (it, re, ro)
        outcomes.add(re)
    assert {0, 1} <= outcomes
    x, V, nx = o.get_state()
    np.testing.assert_allclose(e.get_beads(), x, rtol=0, atol=1e-10)
    np.testing.assert_allclose(e.get_links(), V, rtol=1e-10, atol=1e-10)


def test_lattice_gradient_in_the_adjoint(engine_lib):
    """per-bead dS/dr with the optical lattice (+ trap + pair) against central
    differences of the action (h = 1e-5, 1e-6 relative)"""
    import pimc
    from pimc.engine import ChainParams, Engine
    rng = np.random.default_rng(12)
    N, M = 5, 8
    e = Engine(ChainParams(dim=2, N=N, M=M, L=4.0, T=0.25, lam=0.5, harmonic_omega=0.7,
                           interactions=True, pair_g=1.0, pair_sigma=0.6, r_a=1.0, semantics=1))
    e.set_beams(pimc.lattice_angles("l65"), 0.8, -2.5, True)
    x = rng.normal(scale=0.8, size=(2, N, M))
    e.set_beads(x)
    e.set_next(rng.permutation(N).astype(np.int32))
    g, _, ex = e.adjoint()

    def action():
        k, v, u, c = e.eval_action()
        return -(v + u)

    h = 1e-5
    for (d, n, j) in [(0, 0, 0), (1, 2, 5), (0, 3, 7), (1, 4, 1)]:
        xp, xm = x.copy(), x.copy()
        xp[d, n, j] += h
        xm[d, n, j] -= h
        e.set_beads(xp)
        sp = action()
        e.set_beads(xm)
        sm = action()
        fd = (sp - sm) / (2 * h)
        assert abs(g[d, n, j] - fd) <= 1e-6 * max(abs(fd), 1e-3), (d, n, j, g[d, n, j], fd)
    e.set_beads(x)
    assert abs((ex[0] + ex[1]) - action()) <= 1e-10 * max(1.0, abs(action()))


def test_generate_V_through_the_api(engine_lib):
    import pimc
    V = pimc.generate_V(0.5, 2.0, "l25") + pimc.Harmonic(0.3)
    s = pimc.System(V, M=16, N=6, L=6.0, T=1.0, λ=0.5, length_measurement_cycle=1)
    r = np.array([0.3, -0.8])
    x = s.engine.get_beads()
    x[:, 0, 0] = r
    s.set_world(x)
    # the cached link of bead 0 is -tau/2 (V(r0) + V(r1)) with the host's V
    r1 = x[:, 0, 1]
    want = -0.5 * s.τ * (V(r) + V(r1))
    assert abs(s.engine.get_links()[0, 0] - want) <= 1e-12 * max(1.0, abs(want))
    ups = [(1, pimc.ReshapeLinear(s, 8)), (1, pimc.SingleCenterOfMass(s, 1.0))]
    E = pimc.Energy(s, 10_000)
    pimc.run(s, 3000, ups, Zmeasurements=[E])
    assert len(E.energy[6]) > 0 and np.isfinite(E.energy[6]).all()
