"""The tabulated contact-interaction propagator (build_prop_int,
src/propagator.jl:35-89, with lnU of src/system.jl:26-28) on the device.

- The device table agrees with independent adaptive-quadrature values of
  the reference's integrals (tests/golden/contact_table.json) within 1e-10
  relative, above an absolute floor of 1e-13 of the table's largest entry.
- Pair link actions, staging weights and every move with injected draws
  agree with the CPU oracle given the same table (1e-12 relative; the same
  decisions), in both acceptance semantics.
- Sweeps stay finite, the batched and the plain paths agree bit for bit,
  and the FP32 log-space Metropolis test decides as the FP64 one does.
"""
import json
import os

import numpy as np
import pytest

from common import HERE, random_config

pytestmark = pytest.mark.gpu

RTOL = 1e-12
G0, RANGE = 1.16, 5.0


def contact_params(sem, N=16, M=16, L=3.0, mu=0.3):
    eng = dict(dim=2, N=N, M=M, L=L, T=1.0, lam=0.5, mu=mu, harmonic_omega=1.0,
               interactions=True, pair_g=0.0, pair_sigma=1.0, r_a=1.0, semantics=sem)
    orc = dict(dim=2, N=N, M=M, L=L, T=1.0, lam=0.5, mu=mu, hcoef=0.5, interactions=True,
               r_a=1.0, semantics=sem)
    return eng, orc


def make_pair(sem, oracle_mod, seed=1, spread=1.0, perm=True):
    from pimc.engine import ChainParams, Engine
    ek, ok = contact_params(sem)
    e = Engine(ChainParams(**ek))
    e.set_contact_propagator(G0, RANGE)
    tab, rng_ = e.contact_table()
    assert tab.shape == (600, 600) and rng_ == RANGE
    o = oracle_mod.Oracle(oracle_mod.make_params(contact_table=tab, contact_range=rng_, **ok))
    rng = np.random.default_rng(seed)
    x, nxt = random_config(rng, ek["dim"], ek["N"], ek["M"], ek["L"], spread, perm)
    e.set_beads(x)
    e.set_next(nxt)
    o.set_state(x, nxt)
    return e, o, rng, ek


def assert_states_equal(e, o, tol=1e-11):
    x, V, nx = o.get_state()
    np.testing.assert_array_equal(e.get_next(), nx)
    np.testing.assert_allclose(e.get_beads(), x, rtol=0, atol=tol)
    np.testing.assert_allclose(e.get_links(), V, rtol=tol, atol=tol)


def test_contact_table_matches_golden(engine_lib):
    from pimc.engine import contact_table
    gold = json.load(open(os.path.join(HERE, "golden", "contact_table.json")))
    for c in gold["configs"]:
        tab = contact_table(c["g0"], c["tau"], c["range"], c["n"])
        assert np.isfinite(tab).all()
        np.testing.assert_array_equal(tab, tab.T)  # T(r1, r2) = T(r2, r1)
        big = max(abs(v) for _, _, v in c["entries"])
        for i1, i2, v in c["entries"]:
            err = abs(tab[i1, i2] - v)
            assert err <= 1e-10 * abs(v) + 1e-13 * big, (c["g0"], i1, i2, tab[i1, i2], v)


def test_contact_table_rejects_bad_arguments(engine_lib):
    from pimc import PimcError
    from pimc.engine import ChainParams, Engine, contact_table
    with pytest.raises(PimcError):
        contact_table(0.0, 0.01, 6.0, 600)
    with pytest.raises(PimcError):
        contact_table(1.0, -0.01, 6.0, 600)
    with pytest.raises(PimcError):
        contact_table(1.0, 0.01, 6.0, 1)
    e = Engine(ChainParams(dim=2, N=4, M=8, L=3.0))  # no interactions
    with pytest.raises(PimcError):
        e.set_contact_propagator(G0, RANGE)
    ek, _ = contact_params(0)
    e = Engine(ChainParams(**ek))
    assert e.contact_table() == (None, 0.0)
    with pytest.raises(PimcError):
        e.set_contact_table(np.full((4, 4), np.nan), RANGE)
    e.set_contact_propagator(G0, RANGE, n=64)
    with pytest.raises(PimcError):  # the adjoint covers the Gaussian pair only
        e.adjoint()
    e.clear_contact()
    assert e.contact_table() == (None, 0.0)


@pytest.mark.parametrize("sem", [0, 1])
def test_contact_eval_action(sem, oracle_mod, engine_lib):
    for seed, spread in ((3, 1.0), (4, 0.4)):
        e, o, _, _ = make_pair(sem, oracle_mod, seed=seed, spread=spread)
        ge, go = e.eval_action(), o.eval_action()
        assert go[2] != 0.0
        scale = np.maximum(np.abs(go), 1.0)
        assert np.all(np.abs(ge - go) <= RTOL * scale), (ge, go)


def test_contact_both_branches_reached(oracle_mod, engine_lib):
    """a caller-given table (the device table scaled by 6) makes close pairs'
    prop_int negative (lnU = -mu) while farther pairs keep log(prop_int)"""
    from pimc.engine import ChainParams, Engine
    ek, ok = contact_params(0, N=2, M=4)
    e = Engine(ChainParams(**ek))
    e.set_contact_propagator(G0, RANGE)
    tab, rng_ = e.contact_table()
    tab = 6.0 * tab
    e.set_contact_table(tab, rng_)
    np.testing.assert_array_equal(e.contact_table()[0], tab)
    o = oracle_mod.Oracle(oracle_mod.make_params(contact_table=tab, contact_range=rng_, **ok))
    vals = []
    for sep in (0.001, 0.01, 0.05, 0.2, 0.5, 0.9):
        x = np.zeros((2, 2, 4))
        x[0, 1, :] = sep
        x[1, 1, :] = 0.3 * sep
        e.set_beads(x)
        o.set_state(x)
        ge, go = e.eval_action(), o.eval_action()
        assert abs(ge[2] - go[2]) <= RTOL * max(1.0, abs(go[2])), (sep, ge, go)
        vals.append(go[2] / 4)  # four links, one pair each
    assert any(abs(v + ek["mu"]) < 1e-15 for v in vals), vals
    assert any(abs(v + ek["mu"]) > 1e-6 for v in vals), vals


@pytest.mark.parametrize("sem", [0, 1])
def test_contact_staging_weights(sem, oracle_mod, engine_lib):
    e, o, rng, ek = make_pair(sem, oracle_mod, seed=5)
    for _ in range(40):
        n = int(rng.integers(ek["N"]))
        j0 = int(rng.integers(ek["M"]))
        m = int(rng.integers(2, 12))
        rp = rng.normal(size=(m + 1, ek["dim"])).clip(-ek["L"] * 0.99, ek["L"] * 0.99)
        ge = e.staging_weights(n, j0, m, rp.ravel())
        go = o.staging_weights(n, j0, m, rp.ravel())
        for a, b in zip(ge, go):
            assert abs(a - b) <= RTOL * max(1.0, abs(b)), (ge, go)


@pytest.mark.parametrize("sem", [0, 1])
def test_contact_moves(sem, oracle_mod, engine_lib):
    """staging, swap and centre-of-mass moves with injected draws: the same
    proposals and decisions, interleaved over a long sequence"""
    from pimc.engine import HARDCORE, SKIP
    e, o, rng, ek = make_pair(sem, oracle_mod, seed=13, spread=0.6)
    N, M, dim = ek["N"], ek["M"], ek["dim"]
    seen = {0: set(), 1: set(), 2: set()}
    for it in range(360):
        kind = int(rng.choice(3, p=[0.5, 0.35, 0.15]))
        if kind == 0:
            n, j0, m = int(rng.integers(N)), int(rng.integers(M)), int(rng.integers(2, M - 1))
            nr, u = rng.standard_normal((m - 1) * dim), rng.random(1)
            re, pe = e.attempt_staging(n, j0, m, nr, u)
            ro, po = o.staging(n, j0, m, oracle_mod.Draw(nr, u))
            np.testing.assert_allclose(pe, po, rtol=0, atol=1e-12)
        elif kind == 1:
            j0, m, n1 = int(rng.integers(M)), int(rng.integers(2, M - 1)), int(rng.integers(N))
            up = float(rng.random())
            nr, u = rng.standard_normal(2 * (m - 1) * dim), rng.random(1)
            re, n2e, pe = e.attempt_swap(j0, m, n1, up, nr, u)
            ro, n2o, po = o.swap(j0, m, n1, up, oracle_mod.Draw(nr, u))
            assert n2e == n2o
            if re not in (SKIP, HARDCORE):
                np.testing.assert_allclose(pe, po, rtol=0, atol=1e-12)
        else:
            nx = o.get_state()[2]
            singles = [i for i in range(N) if nx[i] == i]
            if not singles:
                continue
            n = int(rng.choice(singles))
            u = rng.random(3)
            re = e.attempt_com(n, 0.7, u)
            ro = o.com(n, 0.7, oracle_mod.Draw([], u))
        assert re == ro, (it, kind, re, ro)
        seen[kind].add(re)
    assert_states_equal(e, o, tol=1e-10)
    assert {0, 1} <= seen[0] and 1 in seen[1]
    ge, go = e.eval_action(), o.eval_action()
    assert np.all(np.abs(ge - go) <= 1e-10 * np.maximum(np.abs(go), 1.0))


@pytest.mark.parametrize("sem", [0, 1])
def test_contact_sweeps(sem, engine_lib):
    """batched sweeps of contact chains: finite, both outcomes, identical to
    one launch per chain and to exact FP64 decisions"""
    from pimc.engine import ChainParams, Engine, Mix, OPT_EXACT_DECISIONS
    ps = [ChainParams(dim=2, N=N, M=M, L=4.0, T=1.0, lam=0.5, mu=0.2, harmonic_omega=1.0,
                      interactions=True, r_a=1.0, semantics=sem, seed=70 + i, energy_capacity=8)
          for i, (N, M) in enumerate([(12, 16), (24, 32), (40, 16), (8, 64)])]
    engines = [Engine(ps) for _ in range(3)]
    for k, e in enumerate(engines):
        e.set_contact_propagator(G0, 6.0)
        for i, p in enumerate(ps):
            e.set_mix(Mix(stage_slices=8, stage_min=2, stage_max=8, stage_minacc=0.0,
                          stage_maxacc=1.0, swaps_per_sweep=p.N, swap_slices=8, swap_min=2,
                          swap_max=8, swap_minacc=0.0, swap_maxacc=1.0, com_phases=1,
                          com_step=1.0, com_minstep=0.1, com_maxstep=2.0, adapt=1,
                          measure_every=2), chain=i)
    engines[2].set_option(OPT_EXACT_DECISIONS, 1)
    engines[0].run_batched(10)
    engines[1].run_plain(10)
    engines[2].run_batched(10)
    for c in range(len(ps)):
        b = engines[0].get_beads(c)
        assert np.isfinite(b).all() and np.abs(b).max() <= 4.0
        for other in engines[1:]:
            np.testing.assert_array_equal(other.get_beads(c), b)
            np.testing.assert_array_equal(other.get_next(c), engines[0].get_next(c))
    st = engines[0].total_stats()
    assert all(0 < st.accepts[k] < st.attempts[k] for k in range(3)), st
    # pair energies are not defined for the table: the estimator's pair columns read 0
    assert np.all(engines[0].energies(0)[:, 2:] == 0.0)


def test_contact_system_api(engine_lib):
    """System(...; interactions=true, propint=build_prop_int(...)) without r_a:
    the neighbour range comes from determine_nnrange (src/system.jl:10-34)"""
    import pimc
    M, T, L = 16, 1.0, 3.0
    prop = pimc.build_prop_int(float(np.ceil(np.sqrt(2) * L)), G0, 1.0 / (T * M))
    s = pimc.System(pimc.Harmonic(1.0), M=M, N=6, L=L, T=T, λ=0.5, interactions=True,
                    propint=prop)
    assert 0.0 < s.rₐ < L
    r = s.rₐ
    assert abs(prop([r], [r], 1.0 / (T * M)) - 0.999) < 1e-9
    tab, rng_ = s.engine.contact_table()
    np.testing.assert_array_equal(tab, prop.table)
    ups = [(1, pimc.ReshapeLinear(s, 6)), (1, pimc.ReshapeSwapLinear(s, 6)),
           (1, pimc.SingleCenterOfMass(s, 1.0))]
    pimc.run(s, 30, ups)
    assert np.isfinite(s.engine.get_beads()).all()
