"""Parity of the CUDA engine with the CPU oracle on the same inputs.

Level (a): action values and staging action differences on given path
configurations agree within 1e-12 relative (FP64).
Level (b): with the same injected normal and uniform draws, every move
(staging, swap, single and cycle centre of mass) proposes the same beads
(within 1e-12) and takes the same accept/reject decision; the chain states
stay equal through long mixed sequences.  Both acceptance semantics, ideal,
trapped, lattice, interacting and hard-core chains, identity and permuted
cycle structures are covered.
"""
import numpy as np
import pytest

from common import c1_small, free_small, pair_small, random_config

pytestmark = pytest.mark.gpu

RTOL = 1e-12

CONFIGS = {
    "trap_ref": c1_small(0),
    "trap_phys": c1_small(1),
    "free_ref": free_small(0),
    "pair_ref": pair_small(0),
    "pair_phys": pair_small(1),
    "pair_phys_lattice": pair_small(1, lattice=2.0),
    "hardcore_phys": pair_small(1, hard=0.05),
    "hardcore_ref": pair_small(0, hard=0.05),
}


def make_pair(name, oracle_mod, seed=1, perm=True, spread=1.0):
    from pimc.engine import ChainParams, Engine
    ek, ok = CONFIGS[name]
    e = Engine(ChainParams(**ek))
    o = oracle_mod.Oracle(oracle_mod.make_params(**ok))
    rng = np.random.default_rng(seed)
    x, nxt = random_config(rng, ek["dim"], ek["N"], ek["M"], ek["L"], spread, perm)
    e.set_beads(x)
    e.set_next(nxt)
    o.set_state(x, nxt)
    return e, o, rng


def assert_states_equal(e, o, tol=1e-11):
    x, V, nx = o.get_state()
    np.testing.assert_array_equal(e.get_next(), nx)
    np.testing.assert_allclose(e.get_beads(), x, rtol=0, atol=tol)
    np.testing.assert_allclose(e.get_links(), V, rtol=tol, atol=tol)


@pytest.mark.parametrize("name", list(CONFIGS))
def test_eval_action(name, oracle_mod, engine_lib):
    e, o, _ = make_pair(name, oracle_mod, seed=3)
    ge, go = e.eval_action(), o.eval_action()
    scale = np.maximum(np.abs(go), 1.0)
    assert np.all(np.abs(ge - go) <= RTOL * scale), (ge, go)


@pytest.mark.parametrize("name", ["trap_ref", "trap_phys", "pair_phys", "pair_phys_lattice"])
def test_staging_weights(name, oracle_mod, engine_lib):
    e, o, rng = make_pair(name, oracle_mod, seed=5)
    ek, _ = CONFIGS[name]
    for _ in range(40):
        n = int(rng.integers(ek["N"]))
        j0 = int(rng.integers(ek["M"]))
        m = int(rng.integers(2, min(ek["M"] - 1, 12) + 1))
        rp = rng.normal(size=(m + 1, ek["dim"])).clip(-ek["L"] * 0.99, ek["L"] * 0.99)
        ge = e.staging_weights(n, j0, m, rp.ravel())
        go = o.staging_weights(n, j0, m, rp.ravel())
        for a, b in zip(ge, go):
            assert abs(a - b) <= RTOL * max(1.0, abs(b)), (ge, go)


def _draw(oracle_mod, normals, uniforms):
    return oracle_mod.Draw(normals, uniforms)


@pytest.mark.parametrize("name", list(CONFIGS))
@pytest.mark.parametrize("warp", [False, True])
def test_staging_moves(name, warp, oracle_mod, engine_lib):
    from pimc.engine import HARDCORE, OPT_FORCE_WARP_WINDOW
    e, o, rng = make_pair(name, oracle_mod, seed=11)
    if warp:
        e.set_option(OPT_FORCE_WARP_WINDOW, 1)
    ek, _ = CONFIGS[name]
    hard = ek.get("hardcore_a", 0.0) > 0
    decisions = []
    for _ in range(150):
        n = int(rng.integers(ek["N"]))
        j0 = int(rng.integers(ek["M"]))
        m = int(rng.integers(2, ek["M"] - 2 + 1))
        nn = (m - 1) * ek["dim"] * (40 if hard else 1)
        normals = rng.standard_normal(nn)
        u = rng.random(1)
        re, pe = e.attempt_staging(n, j0, m, normals, u)
        d = _draw(oracle_mod, normals, u)
        ro, po = o.staging(n, j0, m, d)
        assert re == ro, (n, j0, m, re, ro)
        if re != HARDCORE:
            np.testing.assert_allclose(pe, po, rtol=0, atol=1e-12)
        decisions.append(re)
    assert_states_equal(e, o)
    if not name.startswith("free"):  # without a potential every staging move accepts
        assert len(set(decisions)) > 1  # both outcomes exercised


@pytest.mark.parametrize("name", list(CONFIGS))
def test_swap_moves(name, oracle_mod, engine_lib):
    from pimc.engine import HARDCORE, SKIP
    e, o, rng = make_pair(name, oracle_mod, seed=13, spread=0.6)
    ek, _ = CONFIGS[name]
    hard = ek.get("hardcore_a", 0.0) > 0
    seen = set()
    for _ in range(120):
        j0 = int(rng.integers(ek["M"]))
        m = int(rng.integers(2, ek["M"] - 2 + 1))
        n1 = int(rng.integers(ek["N"]))
        up = float(rng.random())
        normals = rng.standard_normal(2 * (m - 1) * ek["dim"] * (40 if hard else 1))
        u = rng.random(1)
        re, n2e, pe = e.attempt_swap(j0, m, n1, up, normals, u)
        ro, n2o, po = o.swap(j0, m, n1, up, _draw(oracle_mod, normals, u))
        assert (re, n2e) == (ro, n2o), (j0, m, n1, re, ro, n2e, n2o)
        if re not in (SKIP, HARDCORE):
            np.testing.assert_allclose(pe, po, rtol=0, atol=1e-12)
        seen.add(re)
    assert_states_equal(e, o)
    assert 1 in seen


@pytest.mark.parametrize("name", list(CONFIGS))
def test_com_moves(name, oracle_mod, engine_lib):
    e, o, rng = make_pair(name, oracle_mod, seed=17, perm=False)
    ek, _ = CONFIGS[name]
    hard = ek.get("hardcore_a", 0.0) > 0
    for _ in range(60):
        n = int(rng.integers(ek["N"]))
        step = float(rng.uniform(0.1, 1.5))
        u = rng.random((3 * 50) if hard else 3)
        re = e.attempt_com(n, step, u)
        ro = o.com(n, step, _draw(oracle_mod, [], u))
        assert re == ro
    assert_states_equal(e, o)


@pytest.mark.parametrize("name", ["trap_ref", "trap_phys", "pair_phys", "free_ref"])
def test_polymer_com_moves(name, oracle_mod, engine_lib):
    e, o, rng = make_pair(name, oracle_mod, seed=19, perm=True)
    ek, _ = CONFIGS[name]
    for _ in range(40):
        n = int(rng.integers(ek["N"]))
        step = float(rng.uniform(0.05, 0.8))
        u = rng.random(3)
        re = e.attempt_polymer_com(n, step, u)
        ro = o.polymer_com(n, step, _draw(oracle_mod, [], u))
        assert re == ro
    assert_states_equal(e, o)


@pytest.mark.parametrize("name", ["trap_ref", "trap_phys", "pair_ref", "pair_phys", "free_ref"])
def test_mixed_sequence(name, oracle_mod, engine_lib):
    """a long random interleaving of all moves keeps both chains identical"""
    from pimc.engine import HARDCORE, SKIP
    e, o, rng = make_pair(name, oracle_mod, seed=23, spread=0.7)
    ek, _ = CONFIGS[name]
    N, M, dim = ek["N"], ek["M"], ek["dim"]
    for it in range(400):
        kind = rng.choice(4, p=[0.55, 0.25, 0.15, 0.05])
        if kind == 0:
            n, j0, m = int(rng.integers(N)), int(rng.integers(M)), int(rng.integers(2, M - 1))
            nr, u = rng.standard_normal((m - 1) * dim), rng.random(1)
            re, _ = e.attempt_staging(n, j0, m, nr, u)
            ro, _ = o.staging(n, j0, m, _draw(oracle_mod, nr, u))
        elif kind == 1:
            j0, m, n1 = int(rng.integers(M)), int(rng.integers(2, M - 1)), int(rng.integers(N))
            up = float(rng.random())
            nr, u = rng.standard_normal(2 * (m - 1) * dim), rng.random(1)
            re, _, _ = e.attempt_swap(j0, m, n1, up, nr, u)
            ro, _, _ = o.swap(j0, m, n1, up, _draw(oracle_mod, nr, u))
        elif kind == 2:
            nx = o.get_state()[2]
            singles = [i for i in range(N) if nx[i] == i]
            if not singles:
                continue
            n = int(rng.choice(singles))
            u = rng.random(3)
            re = e.attempt_com(n, 0.7, u)
            ro = o.com(n, 0.7, _draw(oracle_mod, [], u))
        else:
            n = int(rng.integers(N))
            u = rng.random(3)
            re = e.attempt_polymer_com(n, 0.3, u)
            ro = o.polymer_com(n, 0.3, _draw(oracle_mod, [], u))
        assert re == ro, (it, kind, re, ro)
    assert_states_equal(e, o, tol=1e-10)
    ge, go = e.eval_action(), o.eval_action()
    assert np.all(np.abs(ge - go) <= 1e-10 * np.maximum(np.abs(go), 1.0))


def test_density_counts_bit_exact(oracle_mod, engine_lib):
    """Density binning (integer work) is identical, including the reference's
    dropped first row/column (src/measurement.jl:45-55)"""
    from pimc.engine import ChainParams, Engine
    rng = np.random.default_rng(29)
    e = Engine(ChainParams(dim=2, N=12, M=20, L=5.0, T=1.0, lam=0.5, harmonic_omega=1.0,
                           density_nbins=64))
    o = oracle_mod.Oracle(oracle_mod.make_params(dim=2, N=12, M=20, L=5.0, T=1.0, lam=0.5, hcoef=0.5))
    x = rng.uniform(-5.0, 5.0, size=(2, 12, 20))
    x[0, 0, :4] = -5.0  # exactly on the dropped first row
    x[1, 1, :3] = -5.0 + 10.0 / 64 * 0.5
    e.set_beads(x)
    o.set_state(x)
    e.reset_measurements()
    e.measure()
    hist, nd = e.density()
    ho = o.density(64)
    np.testing.assert_array_equal(hist, ho)
    assert nd == 20
    assert hist.sum() < 12 * 20  # the shifted histogram drops beads


def test_energy_estimator(oracle_mod, engine_lib):
    """Energy (src/measurement.jl:92-122) on the same configuration"""
    from pimc.engine import ChainParams, Engine
    for name in ("trap_ref", "pair_phys", "pair_phys_lattice"):
        e, o, _ = make_pair(name, oracle_mod, seed=31)
        ek, _ = CONFIGS[name]
        e2 = Engine(ChainParams(**dict(ek, energy_capacity=4)))
        e2.set_beads(e.get_beads())
        e2.set_next(e.get_next())
        e2.measure()
        ge = e2.energies()[0]
        go = o.energy()
        assert np.all(np.abs(ge - go) <= 1e-11 * np.maximum(np.abs(go), 1.0)), (ge, go)
