"""Parity level (c) and whole-engine behaviour on the GPU.

Energies from the device sweeps agree within 2 sigma (blocking over 32
blocks) with exact results of the reference's own Z_N recursion and within
3 sigma (two independent estimates) with the CPU oracle's run! of the
reference algorithm; density normalisation and beads-in-box as the
reference's tests; bit-exact checkpoint/resume; batched == plain launches;
adjoint against central finite differences; failure paths.
"""
import math

import numpy as np
import pytest

from common import GOLDEN, blocking

pytestmark = pytest.mark.gpu


def engine(**kw):
    from pimc.engine import ChainParams, Engine
    return Engine(ChainParams(**kw))


def mix(N, M, ell, L, measure_every=1, swaps=None, com=1, adapt=1, pcom=0):
    from pimc.engine import Mix
    return Mix(stage_slices=ell, stage_min=2, stage_max=ell, stage_minacc=0.0, stage_maxacc=1.0,
               swaps_per_sweep=N if swaps is None else swaps, swap_slices=ell, swap_min=2,
               swap_max=ell, swap_minacc=0.0, swap_maxacc=1.0, com_phases=com, com_step=1.0,
               com_minstep=0.1, com_maxstep=L / 2, adapt=adapt, measure_every=measure_every,
               polymer_com_phases=pcom, pcom_step=0.5, pcom_maxstep=L / 2)


def sweep_energies(e, N, M, ell, L, therm, sweeps, **mk):
    e.set_mix(mix(N, M, ell, L, measure_every=0, **mk))
    e.run(therm)
    e.set_mix(mix(N, M, ell, L, measure_every=1, **mk))
    e.reset_measurements()
    e.run(sweeps)
    return e.energies()


def test_c1_energy_matches_exact():
    """C1: 2D trapped ideal bosons N=10, beta=1, M=20 (physical semantics):
    <E_th> equals the exact canonical energy of the primitive action at M=20
    (13.4986, Z_N recursion of examples/tools/energytools.jl) within 2 sigma"""
    rng = np.random.default_rng(1)
    e = engine(dim=2, N=10, M=20, L=5.0, T=1.0, lam=0.5, harmonic_omega=1.0, semantics=1,
               seed=101, energy_capacity=40000)
    e.set_beads(rng.normal(size=(2, 10, 20)))
    E = sweep_energies(e, 10, 20, 8, 5.0, 2000, 40000)
    m, err = blocking(E[:, 0])
    assert abs(m - GOLDEN["E_C1_primitive_M20"]) < 2 * err, (m, err)
    # and is far from the boltzmannon value: exchange is sampled
    assert m < GOLDEN["E_C1_boltzmannon"] - 3.0


def test_bosons_permutation_sector():
    """4 bosons, M=8: swaps with the heat-bath ratio give the exact bosonic energy"""
    rng = np.random.default_rng(2)
    e = engine(dim=2, N=4, M=8, L=8.0, T=1.0, lam=0.5, harmonic_omega=1.0, semantics=1,
               seed=202, energy_capacity=60000)
    e.set_beads(rng.normal(size=(2, 4, 8)))
    E = sweep_energies(e, 4, 8, 4, 8.0, 2000, 60000)
    m, err = blocking(E[:, 0])
    assert abs(m - GOLDEN["E_N4_primitive_M8"]) < 2 * err, (m, err)
    st = e.stats()
    assert st.accepts[1] > 1000


def test_reference_semantics_matches_oracle(oracle_mod):
    """trapped bosons in the reference's own (bug-compatible) semantics: the
    device sweep and the oracle's run! sample the same distribution"""
    O = oracle_mod
    N, M, ell = 6, 12, 6
    rng = np.random.default_rng(3)
    x0 = rng.normal(size=(2, N, M))
    e = engine(dim=2, N=N, M=M, L=5.0, T=1.0, lam=0.5, harmonic_omega=1.0, semantics=0,
               seed=303, energy_capacity=60000)
    e.set_beads(x0)
    E = sweep_energies(e, N, M, ell, 5.0, 2000, 60000)
    mg, eg = blocking(E[:, 0])
    p = O.make_params(dim=2, N=N, M=M, L=5.0, T=1.0, lam=0.5, hcoef=0.5, semantics=0)
    o = O.Oracle(p)
    o.set_state(x0)
    k = math.ceil(M / ell)
    ups = [(0, 1, ell, 2, ell, 0.0, 1.0, 10, 10000), (1, k, ell, 2, ell, 0.0, 1.0, 10, 10000),
           (2, k, 1.0, 0.1, 2.5, 0.4, 0.6, 10, 10000)]
    per = N * (k + 2)
    o.run(2000 * per, ups, seed=5)
    r = o.run(60000 * per, ups, seed=6, ncycle=per, e_cap=61000)
    mo, eo = blocking(r["energies"][:, 0])
    assert abs(mg - mo) < 3 * math.hypot(eg, eo), (mg, eg, mo, eo)


def test_interacting_physical_matches_oracle(oracle_mod):
    """trapped bosons with the Gaussian pair action in every move (physical
    semantics): device sweep vs the oracle's run!, thermodynamic energy
    including the pair term"""
    O = oracle_mod
    N, M, ell = 8, 12, 6
    rng = np.random.default_rng(4)
    x0 = rng.normal(scale=1.2, size=(2, N, M))
    kw = dict(dim=2, N=N, M=M, L=4.0, T=1.0, lam=0.5)
    e = engine(**kw, harmonic_omega=1.0, interactions=True, pair_g=2.0, pair_sigma=0.5, r_a=1.0,
               semantics=1, seed=404, energy_capacity=30000)
    e.set_beads(x0)
    E = sweep_energies(e, N, M, ell, 4.0, 1000, 30000)
    Eg = E[:, 0] + E[:, 2]
    mg, eg = blocking(Eg)
    p = O.make_params(**kw, hcoef=0.5, interactions=True, pair_g=2.0, pair_sigma=0.5, r_a=1.0,
                      semantics=1)
    o = O.Oracle(p)
    o.set_state(x0)
    k = math.ceil(M / ell)
    ups = [(0, 1, ell, 2, ell, 0.0, 1.0, 10, 10000), (1, k, ell, 2, ell, 0.0, 1.0, 10, 10000),
           (2, k, 1.0, 0.1, 2.0, 0.4, 0.6, 10, 10000)]
    per = N * (k + 2)
    o.run(1000 * per, ups, seed=7)
    r = o.run(30000 * per, ups, seed=8, ncycle=per, e_cap=31000)
    Eo = r["energies"][:, 0] + r["energies"][:, 2]
    mo, eo = blocking(Eo)
    assert abs(mg - mo) < 3 * math.hypot(eg, eo), (mg, eg, mo, eo)
    # the interaction raises the energy above the ideal-gas value
    assert E[:, 2].mean() > 0


def test_density_normalisation_and_box():
    """test/testmeasurements.jl:21-29 and test/testsystem.jl:37-56 on the device"""
    e = engine(dim=2, N=2, M=100, L=4.0, T=1.0, lam=1.0, lattice_V0=8.0, lattice_a=2.0,
               density_nbins=500, seed=505)
    from pimc.engine import Mix
    e.set_mix(Mix(stage_slices=20, stage_max=64, swaps_per_sweep=2, swap_slices=20, swap_max=64,
                  com_step=3.0, com_maxstep=2.0, measure_every=1))
    e.run(400)
    hist, nd = e.density()
    assert abs(hist.sum() / nd - 2) < 2e-2
    x = e.get_beads()
    assert not (np.all(x > 4.0, axis=0) | np.all(x < -4.0, axis=0)).any()
    assert np.all(x >= -4.0) and np.all(x <= 4.0)


def test_checkpoint_resume_bit_exact():
    e = engine(dim=2, N=16, M=16, L=4.0, T=0.5, lam=0.5, harmonic_omega=1.0, interactions=True,
               pair_g=1.0, pair_sigma=0.5, r_a=1.0, semantics=1, seed=606, density_nbins=32,
               energy_capacity=64)
    e.set_mix(mix(16, 16, 8, 4.0, measure_every=2, pcom=1))
    e.run(10)
    blob = e.get_state()
    e.run(12)
    xa, na, Ea = e.get_beads(), e.get_next(), e.energies()
    e.set_state(blob)
    e.run(12)
    np.testing.assert_array_equal(e.get_beads(), xa)
    np.testing.assert_array_equal(e.get_next(), na)
    np.testing.assert_array_equal(e.energies(), Ea)


def test_batched_equals_plain_and_tuner_is_transparent():
    """the persistent/queue/graph path, in every launch shape (one CTA per
    chain with and without shared-memory staging, one warp per chain), and
    one launch per chain produce the same chains bit for bit; the tuner
    restores the state it advances"""
    from pimc.engine import ChainParams, Engine
    rng = np.random.default_rng(7)
    ps = []
    for i in range(24):
        N = int(rng.integers(4, 40))
        M = int(rng.choice([8, 16, 32]))
        ps.append(ChainParams(dim=2, N=N, M=M, L=6.0, T=1.0 / rng.uniform(0.5, 3), lam=0.5,
                              harmonic_omega=1.0, interactions=bool(i % 2), pair_g=float(rng.uniform(0, 2)),
                              pair_sigma=0.5, r_a=1.5, semantics=int(i % 3 == 0), seed=1000 + i,
                              energy_capacity=8))
    shapes = [None, dict(block=64, sweeps_per_launch=2, warp_per_chain=True),
              dict(block=256, sweeps_per_launch=1, warp_per_chain=True),
              dict(block=128, sweeps_per_launch=3, state_smem_bytes=0),
              dict(block=256, sweeps_per_launch=1, state_smem_bytes=100 * 1024),
              dict(block=64, sweeps_per_launch=2, state_smem_bytes=0, split_phases=1),
              dict(block=128, sweeps_per_launch=1, state_smem_bytes=32 * 1024, split_phases=1),
              dict(block=64, sweeps_per_launch=1, state_smem_bytes=0, split_phases=1,
                   phase_block=[256, 64, 128]),
              dict(block=64, sweeps_per_launch=1, state_smem_bytes=0, split_phases=1,
                   phase_block=[128, 64, 128], phase_warp=[0, 1, 0]),
              dict(block=128, sweeps_per_launch=1, state_smem_bytes=0, split_phases=1,
                   phase_block=[128, 32, 0], phase_warp=[0, 1, 0]),
              # the swap kernels compiled for 170 and 255 registers a thread
              dict(block=64, sweeps_per_launch=1, state_smem_bytes=0, split_phases=1,
                   phase_block=[128, 64, 128], phase_regs=[0, 170, 0]),
              dict(block=64, sweeps_per_launch=1, state_smem_bytes=32 * 1024, split_phases=1,
                   phase_regs=[0, 255, 0]),
              # neighbour candidates from row scans, from cell lists everywhere
              dict(block=64, sweeps_per_launch=1, state_smem_bytes=0, split_phases=1,
                   phase_block=[128, 64, 128], cell_lists=1),
              dict(block=128, sweeps_per_launch=1, state_smem_bytes=0, cell_lists=3)]
    b = Engine(ps)
    for i, p in enumerate(ps):
        b.set_mix(mix(p.N, p.M, min(8, p.M // 2), 6.0, measure_every=3), chain=i)
    b.run_plain(6)
    sb = b.total_stats()
    for shape in shapes:
        a = Engine(ps)
        for i, p in enumerate(ps):
            a.set_mix(mix(p.N, p.M, min(8, p.M // 2), 6.0, measure_every=3), chain=i)
        if shape is None:
            a.tune(sweeps_per_trial=2)
        else:
            a.set_launch(**shape)
            got = a.launch
            for k, v in shape.items():
                assert got[k] == v
        a.run_batched(6)
        for c in range(len(ps)):
            np.testing.assert_array_equal(a.get_beads(c), b.get_beads(c))
            np.testing.assert_array_equal(a.get_next(c), b.get_next(c))
            # the estimator's reduction order follows the threads per chain
            np.testing.assert_allclose(a.energies(c), b.energies(c), rtol=1e-13, atol=1e-13)
        sa = a.total_stats()
        assert sa.bead_updates == sb.bead_updates and sa.sweeps == sb.sweeps == 6 * len(ps)
        a.close()


def test_launch_shape_rejects_bad_values():
    from pimc.engine import ChainParams, Engine
    from pimc._native import PimcError
    e = Engine([ChainParams(dim=2, N=4, M=8, L=6.0, T=1.0, lam=0.5, harmonic_omega=1.0, seed=1)] * 2)
    for bad in [dict(block=48), dict(block=512, warp_per_chain=True), dict(block=16, warp_per_chain=True),
                dict(block=128, sweeps_per_launch=0), dict(block=128, state_smem_bytes=-1),
                dict(block=64, split_phases=2), dict(block=64, warp_per_chain=True, split_phases=1),
                dict(block=64, split_phases=0, phase_block=(128, 0, 0)),
                dict(block=64, split_phases=1, phase_block=(96 + 1, 0, 0)),
                dict(block=64, split_phases=1, phase_warp=(1, 0, 0)),
                dict(block=64, split_phases=0, phase_block=(0, 64, 0), phase_warp=(0, 1, 0)),
                dict(block=64, split_phases=1, phase_block=(0, 512, 0), phase_warp=(0, 1, 0)),
                dict(block=64, split_phases=1, phase_warp=(0, 2, 0)),
                dict(block=64, split_phases=0, phase_regs=(0, 170, 0)),
                dict(block=64, split_phases=1, phase_regs=(0, 200, 0)),
                dict(block=64, split_phases=1, phase_regs=(170, 0, 0)),
                dict(block=64, split_phases=1, phase_block=(0, 128, 0), phase_regs=(0, 255, 0)),
                dict(block=64, split_phases=1, phase_block=(0, 64, 0), phase_warp=(0, 1, 0),
                     phase_regs=(0, 170, 0)),
                dict(block=64, cell_lists=-1), dict(block=64, cell_lists=4)]:
        with pytest.raises(PimcError):
            e.set_launch(**bad)
    e.close()


def _fd_action(e, oracle_free=None):
    a = e.eval_action()
    return -(a[1] + a[2])  # S_pot = -sum lnV - sum lnU


def test_adjoint_matches_finite_differences():
    """C5-like small chain: lattice + trap + Gaussian pair; dS/dr per bead and
    dS/d(V0, omega, g) within 1e-6 relative of central differences (h = 1e-5)"""
    rng = np.random.default_rng(8)
    N, M = 6, 8
    e = engine(dim=2, N=N, M=M, L=4.0, T=0.25, lam=0.5, harmonic_omega=0.7, lattice_V0=4.0,
               lattice_a=1.0, interactions=True, pair_g=1.0, pair_sigma=0.6, r_a=1.0, semantics=1)
    x = rng.normal(scale=0.6, size=(2, N, M))
    nxt = rng.permutation(N).astype(np.int32)
    e.set_beads(x)
    e.set_next(nxt)
    g, th, ex = e.adjoint()
    h = 1e-5
    for (d, n, j) in [(0, 0, 0), (1, 2, 5), (0, 3, 7), (1, 5, 1), (0, 1, 4)]:
        xp, xm = x.copy(), x.copy()
        xp[d, n, j] += h
        xm[d, n, j] -= h
        e.set_beads(xp)
        sp = _fd_action(e)
        e.set_beads(xm)
        sm = _fd_action(e)
        fd = (sp - sm) / (2 * h)
        assert abs(g[d, n, j] - fd) <= 1e-6 * max(abs(fd), 1e-3), (d, n, j, g[d, n, j], fd)
    e.set_beads(x)
    base = (4.0, 0.7, 1.0)
    for q in range(3):
        vp, vm = list(base), list(base)
        vp[q] += h
        vm[q] -= h
        e.set_potential(*vp)
        sp = _fd_action(e)
        e.set_potential(*vm)
        sm = _fd_action(e)
        fd = (sp - sm) / (2 * h)
        assert abs(th[q] - fd) <= 1e-6 * max(abs(fd), 1e-6), (q, th[q], fd)
    e.set_potential(*base)
    S = _fd_action(e)
    assert abs((ex[0] + ex[1]) - S) <= 1e-10 * max(1.0, abs(S))


def test_virial_from_adjoint_matches_thermodynamic():
    """the adjoint's virial estimator and the thermodynamic estimator sample
    the same energy (-d ln Z / d beta) on a small lattice + trap + pair chain"""
    rng = np.random.default_rng(9)
    N, M = 4, 16
    e = engine(dim=2, N=N, M=M, L=6.0, T=0.5, lam=0.5, harmonic_omega=1.0, lattice_V0=1.0,
               lattice_a=1.0, interactions=True, pair_g=1.0, pair_sigma=0.3, r_a=1.0, semantics=1,
               energy_capacity=10, seed=909)
    e.set_beads(rng.normal(size=(2, N, M)))
    e.set_mix(mix(N, M, 8, 6.0, measure_every=0))
    e.run(500)
    eth, ev = [], []
    for _ in range(4000):
        e.run(2)
        e.reset_measurements()
        e.measure()
        r = e.energies()[0]
        eth.append(r[0] + r[2])
        ev.append(e.adjoint(want_beads=False)[2][2])
    mt, et = blocking(eth)
    mv, evv = blocking(ev)
    assert abs(mt - mv) < 3 * math.hypot(et, evv), (mt, et, mv, evv)
    # the virial from the adjoint equals the estimator's own virial column
    assert abs(ev[-1] - (r[1] + r[3])) < 1e-9 * max(1.0, abs(ev[-1]))


def test_failure_paths():
    from pimc import PimcError
    e = engine(dim=2, N=5, M=10, L=4.0, T=1.0, lam=0.5, harmonic_omega=1.0, seed=11)
    x0 = e.get_beads()
    with pytest.raises(PimcError, match="permutation"):
        e.set_next(np.array([0, 0, 1, 2, 3], dtype=np.int32))
    with pytest.raises(PimcError, match="normals"):
        e.attempt_staging(0, 0, 5, np.zeros(3), [0.5])
    # a run-out of the Metropolis uniform restores the chain
    for _ in range(200):
        xb = e.get_beads()
        try:
            e.attempt_staging(1, 2, 6, np.full(10, 3.0), [])
        except PimcError as err:
            assert "draws" in str(err)
            np.testing.assert_array_equal(e.get_beads(), xb)
            break
    else:
        pytest.fail("the missing uniform was never needed")
    with pytest.raises(PimcError):
        e.attempt_com(0, 1.0, [0.5])  # too few uniforms
    with pytest.raises(PimcError, match="window"):
        e.attempt_staging(0, 0, 10, np.zeros(20), [0.5])
    # windows longer than the device's 64-slice limit are refused on the host
    big = engine(dim=2, N=3, M=80, L=4.0, T=1.0, lam=0.5, harmonic_omega=1.0, seed=13)
    with pytest.raises(PimcError, match="window"):
        big.staging_weights(0, 0, 70, np.zeros(71 * 2))
    with pytest.raises(PimcError, match="window"):
        big.attempt_staging(0, 0, 70, np.zeros(69 * 2), [0.5])
    # the hard-core retry cap ends a move as a rejection, not a hang: with
    # zero normals every retry proposes the bridge's mean, here particle 0's
    # own start, where particle 1 sits
    h = engine(dim=2, N=3, M=8, L=1.0, T=1.0, lam=0.5, hardcore_a=0.3, r_a=0.6, retry_cap=50,
               seed=12, interactions=True, pair_g=0.0, pair_sigma=0.3)
    x = np.zeros((2, 3, 8))
    x[:, 2, :] = 0.7
    h.set_beads(x)
    r, _ = h.attempt_staging(0, 0, 4, np.zeros(3 * 2 * 60), [0.5])
    assert r == 3


def test_api_mirror_end_to_end():
    """System / updates / run / Density / Energy as a PIMC.jl user writes them
    (examples/energy_2d_harmonically_trapped_bose_gas.jl)"""
    import pimc
    s = pimc.System(pimc.Harmonic(1.0), dV="grad", λ=0.5, M=10, N=3, L=5.0, T=1.0,
                    length_measurement_cycle=10, semantics=pimc.SEM_PHYSICAL)
    ups = [(1, pimc.SingleCenterOfMass(s, 1.0)), (1, pimc.ReshapeLinear(s, 5)),
           (1, pimc.ReshapeSwapLinear(s, 5))]
    mea = [pimc.Energy(s, 100000), pimc.Density(s, nbins=32)]
    pimc.run(s, 3000, ups)
    pimc.run(s, 30000, ups, Zmeasurements=mea)
    E = np.array(mea[0].energy[3])
    assert len(E) > 50 and np.isfinite(E).all()
    assert s.N_MC[3] == len(E)
    assert abs(mea[1].dens.sum() / mea[1].ndata - 3) < 0.05
    assert 0 < pimc.acceptance(ups[1][1].counter_var.queue) <= 1
    # single attempts through the callables
    for _ in range(20):
        pimc.apply(s, ups[1][1])
    w = s.world
    assert len(w) == 3 and w[0].r.shape == (10, 2)


@pytest.mark.parametrize("semantics", [0, 1])
def test_bounded_decisions_equal_exact_decisions(semantics):
    """sweeps decide most moves from bounded estimates (pair sums from the
    position mirror, FP32 log-space Metropolis tests, the reference rules'
    pair-free early accept); with PIMC_OPT_EXACT_DECISIONS every decision
    comes from the exact FP64 sums instead, and the chains stay identical bit
    for bit through many sweeps of interacting, permuting chains"""
    from pimc.engine import ChainParams, Engine, OPT_EXACT_DECISIONS
    rng = np.random.default_rng(11 + semantics)
    ps = []
    for i in range(16):
        N = int(rng.integers(8, 64))
        M = int(rng.choice([16, 32]))
        ps.append(ChainParams(dim=2, N=N, M=M, L=6.0, T=1.0 / rng.uniform(0.5, 3), lam=0.5,
                              harmonic_omega=1.0, interactions=True, pair_g=float(rng.uniform(0.2, 2)),
                              pair_sigma=0.5, r_a=1.5, semantics=semantics, seed=500 + i,
                              energy_capacity=8))
    fast, exact = Engine(ps), Engine(ps)
    exact.set_option(OPT_EXACT_DECISIONS, 1)
    for i, p in enumerate(ps):
        m = mix(p.N, p.M, min(8, p.M // 2), 6.0, measure_every=2, pcom=1)
        fast.set_mix(m, chain=i)
        exact.set_mix(m, chain=i)
    fast.run_batched(12)
    exact.run_batched(12)
    for c in range(len(ps)):
        np.testing.assert_array_equal(fast.get_beads(c), exact.get_beads(c))
        np.testing.assert_array_equal(fast.get_next(c), exact.get_next(c))
    sf, se = fast.total_stats(), exact.total_stats()
    assert sf.accepts == se.accepts and sf.attempts == se.attempts
    assert sum(sf.accepts) > 0 and min(sf.accepts[:3]) > 0  # staging, swaps, CoM all accept
    fast.close()
    exact.close()


def test_reference_rules_swap_kernel_equals_generic():
    """a batch whose every chain follows the reference's rules (Gaussian pair,
    no hard core, no contact table) runs its swaps in the kernel compiled for
    those rules alone; the chains equal, bit for bit, the same chains swept by
    the generic kernels (plain launches, and a batch with one physical-rules
    chain added, which keeps the generic swap kernel)"""
    from pimc.engine import ChainParams, Engine
    rng = np.random.default_rng(17)
    ps = []
    for i in range(12):
        N = int(rng.integers(8, 96))
        M = int(rng.choice([16, 32]))
        ps.append(ChainParams(dim=2, N=N, M=M, L=6.0, T=1.0 / rng.uniform(0.5, 3), lam=0.5,
                              harmonic_omega=1.0, interactions=bool(i % 4), pair_g=float(rng.uniform(0, 2)),
                              pair_sigma=0.5, r_a=1.5, semantics=0, seed=3000 + i, energy_capacity=8))
    extra = ChainParams(dim=2, N=12, M=16, L=6.0, T=1.0, lam=0.5, harmonic_omega=1.0,
                        interactions=True, pair_g=1.0, pair_sigma=0.5, r_a=1.5, semantics=1,
                        seed=3999, energy_capacity=8)
    engines = [Engine(ps), Engine(ps), Engine(ps + [extra])]
    for e in engines:
        for i, p in enumerate(ps):
            e.set_mix(mix(p.N, p.M, min(8, p.M // 2), 6.0, measure_every=3), chain=i)
    engines[2].set_mix(mix(12, 16, 8, 6.0, measure_every=3), chain=len(ps))
    for e in (engines[0], engines[2]):
        e.set_launch(block=64, sweeps_per_launch=1, state_smem_bytes=0, split_phases=1,
                     phase_block=[128, 64, 128])
        e.run_batched(8)
    engines[1].run_plain(8)
    for c in range(len(ps)):
        for e in engines[1:]:
            np.testing.assert_array_equal(engines[0].get_beads(c), e.get_beads(c))
            np.testing.assert_array_equal(engines[0].get_next(c), e.get_next(c))
    assert engines[0].total_stats().accepts[1] > 0
    for e in engines:
        e.close()
