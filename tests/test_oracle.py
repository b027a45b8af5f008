"""CPU tests of the oracle: pinned against the reference's own known answers
(the exact N=1 energy constant, the Z_N recursion of
examples/tools/energytools.jl, the density normalisation of
test/testmeasurements.jl and the beads-in-box check of test/testsystem.jl),
against published Philox known-answer vectors, and for internal consistency
of its action differences."""
import math

import numpy as np
import pytest

from common import GOLDEN, blocking


def test_philox_known_answers(oracle_mod):
    # Random123 known-answer vectors for philox4x32-10
    O = oracle_mod
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6,
                                                             0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                    [0xA4093822, 0x299F31D0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_teleport_and_distance(oracle_mod):
    O = oracle_mod
    # src/propagator.jl:6-9, 30-32
    assert O.teleport(5.5, 5.0) == -4.5
    assert O.teleport(-5.0, 5.0) == -5.0
    assert O.teleport(-5.5, 5.0) == 4.5
    assert O.teleport(14.0, 5.0) == 4.0
    assert O.distance(4.5, -4.5, 5.0) == 1.0
    assert O.distance(1.0, -2.0, 5.0) == 3.0
    for x in np.linspace(-12, 12, 97):
        y = O.teleport(float(x), 5.0)
        assert -5.0 <= y < 5.0 + 1e-12


def test_action_pieces(oracle_mod):
    O = oracle_mod
    p = O.make_params(dim=2, N=2, M=10, L=5.0, T=1.0, lam=0.5, hcoef=0.5, V0=2.0, lat_a=1.0,
                      interactions=True, pair_g=1.5, pair_sigma=0.5, r_a=1.25)
    L = O.lib()
    a = np.array([0.3, -0.7])
    b = np.array([4.8, -4.9])
    dp = lambda v: v.ctypes.data_as(O.C.POINTER(O.C.c_double))
    d = [min(2 * 5.0 - abs(a[i] - b[i]), abs(a[i] - b[i])) for i in range(2)]
    lnK = L.orc_lnK(O.C.byref(p), dp(a), dp(b), 0.2)
    assert math.isclose(lnK, -(d[0] ** 2 + d[1] ** 2) / (4 * 0.2 * 0.5), rel_tol=1e-15)
    V = lambda r: 0.5 * (r[0] ** 2 + r[1] ** 2) + 2.0 * (math.sin(math.pi * r[0]) ** 2 + math.sin(math.pi * r[1]) ** 2)
    assert math.isclose(L.orc_Vext(O.C.byref(p), dp(a)), V(a), rel_tol=1e-14)
    tau = 1.0 / 10
    assert math.isclose(L.orc_lnV(O.C.byref(p), dp(a), dp(b)), -0.5 * tau * (V(a) + V(b)), rel_tol=1e-14)
    v = lambda r2: 1.5 * math.exp(-r2 / (2 * 0.25))
    d1, d2 = np.array([0.1, 0.2]), np.array([0.3, 0.05])
    assert math.isclose(L.orc_lnU(O.C.byref(p), dp(d1), dp(d2)),
                        math.log(math.exp(-0.5 * tau * (v(0.05) + v(0.0925)))), rel_tol=1e-13)
    assert p.nbins == 8 and math.isclose(p.rc, 1.25)


def test_golden_pins_reference_constant():
    # the recursion restated in make_golden.py reproduces the reference's
    # hard-coded N=1 value (examples/energy_2d_harmonically_trapped_bose_gas.jl:28)
    assert math.isclose(GOLDEN["E_N1_d2_beta1"], GOLDEN["E_N1_d2_beta1_reference_constant"],
                        rel_tol=1e-14)
    assert math.isclose(GOLDEN["E_N1_d2_beta1"], 1.0 / math.tanh(0.5), rel_tol=1e-14)  # coth(1/2)
    # values quoted for the configs
    assert abs(GOLDEN["E_C1_exact"] - 13.5018169110) < 1e-9
    assert abs(GOLDEN["E_C1_primitive_M20"] - 13.4986242011) < 1e-9
    assert abs(GOLDEN["E_C2_winding0"] - 19.6914005254) < 1e-9


def _run_energy(O, params, sweeps, ell, seed, x0=None, nxt=None, com=True, swap=True):
    o = O.Oracle(params)
    rng = np.random.default_rng(seed)
    if x0 is None:
        x0 = rng.normal(size=(params.dim, params.N, params.M))
    o.set_state(x0, nxt)
    M, N = params.M, params.N
    k = math.ceil(M / ell)
    ups = [(0, 1, ell, 2, M - 2, 0.0, 1.0, 10, 10000)]
    if swap and N > 1:
        ups.append((1, k, ell, 2, M - 2, 0.0, 1.0, 10, 10000))
    if com:
        ups.append((2, k, 1.0, 0.1, params.L / 2, 0.4, 0.6, 10, 10000))
    per = N * (k + len(ups) - 1)
    o.run(200 * per, ups, seed=seed)
    r = o.run(sweeps * per, ups, seed=seed + 1, ncycle=per, e_cap=sweeps + 10)
    return r


def test_oracle_single_particle_energy(oracle_mod):
    """N=1, 2D oscillator, M=20: the primitive estimator averages to the
    exact finite-M value (closed Gaussian chain)"""
    O = oracle_mod
    p = O.make_params(dim=2, N=1, M=20, L=8.0, T=1.0, lam=0.5, hcoef=0.5, semantics=O.SEM_PHYSICAL)
    r = _run_energy(O, p, 40000, 8, 3)
    E, err = blocking(r["energies"][:, 0])
    assert abs(E - GOLDEN["E_N1_primitive_M20"]) < 2.5 * err, (E, err)


def test_oracle_swap_detailed_balance(oracle_mod):
    """four bosons with permutations, M=8: the physical semantics (with the
    heat-bath normalisation ratio) reproduces the exact bosonic energy of the
    primitive action from the Z_N recursion"""
    O = oracle_mod
    p = O.make_params(dim=2, N=4, M=8, L=8.0, T=1.0, lam=0.5, hcoef=0.5, semantics=O.SEM_PHYSICAL)
    r = _run_energy(O, p, 60000, 4, 5)
    E, err = blocking(r["energies"][:, 0])
    assert abs(E - GOLDEN["E_N4_primitive_M8"]) < 2.5 * err, (E, err)
    # permutations happened (bosonic energy is far below the boltzmannon one)
    assert r["accepts"][1] > 100


def test_density_normalisation_and_box(oracle_mod):
    """sum(dens)/ndata ~ N (test/testmeasurements.jl:21-29) and no bead outside
    the box after a run (test/testsystem.jl:37-56)"""
    O = oracle_mod
    p = O.make_params(dim=2, N=2, M=100, L=4.0, T=1.0, lam=1.0, V0=8.0, lat_a=2.0)
    o = O.Oracle(p)
    o.init_world(seed=9)
    ups = [(2, 2, 3.0, 0.1, 2.0, 0.4, 0.6, 10, 10000), (0, 1, 20, 2, 98, 0.6, 0.8, 10, 10000),
           (1, 1, 20, 2, 98, 0.6, 0.8, 10, 10000)]
    r = o.run(10000, ups, seed=11, ncycle=10, dens_nb=500)
    numb = r["hist"].sum() / r["ndata"]
    # the reference's histogram drops the first row and column (about 2/500)
    assert abs(numb - p.N) < 2e-2
    x, _, _ = o.get_state()
    outside = np.all(x > p.L, axis=0) | np.all(x < -p.L, axis=0)
    assert not outside.any()


def test_physical_weights_are_action_differences(oracle_mod):
    """w_upd - w_init of a staging window equals the change of the potential +
    pair action evaluated on the whole configuration"""
    O = oracle_mod
    rng = np.random.default_rng(2)
    p = O.make_params(dim=2, N=12, M=16, L=4.0, T=0.5, lam=0.5, hcoef=0.5, interactions=True,
                      pair_g=1.0, pair_sigma=0.5, r_a=1.0, semantics=O.SEM_PHYSICAL)
    o = O.Oracle(p)
    x = rng.normal(scale=0.8, size=(2, 12, 16))
    nxt = rng.permutation(12).astype(np.int32)
    o.set_state(x, nxt)
    for _ in range(20):
        n, j0, m = int(rng.integers(12)), int(rng.integers(16)), int(rng.integers(2, 10))
        x, _, nx = o.get_state()
        own = [n if j0 + t < 16 else nx[n] for t in range(m + 1)]
        sl = [(j0 + t) % 16 for t in range(m + 1)]
        rp = np.array([[x[0, own[t], sl[t]], x[1, own[t], sl[t]]] for t in range(m + 1)])
        rp[1:m] += rng.normal(scale=0.2, size=(m - 1, 2))
        wi, wu = o.staging_weights(n, j0, m, rp.ravel())
        a0 = o.eval_action()
        x2 = x.copy()
        for t in range(1, m):
            x2[:, own[t], sl[t]] = rp[t]
        o2 = O.Oracle(p)
        o2.set_state(x2, nx)
        a1 = o2.eval_action()
        dS = (a1[1] + a1[2]) - (a0[1] + a0[2])
        assert abs((wu - wi) - dS) < 1e-11 * max(1.0, abs(dS))


def _contact_lnU_formula(tab, R, tau, mu, d1, d2, physical, L):
    """build_prop_int's prop_int (src/propagator.jl:74-89) and lnU
    (src/system.jl:26-28) restated with scipy's grid interpolator"""
    from scipy.interpolate import RegularGridInterpolator
    n = tab.shape[0]
    grid = 1e-20 + np.arange(n) * ((R - 1e-20) / (n - 1))
    itp = RegularGridInterpolator((grid, grid), tab, method="linear")
    a, b = np.abs(d1), np.abs(d2)
    r1 = min(max(float(np.sqrt(a @ a)), grid[0]), R)
    r2 = min(max(float(np.sqrt(b @ b)), grid[0]), R)
    if physical:
        e = d1 - d2
        e = np.where(np.abs(e) > L, e - np.sign(e) * 2 * L, e)
    else:
        e = a - b
    rel0 = math.exp(-float(e @ e) / (4 * tau)) / (4 * math.pi * tau)
    p = 1.0 + float(itp([[r1, r2]])[0]) / rel0
    return -mu if p < 0 else math.log(p)


def test_oracle_contact_lnU(oracle_mod):
    """the oracle's tabulated contact lnU against an independent restatement:
    linear interpolation on the reference's grid, per-component absolute
    differences (reference rules) or wrapped signed ones (physical rules),
    -mu where prop_int < 0, radii clamped to the table"""
    O = oracle_mod
    L = O.lib()
    dp = lambda v: v.ctypes.data_as(O.C.POINTER(O.C.c_double))
    rng = np.random.default_rng(3)
    n, R, Lh, mu = 12, 2.0, 1.5, 0.7
    tab = rng.normal(size=(n, n))
    tab = tab + tab.T
    for sem in (O.SEM_REFERENCE, O.SEM_PHYSICAL):
        p = O.make_params(dim=2, N=2, M=8, L=Lh, T=2.0, interactions=True, r_a=0.5, semantics=sem,
                          mu=mu, contact_table=tab, contact_range=R)
        tau = p.tau
        branches = set()
        for _ in range(300):
            d1 = rng.uniform(-Lh, Lh, 2)
            d2 = rng.uniform(-Lh, Lh, 2) * rng.choice([0.05, 1.0])
            got = L.orc_lnU(O.C.byref(p), dp(d1), dp(d2))
            want = _contact_lnU_formula(tab, R, tau, mu, d1, d2, sem == O.SEM_PHYSICAL, Lh)
            assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (sem, d1, d2, got, want)
            branches.add(got == -mu)
        assert branches == {True, False}
    # radii beyond the table clamp to its last row and column
    p = O.make_params(dim=2, N=2, M=8, L=4.0, T=2.0, interactions=True, r_a=0.5, mu=mu,
                      contact_table=tab, contact_range=R)
    d1, d2 = np.array([3.0, 1.0]), np.array([2.9, 1.1])
    got = L.orc_lnU(O.C.byref(p), dp(d1), dp(d2))
    assert abs(got - _contact_lnU_formula(tab, R, p.tau, mu, d1, d2, False, 4.0)) <= 1e-12


def test_contact_propagator_host_and_nnrange(oracle_mod):
    """pimc.build_prop_int's host evaluation is the oracle's prop_int, and
    determine_nnrange finds the 0.999 crossing (src/system.jl:10-15)"""
    import pimc
    O = oracle_mod
    L = O.lib()
    dp = lambda v: v.ctypes.data_as(O.C.POINTER(O.C.c_double))
    rng = np.random.default_rng(5)
    n, R = 40, 3.0
    tab = -np.abs(rng.normal(scale=0.05, size=(n, n)))
    tab = tab + tab.T
    p = O.make_params(dim=2, N=2, M=8, L=2.0, T=2.0, interactions=True, r_a=0.5, mu=0.0,
                      contact_table=tab, contact_range=R)
    prop = pimc.ContactPropagator(R, 1.0, p.tau, n=n, table=tab)
    for _ in range(100):
        d1, d2 = rng.uniform(0, 2.0, 2), rng.uniform(0, 2.0, 2)
        v = prop(d1, d2, p.tau)
        lnu = L.orc_lnU(O.C.byref(p), dp(d1), dp(d2))
        if v > 0:
            assert abs(math.log(v) - lnu) <= 1e-12 * max(1.0, abs(lnu))
        else:
            assert lnu == 0.0
    f = lambda r1, r2, t: 1.0 - 0.5 * math.exp(-float(np.asarray(r1)[0]) ** 2)
    r = pimc.determine_nnrange(f, 0.1, 1e-20, 4.0)
    assert abs(r - math.sqrt(math.log(500.0))) < 1e-12


def test_oracle_superfluid_and_radial_on_known_paths(oracle_mod):
    """a square path of side s enclosing the origin counter-clockwise has
    A_z = s^2 and sum r^2 / M = s^2 / 2; a path that wraps the periodic box
    once has W^2 = (2L)^2; pair distances land in their floor bins"""
    O = oracle_mod
    s = 0.8
    o = O.Oracle(O.make_params(dim=2, N=1, M=4, L=3.0, T=1.0))
    x = np.array([[[s / 2, -s / 2, -s / 2, s / 2]], [[s / 2, s / 2, -s / 2, -s / 2]]])
    o.set_state(x)
    w2, az, rsq = o.superfluid()
    assert abs(w2) < 1e-24 and abs(az - s * s) < 1e-15 and abs(rsq - s * s / 2) < 1e-15
    L, M = 2.0, 10
    o = O.Oracle(O.make_params(dim=2, N=1, M=M, L=L, T=1.0))
    xs = -L + 2 * L * (np.arange(M) + 0.5) / M
    o.set_state(np.array([[xs], [np.zeros(M)]]))
    w2, az, _ = o.superfluid()
    assert abs(w2 - (2 * L) ** 2) < 1e-12 and abs(az) < 1e-15
    o = O.Oracle(O.make_params(dim=2, N=3, M=1 + 3, L=2.0, T=1.0))
    x = np.zeros((2, 3, 4))
    x[0, 1, :] = 0.55     # particle 1 at distance 0.55 from particle 0
    x[0, 2, :] = -1.9     # particle 2: 1.9 from 0 and, through the wall, 1.55 from 1
    o.set_state(x)
    hist = o.radial(20, 0.1)
    want = np.zeros(20)
    for r in (0.55, 1.9, 4.0 - 2.45):
        want[int(np.floor(r / 0.1))] += 4
    np.testing.assert_array_equal(hist, want)


def test_lattice_angle_sets_match_the_reference():
    """l25 / l65 (examples/tools/potentialtools.jl) are the directions of the
    integer points on x^2 + y^2 = 25 and 65; the engine builds them that way"""
    import json
    import os

    import pimc
    from common import HERE
    gold = json.load(open(os.path.join(HERE, "golden", "lattice_angles.json")))
    for name in ("l25", "l65"):
        np.testing.assert_allclose(pimc.lattice_angles(name), sorted(gold[name]), rtol=0, atol=1e-15)
    assert pimc.lattice_angles("cubic") == [0.0, math.pi / 2, math.pi, 3 * math.pi / 2]


def test_oracle_optical_lattice_potential(oracle_mod):
    """the oracle's V with beams equals normalized_intensity restated in
    numpy (pimc.OpticalLattice), helical or not, summed with the trap"""
    import pimc
    O = oracle_mod
    L = O.lib()
    dp = lambda v: v.ctypes.data_as(O.C.POINTER(O.C.c_double))
    rng = np.random.default_rng(8)
    for helical in (False, True):
        ang = pimc.lattice_angles("l25")
        p = O.make_params(dim=2, N=1, M=4, L=5.0, T=1.0, hcoef=0.5,
                          beams=(ang, 0.7, -4.0, helical))
        host = pimc.OpticalLattice(ang, 0.7, -4.0, helical) + pimc.Harmonic(1.0)
        for _ in range(50):
            r = rng.uniform(-5, 5, 2)
            assert abs(L.orc_Vext(O.C.byref(p), dp(r)) - host(r)) <= 1e-12 * max(1.0, abs(host(r)))
            h = 1e-6
            fd = [(host(r + h * e) - host(r - h * e)) / (2 * h) for e in np.eye(2)]
            np.testing.assert_allclose(host.grad(r), fd, rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("kind", ["contact", "lattice"])
def test_physical_weights_are_action_differences_new_terms(oracle_mod, kind):
    """the same identity with the tabulated contact propagator and with the
    optical lattice: a staging window's w_upd - w_init is the change of the
    whole configuration's potential + pair action"""
    import pimc
    O = oracle_mod
    rng = np.random.default_rng(4)
    extra = {}
    if kind == "contact":
        n = 40
        tab = -np.abs(rng.normal(scale=0.02, size=(n, n)))
        extra = dict(interactions=True, r_a=1.0, contact_table=tab + tab.T, contact_range=6.0)
    else:
        extra = dict(beams=(pimc.lattice_angles("l25"), 0.6, -2.0, False))
    p = O.make_params(dim=2, N=10, M=16, L=4.0, T=0.5, lam=0.5, hcoef=0.5,
                      semantics=O.SEM_PHYSICAL, **extra)
    o = O.Oracle(p)
    x = rng.normal(scale=0.8, size=(2, 10, 16))
    nxt = rng.permutation(10).astype(np.int32)
    o.set_state(x, nxt)
    for _ in range(20):
        nn, j0, m = int(rng.integers(10)), int(rng.integers(16)), int(rng.integers(2, 10))
        x, _, nx = o.get_state()
        own = [nn if j0 + t < 16 else nx[nn] for t in range(m + 1)]
        sl = [(j0 + t) % 16 for t in range(m + 1)]
        rp = np.array([[x[0, own[t], sl[t]], x[1, own[t], sl[t]]] for t in range(m + 1)])
        rp[1:m] += rng.normal(scale=0.2, size=(m - 1, 2))
        wi, wu = o.staging_weights(nn, j0, m, rp.ravel())
        a0 = o.eval_action()
        x2 = x.copy()
        for t in range(1, m):
            x2[:, own[t], sl[t]] = rp[t]
        o2 = O.Oracle(p)
        o2.set_state(x2, nx)
        a1 = o2.eval_action()
        dS = (a1[1] + a1[2]) - (a0[1] + a0[2])
        assert abs((wu - wi) - dS) < 1e-11 * max(1.0, abs(dS)), (kind, wu - wi, dS)


def test_oracle_virial_matches_thermodynamic_with_the_lattice(oracle_mod):
    """one particle in an optical lattice plus a trap: the virial estimator,
    which uses the lattice's analytic gradient, and the thermodynamic one
    sample the same energy"""
    import pimc
    O = oracle_mod
    p = O.make_params(dim=2, N=1, M=16, L=6.0, T=1.0, lam=0.5, hcoef=0.5, semantics=O.SEM_PHYSICAL,
                      beams=(pimc.lattice_angles("cubic"), 0.5, -1.5, False))
    r = _run_energy(O, p, 30000, 8, 7)
    eth, s1 = blocking(r["energies"][:, 0])
    ev, s2 = blocking(r["energies"][:, 1])
    assert abs(eth - ev) < 3 * math.hypot(s1, s2), (eth, s1, ev, s2)


def test_oracle_init_world_hard_core(oracle_mod):
    """init_world's hard-core redraw (src/system.jl:44-64) in the oracle: no
    two beads of a slice closer than a, and ORC_ESTATE when the spheres do
    not fit"""
    O = oracle_mod
    o = O.Oracle(O.make_params(dim=2, N=20, M=8, L=3.0, T=1.0, lam=0.5, hardcore_a=0.5,
                               interactions=True, r_a=1.0))
    assert o.init_world(seed=3) == 0
    x, _, nxt = o.get_state()
    d = np.abs(x[:, :, None, :] - x[:, None, :, :])
    d = np.minimum(d, 6.0 - d)
    r = np.sqrt((d ** 2).sum(axis=0))
    r[np.arange(20), np.arange(20), :] = np.inf
    assert r.min() >= 0.5 and (nxt == np.arange(20)).all()
    o2 = O.Oracle(O.make_params(dim=2, N=40, M=8, L=1.0, T=1.0, lam=0.5, hardcore_a=0.5,
                                interactions=True, r_a=0.6))
    assert o2.init_world(seed=3) == -3
