"""Cell-list neighbour queries (the cell grid of src/nearest_neighbours.jl:
26-154) against the whole-slice scan.

Every sweep query takes its candidates either from the per-slice cell lists
(counting-sorted at the start of each phase that queries, moved beads tracked
on the side) or from a scan of the slice row; the neighbour sets are the
same, so the chains' moves are the same: the beads after a run agree bit for
bit, and the estimators (the same pair terms summed in another order) agree
to rounding.  A neighbour that a list missed would change pair sums by terms
of order exp(-r^2 / 2 sigma^2) and, over thousands of moves, decisions.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _chains(semantics, hard=0.0, dim=2, L=8.0, trap=1.0):
    from pimc.engine import ChainParams
    rng = np.random.default_rng(11 + semantics + int(10 * hard) + dim)
    ps = []
    for i in range(6):
        N = int(rng.choice([24, 60, 130, 257]))
        M = int(rng.choice([16, 24, 32]))
        ps.append(ChainParams(dim=dim, N=N, M=M, L=L, T=float(rng.uniform(0.3, 2.0)), lam=0.5,
                              harmonic_omega=trap, interactions=True,
                              pair_g=float(rng.uniform(0.2, 2.0)), pair_sigma=0.5, r_a=1.5,
                              hardcore_a=hard, semantics=semantics, seed=5000 + 17 * i,
                              energy_capacity=0, retry_cap=100 if hard > 0 else 0))
    return ps


def _mix(p, measure_every=1):
    from pimc.engine import Mix
    ell = min(16, p.M // 2)
    return Mix(stage_slices=ell, stage_max=ell, stage_minacc=0.0, stage_maxacc=1.0,
               swaps_per_sweep=p.N, swap_slices=ell, swap_max=ell, swap_minacc=0.0,
               swap_maxacc=1.0, com_step=1.0, com_maxstep=2.0, measure_every=measure_every,
               polymer_com_phases=1)


def _run(ps, mode, sweeps, batched=True):
    from pimc.engine import Engine
    e = Engine(ps)
    e.set_cells(mode)
    for c, p in enumerate(ps):
        e.set_mix(_mix(p), chain=c)
    if batched:
        e.run_batched(sweeps)
    else:
        e.run(sweeps)
    x = [e.get_beads(c) for c in range(len(ps))]
    nx = [e.get_next(c) for c in range(len(ps))]
    s, _, cnt = e.energy_sums_all()
    st = [e.stats(c) for c in range(len(ps))]
    e.close()
    return x, nx, s, cnt, st


@pytest.mark.parametrize("semantics,hard,dim,L,trap", [
    (0, 0.0, 2, 8.0, 1.0),     # the reference's rules: pairs in swaps and measurements
    (1, 0.0, 2, 8.0, 1.0),     # physical rules: pairs in every move
    # hard core: the redraw tests query the lists too (257 spheres of radius
    # 0.3 do not fit in this trap, so most redraws fail: a cap of 100 tries
    # instead of 10,000 keeps the run short and the failures frequent)
    (1, 0.3, 2, 8.0, 1.0),
    (0, 0.0, 2, 6.0, 0.0),     # free gas in a periodic box: cells across the wrap
    (1, 0.0, 1, 12.0, 0.5),    # one dimension: rows of cells
])
def test_cell_lists_match_row_scan(semantics, hard, dim, L, trap):
    ps = _chains(semantics, hard=hard, dim=dim, L=L, trap=trap)
    a = _run(ps, 2, 12)
    b = _run(ps, 0, 12)
    for c in range(len(ps)):
        np.testing.assert_array_equal(a[0][c], b[0][c])
        np.testing.assert_array_equal(a[1][c], b[1][c])
        assert a[4][c].accepts == b[4][c].accepts
    np.testing.assert_array_equal(a[3], b[3])
    np.testing.assert_allclose(a[2], b[2], rtol=1e-12, atol=1e-9)
    # the swaps did move beads, so the lists' moved-bead tracking was used
    assert all(st.accepts[1] > 0 for st in a[4])


def test_cell_lists_auto_and_plain_launches():
    """the crowding rule (mode 1) and the per-chain plain launches give the
    same chains as the scan"""
    ps = _chains(0)
    a = _run(ps, 1, 8, batched=False)
    b = _run(ps, 0, 8, batched=False)
    for c in range(len(ps)):
        np.testing.assert_array_equal(a[0][c], b[0][c])
    np.testing.assert_allclose(a[2], b[2], rtol=1e-12, atol=1e-9)
