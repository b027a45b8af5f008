"""Chain state on the device: checkpoints that carry the pair-distance
histogram, the tuner's restore, and the device's own check of next[].

A snapshot (pimc_get_state) holds every chain's beads, links, next, counters,
estimator sums and histograms; restoring it reproduces the following sweeps
bit for bit, including g(r) and its measurement count.  A snapshot whose
next[] holds an out-of-range value is refused on the host; one whose next[]
is in range but not a permutation is caught by the sweep kernels, which flag
the chain (PIMC_EDEVICE) and leave it untouched while the others go on.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair_chain(seed, N=24, M=16, **kw):
    from pimc.engine import ChainParams
    base = dict(dim=2, N=N, M=M, L=4.0, T=0.5, lam=0.5, harmonic_omega=1.0, interactions=True,
                pair_g=1.0, pair_sigma=0.5, r_a=1.0, semantics=1, seed=seed, energy_capacity=32)
    base.update(kw)
    return ChainParams(**base)


def _mix(N, M, measure_every=1):
    from pimc.engine import Mix
    ell = min(8, M - 1)
    return Mix(stage_slices=ell, stage_max=ell, stage_minacc=0.0, stage_maxacc=1.0,
               swaps_per_sweep=N, swap_slices=ell, swap_max=ell, swap_minacc=0.0,
               swap_maxacc=1.0, com_step=1.0,
               com_maxstep=2.0, measure_every=measure_every)


def test_checkpoint_carries_the_radial_histogram():
    from pimc.engine import Engine
    e = Engine([_pair_chain(31)])
    e.set_mix(_mix(24, 16))
    e.set_radial(40, 3.0)
    e.run(5)
    blob = e.get_state()
    e.run(7)
    ha, na = e.radial()
    xa = e.get_beads()
    assert na == 12 and ha.sum() > 0
    e.set_state(blob)
    hb0, nb0 = e.radial()
    assert nb0 == 5 and hb0.sum() < ha.sum()
    e.run(7)
    hb, nb = e.radial()
    np.testing.assert_array_equal(hb, ha)
    assert nb == na
    np.testing.assert_array_equal(e.get_beads(), xa)
    # a snapshot restores only into a handle with the same radial bins
    e.set_radial(20, 3.0)
    from pimc import PimcError
    with pytest.raises(PimcError, match="pair-distance bins"):
        e.set_state(blob)
    e.close()


def test_tuner_leaves_the_radial_histogram_unchanged():
    from pimc.engine import Engine
    ps = [_pair_chain(40 + i, N=16 + 4 * i, M=16) for i in range(6)]
    e = Engine(ps)
    for i, p in enumerate(ps):
        e.set_mix(_mix(p.N, p.M, measure_every=2), chain=i)
    e.set_radial(32, 3.0)
    e.run_batched(4)
    before = [e.radial(c) for c in range(len(ps))]
    e.tune(sweeps_per_trial=1)
    for c in range(len(ps)):
        h, n = e.radial(c)
        np.testing.assert_array_equal(h, before[c][0])
        assert n == before[c][1]
    e.close()


def _next_offset(blob, nxt):
    """byte offset of a chain's next[] in a snapshot (found by its contents)"""
    pat = np.ascontiguousarray(nxt, dtype=np.int32).tobytes()
    off = blob.find(pat)
    assert off >= 0 and blob.find(pat, off + 1) < 0, "next[] not unique in the snapshot"
    return off


def test_device_flags_a_next_that_is_not_a_permutation():
    from pimc import PimcError
    from pimc.engine import Engine
    ps = [_pair_chain(50 + i, N=20, M=16) for i in range(3)]
    e = Engine(ps)
    for i, p in enumerate(ps):
        e.set_mix(_mix(p.N, p.M, measure_every=0), chain=i)
    e.run_batched(20)  # swaps permute the cycles
    nx = e.get_next(1)
    assert (nx != np.arange(20)).any()
    good = e.get_state()
    off = _next_offset(good, nx)
    # in range, not a permutation: the sweep kernels flag chain 1
    bad = bytearray(good)
    dup = nx.copy()
    dup[3] = dup[4]
    bad[off:off + 80] = dup.astype(np.int32).tobytes()
    e.set_state(bytes(bad))
    s0 = [e.stats(c).sweeps for c in range(3)]
    with pytest.raises(PimcError, match="not a permutation.*chain 1"):
        e.run_batched(2)
    s1 = [e.stats(c).sweeps for c in range(3)]
    assert s1[0] == s0[0] + 2 and s1[2] == s0[2] + 2 and s1[1] == s0[1]
    np.testing.assert_array_equal(e.get_next(1), dup)
    with pytest.raises(PimcError, match="not a permutation"):
        e.measure()
    # out of range: refused on the host, nothing written
    bad2 = bytearray(good)
    oor = nx.copy()
    oor[5] = 20 + 7
    bad2[off:off + 80] = oor.astype(np.int32).tobytes()
    with pytest.raises(PimcError, match="out of range"):
        e.set_state(bytes(bad2))
    np.testing.assert_array_equal(e.get_next(1), dup)
    # a good snapshot clears the flag
    e.set_state(good)
    e.run_batched(2)
    assert e.stats(1).sweeps == s0[1] + 2
    e.close()


def test_batch_bead_io_pinned_and_pageable():
    """pimc_batch_set_beads_all / get_beads_all: a page-locked host buffer is
    read and written by the GPU in place, a pageable one through the staging
    copy; both agree bit for bit with the per-chain calls, for chains whose
    sizes are not multiples of the 32 x 32 transpose tiles"""
    torch = pytest.importorskip("torch")
    from pimc.engine import Engine
    rng = np.random.default_rng(77)
    ps = [_pair_chain(90 + i, N=int(rng.integers(1, 100)), M=int(rng.choice([4, 16, 33, 70])),
                      interactions=False, dim=int(1 + i % 2)) for i in range(9)]
    e = Engine(ps)
    n = e.beads_all_size()
    for pinned in (True, False):
        src = rng.uniform(-3.9, 3.9, size=n)
        if pinned:
            t = torch.empty(n, dtype=torch.float64, pin_memory=True)
            buf = t.numpy()
            buf[:] = src
        else:
            buf = src.copy()
        e.set_beads_all(buf)
        o = 0
        for c, p in enumerate(ps):
            k = p.dim * p.N * p.M
            np.testing.assert_array_equal(e.get_beads(c).ravel(), src[o:o + k])
            o += k
        e.run_batched(2)
        want = np.concatenate([e.get_beads(c).ravel() for c in range(len(ps))])
        if pinned:
            out = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
            out[:] = np.nan
        else:
            out = np.full(n, np.nan)
        e.get_beads_all(out)
        np.testing.assert_array_equal(out, want)
    e.close()


def _min_same_slice_distance(x, L):
    """smallest norm of per-component minimum-image distances between two
    particles' beads at the same slice (x[d][n][j])"""
    d = np.abs(x[:, :, None, :] - x[:, None, :, :])
    d = np.minimum(d, 2 * L - d)
    r = np.sqrt((d ** 2).sum(axis=0))
    N = x.shape[1]
    r[np.arange(N), np.arange(N), :] = np.inf
    return r.min()


def test_init_world_hard_core():
    """init_world with a hard core (src/system.jl:44-64): no two beads of one
    slice closer than a; a density at which the spheres cannot be placed
    fails the System constructor with the reference's message"""
    from pimc import PimcError
    from pimc.engine import Engine
    ps = [_pair_chain(200 + i, N=20, M=8, L=3.0, hardcore_a=0.5, pair_g=0.0, r_a=1.0)
          for i in range(4)]
    e = Engine(ps)
    for c in range(4):
        assert _min_same_slice_distance(e.get_beads(c), 3.0) >= 0.5
    e.init_world()
    assert _min_same_slice_distance(e.get_beads(0), 3.0) >= 0.5
    e.close()
    with pytest.raises(PimcError, match="creating world of 40 particles with hardspheres"):
        Engine(_pair_chain(300, N=40, M=8, L=1.0, hardcore_a=0.5, pair_g=0.0, r_a=0.6))


def test_run_io_equals_set_run_get():
    """pimc_batch_run_io (upload, sweep and download in overlapped chunks of
    chains) leaves every chain as set_beads_all + run_batched + get_beads_all
    do, bit for bit, with pinned and pageable buffers, in place or not"""
    torch = pytest.importorskip("torch")
    from pimc.engine import Engine
    rng = np.random.default_rng(91)
    ps = [_pair_chain(400 + i, N=int(rng.integers(2, 90)), M=int(rng.choice([8, 16, 33])),
                      interactions=bool(i % 2), dim=int(1 + (i % 3 > 0))) for i in range(11)]

    def fresh():
        e = Engine(ps)
        for c, p in enumerate(ps):
            e.set_mix(_mix(p.N, p.M, measure_every=1), chain=c)
        return e

    a = fresh()
    n = a.beads_all_size()
    x0 = a.get_beads_all().copy()
    a.set_beads_all(x0)
    a.run_batched(3)
    want = a.get_beads_all()
    want_e = a.energy_sums_all()[0]
    want_next = [a.get_next(c) for c in range(len(ps))]
    a.close()
    for chunks, pinned, inplace in [(1, True, False), (3, True, True), (0, False, False),
                                    (11, False, True), (64, True, False)]:
        b = fresh()
        if pinned:
            xin = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
            xout = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        else:
            xin, xout = np.empty(n), np.empty(n)
        xin[:] = x0
        xout[:] = np.nan
        got = b.run_io(xin, 3, x_out=None if inplace else xout, chunks=chunks)
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(b.energy_sums_all()[0], want_e)
        for c in range(len(ps)):
            np.testing.assert_array_equal(b.get_next(c), want_next[c])
        assert b.last_run_ms() > 0
        b.close()
