"""CPU tests of the host-side logic: the run!-to-sweep mapping of the API
mirror, the synthetic workload definitions, and the multi-rank timing
reduction of bench.py over two gloo ranks."""
import json
import math
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class FakeSystem:
    """only the fields the mapping reads (no engine)"""

    def __init__(self, N, M, L=5.0):
        self.N, self.M, self.L = N, M, L


def test_survey_mix_maps_to_one_sweep():
    """[(1, Reshape(l)), (k, Swap(l)), (k, CoM)] with N(k+2) attempts is one
    sweep: N*k staging windows, N swaps, one CoM phase"""
    from pimc.api import ReshapeLinear, ReshapeSwapLinear, SingleCenterOfMass, _mix_for
    s = FakeSystem(N=64, M=32)
    ell = 16
    k = math.ceil(s.M / ell)
    ups = [(1, ReshapeLinear(s, ell, minacc=0.0, maxacc=1.0)),
           (k, ReshapeSwapLinear(s, ell, minacc=0.0, maxacc=1.0)),
           (k, SingleCenterOfMass(s, 1.0))]
    mix, sweeps, per_sweep, objs = _mix_for(s, 64 * (k + 2) * 10, ups)
    assert sweeps == 10
    assert per_sweep == 64 * (k + 2)
    assert mix.staging_phases == 1 and mix.stage_slices == ell
    assert mix.swaps_per_sweep == 64
    assert mix.com_phases == 1
    assert set(objs) == {"ReshapeLinear", "ReshapeSwapLinear", "SingleCenterOfMass"}


def test_update_defaults_follow_reference():
    from pimc.api import ReshapeLinear, SingleCenterOfMass
    s = FakeSystem(N=2, M=100, L=4.0)
    r = ReshapeLinear(s, 20)
    assert (r.var.m, r.var.minslices, r.var.maxslices, r.var.minacc, r.var.maxacc) == (20, 2, 98, 0.6, 0.8)
    c = SingleCenterOfMass(s, 3.0)
    assert (c.var.size, c.var.minstep, c.var.maxstep, c.var.minacc, c.var.maxacc) == (3.0, 0.1, 2.0, 0.4, 0.6)


def test_acceptance_and_adjust():
    from pimc.api import NumbOfSlices, Step, acceptance, adjust_
    assert math.isnan(acceptance([]))
    assert acceptance([1, 0, 1, 1]) == 0.75
    st = Step(1.0, 0.1, 2.0, 0.4, 0.6)
    adjust_(st, 0.1)
    assert st.size == 0.9
    adjust_(st, float("nan"))  # an empty queue leaves the step alone
    assert st.size == 0.9
    m = NumbOfSlices(5, 2, 6, 0.6, 0.8)
    adjust_(m, 0.9)
    adjust_(m, 0.9)
    assert m.m == 6


def test_potentials_are_callable_like_closures():
    from pimc.api import GaussianPair, Harmonic, SquareLattice, _potential_terms
    V = Harmonic(1.0) + SquareLattice(4.0, 1.0)
    r = np.array([0.25, -0.5])
    assert math.isclose(V(r), 0.5 * 0.3125 + 4.0 * (0.5 + 1.0))
    assert _potential_terms(V) == (1.0, 4.0, 1.0, None)
    gp = GaussianPair(1.0, 0.5)
    assert 0 < gp([0.1, 0.0], [0.2, 0.0], 0.05) < 1
    from pimc import PimcError
    with pytest.raises(PimcError):
        _potential_terms(lambda r: 0.0)


def test_c4_chain_list_is_the_committed_one():
    sys.path.insert(0, ROOT)
    import bench
    chains = bench.c4_chain_list()
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "c4_chains.json")))
    for k in ("N", "M", "beta", "g"):
        assert [c[k] for c in chains] == ref[k]
    N = np.array([c["N"] for c in chains])
    assert len(chains) == 4096 and N.min() >= 8 and N.max() <= 512


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    tmax, tsum = bench.reduce_max_sum(dist, 1.0 + rank, 10.0 * (rank + 1))
    bench.barrier(dist)
    out[rank] = (tmax, tsum)
    dist.destroy_process_group()


def test_multirank_reduction_gloo():
    """weak scaling: the job time is the max over ranks and the work the sum
    (bench.py on world_size 2, gloo, CPU)"""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == (2.0, 30.0) and out[1] == (2.0, 30.0)


def _shard_rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.join(ROOT, "pimc.jl_gb300"))
    import torch.distributed as dist

    from pimc.shard import chain_cost, gather_sums, shard_of
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "c4_chains.json")))
    chains = [dict(N=n, M=m, interactions=True) for n, m in zip(ref["N"], ref["M"])]
    mine = shard_of(chains, rank, world)
    # stand-in estimator sums of each chain this rank ran: a fixed function
    # of the global chain index, as an engine batch's energy_sums_all rows
    rows = np.array([[i, i * i, np.sin(i), 1.0] for i in mine])
    cnt = np.array([10 + i % 7 for i in mine])
    full, fc = gather_sums(dist, mine, rows, cnt, len(chains))
    load = sum(chain_cost(chains[i]) for i in mine)
    out[rank] = (list(mine), full.tolist(), fc.tolist(), load)
    dist.destroy_process_group()


def test_chain_shards_and_gather_gloo():
    """the batched C4 chains split across 2 ranks by LPT: the shards are
    disjoint and cover all 4096 committed chains, their loads agree within
    0.1%, and the estimator sums gathered from both ranks equal a one-rank
    run's (gloo, world_size 2, CPU)"""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from pimc.shard import gather_sums
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_shard_rank_main, args=(2, port, out), nprocs=2, join=True)
    a, b = out[0], out[1]
    assert not set(a[0]) & set(b[0]) and sorted(a[0] + b[0]) == list(range(4096))
    assert abs(a[3] - b[3]) / (a[3] + b[3]) < 1e-3
    allr = list(range(4096))
    rows = np.array([[i, i * i, np.sin(i), 1.0] for i in allr])
    one, oc = gather_sums(None, allr, rows, np.array([10 + i % 7 for i in allr]), 4096)
    for r in (a, b):
        np.testing.assert_array_equal(np.array(r[1]), one)
        np.testing.assert_array_equal(np.array(r[2]), oc)


def test_lpt_partition_edge_cases():
    from pimc.shard import lpt_partition
    s, loads = lpt_partition([], 3)
    assert s == [[], [], []] and loads == [0.0, 0.0, 0.0]
    s, loads = lpt_partition([5.0, 1.0, 1.0, 1.0, 1.0, 1.0], 2)
    assert s == [[0], [1, 2, 3, 4, 5]] and loads == [5.0, 5.0]
    s, _ = lpt_partition([1.0] * 5, 8)
    assert sorted(sum(s, [])) == list(range(5)) and sum(1 for x in s if x) == 5
    with pytest.raises(ValueError):
        lpt_partition([1.0], 0)


def test_radial_and_superfluid_host_formulas():
    """the host side of the new estimators: g(r) of the ideal-gas counts is 1,
    and the superfluid fractions follow their published formulas"""
    from types import SimpleNamespace

    import numpy as np

    import pimc
    s = SimpleNamespace(L=4.0, dim=2, M=8, N=10, λ=0.5, β=2.0)
    rd = pimc.RadialDistribution(s, nbins=16)
    e = np.arange(17) * (s.L / 16)
    rd.ndata = 5
    rd.hist = 5 * s.M * s.N * (s.N - 1) / 2 * np.pi * np.diff(e ** 2) / (2 * s.L) ** 2
    np.testing.assert_allclose(rd.g(), 1.0, rtol=1e-12)
    np.testing.assert_allclose(rd.r(), (np.arange(16) + 0.5) * s.L / 16)
    sf = pimc.Superfluid(s)
    rows = np.zeros((4, 8))
    rows[:, 4] = [4.0, 0.0, 16.0, 4.0]      # W^2
    rows[:, 5] = [0.1, -0.2, 0.3, 0.0]      # A_z
    rows[:, 6] = [2.0, 2.5, 1.5, 2.0]       # sum r^2 / M
    sf._add(SimpleNamespace(N=10), rows)
    assert abs(sf.winding_fraction(10) - 6.0 / (2 * 2 * 0.5 * 2.0 * 10)) < 1e-15
    a2 = np.mean(np.array([0.1, -0.2, 0.3, 0.0]) ** 2)
    assert abs(sf.area_fraction(10) - 2 * a2 / (0.5 * 2.0 * 2.0)) < 1e-15


def test_generate_V_forms():
    """generate_V(scale, depth, sym; attractive) flips the depth's sign for an
    attractive lattice and names the reference's beam sets; the angle-list
    form keeps its depth; :harmonic is the unit trap"""
    import math

    import numpy as np

    import pimc
    V = pimc.generate_V(0.5, 3.0, "l25")
    assert isinstance(V, pimc.OpticalLattice) and V.depth == -3.0 and len(V.angles) == 12
    assert pimc.generate_V(0.5, 3.0, "l65", attractive=False).depth == 3.0
    assert isinstance(pimc.generate_V(1.0, 1.0, "harmonic"), pimc.Harmonic)
    W = pimc.generate_V([0.0, math.pi / 2], 1.0, 2.0, helical=True)
    assert W.helical and W.depth == 2.0
    # at the origin every plane wave has phase 0 (plus its own angle when helical)
    assert abs(V(np.zeros(2)) - (-3.0)) < 1e-15
    c = np.mean(np.cos([0.0, math.pi / 2])); s_ = np.mean(np.sin([0.0, math.pi / 2]))
    assert abs(W(np.zeros(2)) - 2.0 * (c * c + s_ * s_)) < 1e-15


def test_tune_cache_round_trip(tmp_path):
    """the tuner's cache of launch shapes (pimc/tuning.py): the signature
    follows the batch's mix of chain shapes, the device and the ABI version,
    not the chains' order or seeds; a stored shape comes back as stored"""
    from pimc.tuning import TuneCache, batch_signature, n_bucket
    ref = json.load(open(os.path.join(ROOT, "tests", "golden", "c4_chains.json")))
    chains = [dict(N=n, M=m, interactions=True, semantics=0) for n, m in zip(ref["N"], ref["M"])]
    sig = batch_signature(chains, "NVIDIA GB300", 3)
    assert sig == batch_signature(list(reversed(chains)), "NVIDIA GB300", 3)
    assert sig != batch_signature(chains, "NVIDIA B200", 3)
    assert sig != batch_signature(chains, "NVIDIA GB300", 2)
    assert sig != batch_signature(chains[:-1], "NVIDIA GB300", 3)
    assert [n_bucket(n) for n in (8, 15, 16, 300, 512)] == [8, 8, 16, 256, 512]
    path = str(tmp_path / "tune.json")
    shape = dict(warp_per_chain=False, block=64, sweeps_per_launch=1, state_smem_bytes=0,
                 split_phases=1, phase_block=[128, 64, 128], phase_warp=[0, 1, 0],
                 phase_regs=[0, 0, 0], cell_lists=1)
    tc = TuneCache(path)
    assert tc.get(sig) is None
    tc.put(sig, shape, ms_per_sweep=35.7)
    again = TuneCache(path)
    assert again.get(sig) == shape
    assert json.load(open(path))[sig]["ms_per_sweep"] == 35.7
    # an entry missing a key (an older file) is a miss, not an error
    again.data[sig].pop("phase_warp")
    assert again.get(sig) is None
    again.put(sig, shape)
    again.data[sig].pop("cell_lists")
    assert again.get(sig) is None
