"""Shared configurations and helpers of the test-suite."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def blocking(x, nblocks=32):
    """mean and standard error from nblocks contiguous blocks"""
    x = np.asarray(x, dtype=float)
    n = (len(x) // nblocks) * nblocks
    b = x[:n].reshape(nblocks, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nblocks))


# (name, engine kwargs, oracle kwargs): the same chain in both conventions
def c1_small(sem=0, N=10, M=20):
    eng = dict(dim=2, N=N, M=M, L=5.0, T=1.0, lam=0.5, harmonic_omega=1.0, semantics=sem)
    orc = dict(dim=2, N=N, M=M, L=5.0, T=1.0, lam=0.5, hcoef=0.5, semantics=sem)
    return eng, orc


def pair_small(sem=0, N=16, M=16, L=4.0, hard=0.0, lattice=0.0):
    eng = dict(dim=2, N=N, M=M, L=L, T=0.5, lam=0.5, harmonic_omega=1.0, interactions=True,
               pair_g=1.0, pair_sigma=0.5, r_a=1.0, semantics=sem, hardcore_a=hard,
               lattice_V0=lattice, lattice_a=1.0)
    orc = dict(dim=2, N=N, M=M, L=L, T=0.5, lam=0.5, hcoef=0.5, interactions=True, pair_g=1.0,
               pair_sigma=0.5, r_a=1.0, semantics=sem, hardcore_a=hard, V0=lattice, lat_a=1.0)
    return eng, orc


def free_small(sem=0, N=8, M=12, L=3.0):
    eng = dict(dim=2, N=N, M=M, L=L, T=0.5, lam=0.5, semantics=sem)
    orc = dict(dim=2, N=N, M=M, L=L, T=0.5, lam=0.5, semantics=sem)
    return eng, orc


def random_config(rng, dim, N, M, L, spread=1.0, perm=True):
    x = rng.normal(scale=spread, size=(dim, N, M))
    x = np.clip(x, -L * 0.999, L * 0.999)
    nxt = rng.permutation(N).astype(np.int32) if perm else np.arange(N, dtype=np.int32)
    return x, nxt


# ---------------------------------------------------------------------------
# the benchmarked configurations as statistical parity cases.  One sweep is
# the survey's run! mapping: N k staging attempts (k = ceil(M / l)), N swaps
# and N centre-of-mass attempts, window lengths frozen at l (minacc 0,
# maxacc 1), one measurement per sweep.  tests/golden/make_sweep_stats.py
# runs the oracle's run! on these and commits the statistics.
# ---------------------------------------------------------------------------
def _cfg(dim=2, N=10, M=20, L=5.0, T=1.0, lam=0.5, omega=0.0, pair_g=0.0, sigma=0.5, r_a=0.0,
         sem=0):
    inter = pair_g > 0.0
    eng = dict(dim=dim, N=N, M=M, L=L, T=T, lam=lam, harmonic_omega=omega, interactions=inter,
               pair_g=pair_g, pair_sigma=sigma, r_a=r_a, semantics=sem)
    orc = dict(dim=dim, N=N, M=M, L=L, T=T, lam=lam, hcoef=0.5 * omega * omega,
               interactions=inter, pair_g=pair_g, pair_sigma=sigma, r_a=r_a, semantics=sem)
    return eng, orc


def sweep_configs():
    """name -> dict(eng, orc, ell, dens_nb): C1 (2D trapped ideal bosons),
    C2 (2D free bosons, periodic box [-10, 10)^2) in both acceptance
    semantics, C3 (trapped bosons with the Gaussian pair, reference rules)"""
    out = {}
    for sem, tag in ((0, "ref"), (1, "phys")):
        eng, orc = _cfg(N=10, M=20, L=5.0, T=1.0, omega=1.0, sem=sem)
        out[f"c1_{tag}"] = dict(eng=eng, orc=orc, ell=8, dens_nb=64)
        eng, orc = _cfg(N=64, M=32, L=10.0, T=0.5, sem=sem)
        out[f"c2_{tag}"] = dict(eng=eng, orc=orc, ell=16, dens_nb=0)
    eng, orc = _cfg(N=256, M=64, L=8.0, T=0.5, omega=1.0, pair_g=1.0, sigma=0.5, r_a=1.5, sem=0)
    out["c3_ref"] = dict(eng=eng, orc=orc, ell=16, dens_nb=128)
    return out


def c4_sample(count=24):
    """the first `count` chains of the committed C4 list with N <= 48 and
    M <= 32 (small enough for the oracle), as (index, eng, orc, ell) with
    the bench's parameters: L = 8, omega = 1, Gaussian pair sigma = 0.5,
    r_a = 1.5, reference rules, l = min(16, M / 2)"""
    ref = json.load(open(os.path.join(HERE, "golden", "c4_chains.json")))
    out = []
    for i in range(len(ref["N"])):
        N, M = int(ref["N"][i]), int(ref["M"][i])
        if N > 48 or M > 32:
            continue
        eng, orc = _cfg(N=N, M=M, L=8.0, T=1.0 / float(ref["beta"][i]), omega=1.0,
                        pair_g=float(ref["g"][i]), sigma=0.5, r_a=1.5, sem=0)
        # a chain drawn with g = 0 still carries the pair machinery in C4
        eng["interactions"] = orc["interactions"] = True
        out.append((i, eng, orc, min(16, M // 2)))
        if len(out) == count:
            break
    return out


def oracle_updates(N, M, ell, L):
    """run!'s update list for one sweep and the attempts it takes (N(k+2))"""
    k = -(-M // ell)
    ups = [(0, 1, ell, 2, ell, 0.0, 1.0, 10, 10000), (1, k, ell, 2, ell, 0.0, 1.0, 10, 10000),
           (2, k, 1.0, 0.1, L / 2, 0.4, 0.6, 10, 10000)]
    return ups, N * (k + 2)


def engine_mix(N, M, ell, L, measure_every=1):
    """the same sweep for the engine (pimc_move_mix)"""
    from pimc.engine import Mix
    return Mix(stage_slices=ell, stage_min=2, stage_max=ell, stage_minacc=0.0, stage_maxacc=1.0,
               swaps_per_sweep=N if N > 1 else 0, swap_slices=ell, swap_min=2, swap_max=ell,
               swap_minacc=0.0, swap_maxacc=1.0, com_phases=1, com_step=1.0, com_minstep=0.1,
               com_maxstep=L / 2, adapt=1, measure_every=measure_every)


def zscore(a, sa, b, sb):
    return (a - b) / np.hypot(sa, sb)
