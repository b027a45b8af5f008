"""Engine-side statistics of the benchmarked configurations, compared with
the oracle's committed statistics (tests/golden/sweep_stats.json).

Both sides use independent chains: every estimator's value is the mean over
chains of each chain's mean over its measured sweeps, and its standard error
the spread of those chain means / sqrt(chains).  The engine runs its chains as
one batch (pimc_batch_run: the persistent sweep kernels under a CUDA graph),
each chain with its own Philox seed, starting from the device's init_world.

Used by tests/test_gpu_sweep_parity.py and by bench.py's energy check.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from common import c4_sample, engine_mix

HERE = os.path.dirname(os.path.abspath(__file__))
STATS_PATH = os.path.join(HERE, "golden", "sweep_stats.json")


def load_stats():
    return json.load(open(STATS_PATH))


def load_density(name):
    d = np.load(os.path.join(HERE, "golden", f"density_{name}.npz"))
    return d["mean"], d["se"]


def run_replicas(eng_kw, ell, replicas, therm, sweeps, seed0, dens_nb=0, max_batch=4096):
    """replicas independent chains of one configuration on the device:
    per-chain means of the 4 energy columns (E_th, E_v, pair energy, pair
    virial) and, with dens_nb, per-chain density (counts / ndata)"""
    from pimc.engine import ChainParams, Engine
    means, dens = [], []
    for b0 in range(0, replicas, max_batch):
        nb = min(max_batch, replicas - b0)
        ps = [ChainParams(**eng_kw, seed=seed0 + b0 + r, density_nbins=dens_nb, energy_capacity=0)
              for r in range(nb)]
        e = Engine(ps)
        N, M, L = eng_kw["N"], eng_kw["M"], eng_kw["L"]
        e.set_mix(engine_mix(N, M, ell, L, measure_every=0))
        e.run_batched(therm)
        e.set_mix(engine_mix(N, M, ell, L, measure_every=1))
        e.reset_measurements()
        e.run_batched(sweeps)
        s, _, cnt = e.energy_sums_all()
        assert (cnt == sweeps).all(), cnt
        means.append(s / cnt[:, None])
        if dens_nb:
            for c in range(nb):
                h, nd = e.density(c)
                dens.append(h / nd)
        e.close()
    m = np.concatenate(means)
    return m, (np.array(dens) if dens_nb else None)


def summarise(m):
    """value and standard error of E_th, E_v, E_pair, E_th + E_pair from
    per-chain means m[chain][4]"""
    n = len(m)
    cols = {"E_th": m[:, 0], "E_v": m[:, 1], "E_pair": m[:, 2], "E_th_pair": m[:, 0] + m[:, 2]}
    return {k: (float(v.mean()), float(v.std(ddof=1) / math.sqrt(n))) for k, v in cols.items()}


def z(a, b):
    """z-score of two (value, standard error) pairs"""
    return (a[0] - b[0]) / math.hypot(a[1], b[1])


def density_compare(gpu_dens, orc_mean, orc_se, min_mean=None):
    """bin-by-bin comparison of per-chain densities with the oracle's: over the
    bins where the oracle's mean occupancy is at least min_mean (default: 2%
    of the largest bin), the z-scores, chi^2 per bin and the fraction within
    2 sigma"""
    g_mean = gpu_dens.mean(axis=0)
    g_se = gpu_dens.std(axis=0, ddof=1) / math.sqrt(len(gpu_dens))
    if min_mean is None:
        min_mean = 0.02 * orc_mean.max()
    sel = orc_mean >= min_mean
    zz = (g_mean[sel] - orc_mean[sel]) / np.hypot(g_se[sel], orc_se[sel])
    return {"bins": int(sel.sum()), "chi2_per_bin": float(np.mean(zz ** 2)),
            "within_2sigma": float(np.mean(np.abs(zz) < 2.0)), "max_abs_z": float(np.abs(zz).max()),
            "mean_z": float(zz.mean()),
            "total_rel_diff": float(abs(g_mean.sum() - orc_mean.sum()) / orc_mean.sum())}


def c4_energy_check(replicas=32, therm=1000, sweeps=4000, seed0=9100000, semantics=0):
    """the 24 sampled C4 chains (tests/common.py c4_sample), replicas each, in
    one batch of the engine against the oracle's committed per-chain
    statistics: under the reference's rules those of the engine's sweep
    schedule (the rules are not reversible, so the schedule matters), under the
    physical rules those of run!.  Per chain z of E_th + E_pair, and the
    summary."""
    from pimc.engine import ChainParams, Engine
    key = "c4_sample" if semantics == 0 else "c4_sample_phys"
    stats = load_stats()[key]
    by_index = {c["index"]: c for c in stats["chains"]}
    sample = c4_sample()
    ps, which = [], []
    for k, (idx, eng, _, ell) in enumerate(sample):
        for r in range(replicas):
            ps.append(ChainParams(**dict(eng, semantics=semantics), seed=seed0 + 1000 * k + r,
                                  energy_capacity=0))
            which.append(k)
    e = Engine(ps)
    for c, k in enumerate(which):
        idx, eng, _, ell = sample[k]
        e.set_mix(engine_mix(eng["N"], eng["M"], ell, eng["L"], measure_every=0), chain=c)
    e.run_batched(therm)
    for c, k in enumerate(which):
        idx, eng, _, ell = sample[k]
        e.set_mix(engine_mix(eng["N"], eng["M"], ell, eng["L"], measure_every=1), chain=c)
    e.reset_measurements()
    e.run_batched(sweeps)
    s, _, cnt = e.energy_sums_all()
    e.close()
    m = s / cnt[:, None]
    which = np.array(which)
    rows = []
    for k, (idx, eng, _, ell) in enumerate(sample):
        g = summarise(m[which == k])
        o = by_index[idx]
        rows.append({"index": idx, "N": eng["N"], "M": eng["M"], "engine": g["E_th_pair"],
                     "oracle": tuple(o["E_th_pair"]), "z": z(g["E_th_pair"], o["E_th_pair"])})
    zz = np.array([r["z"] for r in rows])
    summary = {"chains": len(rows), "replicas": replicas, "oracle_replicas": stats["replicas"],
               "therm": therm, "sweeps": sweeps, "quantity": "E_th + E_pair per chain",
               "semantics": "reference" if semantics == 0 else "physical",
               "oracle_schedule": "the engine's sweep" if stats["schedule"] == "sweep" else "run!",
               "within_2sigma": int(np.sum(np.abs(zz) < 2.0)), "max_abs_z": float(np.abs(zz).max()),
               "chi2_per_dof": float(np.mean(zz ** 2))}
    return summary, rows
