"""Oracle statistics of the benchmarked configurations.

Runs the oracle (oracle/pimc_oracle.c, the C restatement of the reference's
moves) on independent chains of C1 (2D trapped ideal bosons, N=10, beta=1,
M=20), C2 (2D free bosons in the periodic box [-10, 10)^2, N=64, beta=2,
M=32), C3 (2D trapped bosons with the Gaussian pair g=1, sigma=0.5, N=256,
beta=2, M=64) and a sample of 24 chains of the batched C4 list, in one of two
schedules of the same moves:

* "run": the reference's run! (src/simulation.jl:29-42), attempts chosen at
  random with weights 1/every, with the survey's mapping of a sweep onto
  N(k+2) attempts (N k staging, N swaps, N centre of mass);
* "sweep": the engine's sweep (orc_run_sweeps): a staging phase of one window
  per (slot, particle), N swaps, one centre-of-mass attempt per single path,
  a measurement at the end of the sweep.

Under the physical rules both schedules sample the same distribution and the
engine is held to run!.  The reference's own rules are not reversible (the
swap leaves out its partner-choice ratio and puts the new paths' pair terms
into w_initial), so what they sample depends on the schedule: the engine is
held to the "sweep" schedule under those rules, and the "run" numbers are
kept as the record of the difference.

Each chain starts from the oracle's init_world, is thermalised, then measured
once per sweep.  Per chain the mean of every estimator column is kept; the
configuration's value is the mean over chains and its standard error the
spread of the chain means / sqrt(chains), which needs no autocorrelation model
because the chains are independent.  Densities are kept per bin the same way
(counts / ndata per chain).

Writes tests/golden/sweep_stats.json and tests/golden/density_<name>.npz; an
entry already in the file is kept unless --only names it.  The GPU tests
(tests/test_gpu_sweep_parity.py) and bench.py's energy check compare the
engine's sweeps against these numbers.

    python tests/golden/make_sweep_stats.py [--only c1_ref,c4_sample] [--threads 8]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from common import c4_sample, oracle_updates, sweep_configs  # noqa: E402
from oracle import oracle as O  # noqa: E402

# name: (configuration, schedule, chains, thermalisation sweeps, measured sweeps)
PLAN = {
    "c1_ref": ("c1_ref", "sweep", 64, 2000, 20000),
    "c1_ref_run": ("c1_ref", "run", 64, 2000, 20000),
    "c1_phys": ("c1_phys", "run", 64, 2000, 20000),
    "c2_ref": ("c2_ref", "sweep", 64, 1000, 10000),
    "c2_ref_run": ("c2_ref", "run", 64, 1000, 10000),
    "c2_phys": ("c2_phys", "run", 64, 1000, 10000),
    # the reference's rules give C3 heavy-tailed chain means (a chain's
    # cloud can spread far past the others for much of its run): 256 chains
    "c3_ref": ("c3_ref", "sweep", 256, 300, 1200),
    "c3_ref_run": ("c3_ref", "run", 32, 300, 1200),
}
# C4 sample: name -> (schedule, semantics); replicas, thermalisation, measured
C4_PLAN = {"c4_sample": ("sweep", 0), "c4_sample_run": ("run", 0), "c4_sample_phys": ("run", 1)}
C4_REPLICAS, C4_THERM, C4_SWEEPS = 16, 1000, 4000


def run_chain(orc_kw, ell, dens_nb, therm, sweeps, seed, schedule="run"):
    """one oracle chain: init_world, therm sweeps, then sweeps measured sweeps"""
    p = O.make_params(**orc_kw)
    o = O.Oracle(p)
    o.init_world(seed=seed, stream=1)
    N, M, L = orc_kw["N"], orc_kw["M"], orc_kw["L"]
    if schedule == "run":
        ups, per = oracle_updates(N, M, ell, L)
        o.run(therm * per, ups, seed=seed, stream=2)
        r = o.run(sweeps * per, ups, seed=seed, stream=3, ncycle=per, e_cap=sweeps + 1,
                  dens_nb=dens_nb)
    else:
        com = [1.0, 0.1, L / 2, 0.4, 0.6]
        O.run_sweeps(o, therm, ell, N, com, seed=seed, stream=2)
        r = O.run_sweeps(o, sweeps, ell, N, com, seed=seed, stream=3, measure_every=1,
                         e_cap=sweeps, dens_nb=dens_nb)
    assert r["rc"] == 0, r["rc"]
    E = r["energies"]
    assert len(E) == sweeps, (len(E), sweeps)
    out = {"mean": E.mean(axis=0)}
    if dens_nb:
        out["dens"] = r["hist"] / r["ndata"]
    return out


def summarise(chains):
    m = np.array([c["mean"] for c in chains])
    n = len(chains)
    cols = {"E_th": m[:, 0], "E_v": m[:, 1], "E_pair": m[:, 2], "E_th_pair": m[:, 0] + m[:, 2]}
    return {k: [float(v.mean()), float(v.std(ddof=1) / np.sqrt(n))] for k, v in cols.items()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default="")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    only = set(filter(None, args.only.split(",")))
    O.build()
    path = os.path.join(HERE, "sweep_stats.json")
    stats = json.load(open(path)) if os.path.exists(path) else {}
    stats["_about"] = ("oracle statistics in the run! schedule or the engine's sweep schedule "
                       "(mean over independent chains, standard error from the spread of chain "
                       "means); made by tests/golden/make_sweep_stats.py")
    jobs = []  # (cost, key, arguments)
    cfgs = sweep_configs()
    for name, (cfg, sched, nch, therm, sweeps) in PLAN.items():
        if only and name not in only:
            continue
        c = cfgs[cfg]
        cost = c["orc"]["N"] ** 2 * c["orc"]["M"] * (therm + sweeps) * (8 if c["orc"]["interactions"] else 1)
        for k in range(nch):
            jobs.append((cost, (name, k), (c["orc"], c["ell"], c["dens_nb"], therm, sweeps,
                                           100000 * (1 + list(PLAN).index(name)) + k, sched)))
    sample = c4_sample()
    for name, (sched, sem) in C4_PLAN.items():
        if only and name not in only:
            continue
        for idx, _, orc, ell in sample:
            orc = dict(orc, semantics=sem)
            cost = orc["N"] ** 2 * orc["M"] * (C4_THERM + C4_SWEEPS) * 8
            for r in range(C4_REPLICAS):
                jobs.append((cost, (name, idx, r), (orc, ell, 0, C4_THERM, C4_SWEEPS,
                                                    7000000 + 100 * idx + r, sched)))
    jobs.sort(key=lambda j: -j[0])
    t0 = time.time()
    res = {}
    with cf.ThreadPoolExecutor(max_workers=args.threads) as ex:
        futs = {ex.submit(run_chain, *j[2]): j[1] for j in jobs}
        for f in cf.as_completed(futs):
            res[futs[f]] = f.result()
    print(f"{len(jobs)} chains in {time.time() - t0:.0f} s", flush=True)
    for name, (cfg, sched, nch, therm, sweeps) in PLAN.items():
        if only and name not in only:
            continue
        chains = [res[(name, k)] for k in range(nch)]
        c = cfgs[cfg]
        entry = {"orc": c["orc"], "ell": c["ell"], "chains": nch, "therm": therm,
                 "sweeps": sweeps, "schedule": sched}
        entry.update(summarise(chains))
        if c["dens_nb"]:
            d = np.array([ch["dens"] for ch in chains])
            fn = f"density_{name}.npz"
            np.savez_compressed(os.path.join(HERE, fn), mean=d.mean(axis=0).astype(np.float64),
                                se=(d.std(axis=0, ddof=1) / np.sqrt(nch)).astype(np.float64))
            entry["density"] = fn
            entry["dens_nb"] = c["dens_nb"]
        stats[name] = entry
    for name, (sched, sem) in C4_PLAN.items():
        if only and name not in only:
            continue
        per = []
        for idx, _, orc, ell in sample:
            s = summarise([res[(name, idx, r)] for r in range(C4_REPLICAS)])
            per.append({"index": idx, "N": orc["N"], "M": orc["M"], "beta": 1.0 / orc["T"],
                        "g": orc["pair_g"], **s})
        stats[name] = {"replicas": C4_REPLICAS, "therm": C4_THERM, "sweeps": C4_SWEEPS,
                       "schedule": sched, "semantics": sem, "chains": per}
    with open(path, "w") as f:
        json.dump(stats, f, indent=1, sort_keys=True)
    print("wrote", path)


if __name__ == "__main__":
    main()
