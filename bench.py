"""Benchmark of the GB300 PIMC sweep engine (bead-updates per second).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c4|c1|c2|c3|c5]
                    [--impl ours|reference]

A step is one sweep (every particle's staging windows, N permutation swaps,
one centre-of-mass phase) of every chain of the workload; a bead-update is
one proposed bead position (staging m-1, swap 2(m-1), centre of mass M per
attempt).  Default workload: 4096 independent trapped-gas chains of uneven
size (N in [8, 512], M in {16, 32, 64, 128}, beta in [0.5, 4], Gaussian pair
g in [0, 2], sigma 0.5, trap omega 1; seeds per chain), run by the persistent
batched kernel under a CUDA graph.  The JSON line adds the plain per-chain
launch path on the same chains, the CPU oracle on the machine's host cores, the
end-to-end rate through host buffers, the roofline of the sweep kernel and
the SM clocks seen during the timed region.

--impl reference times the CPU restatement of the reference's own sweep
(reference semantics, run!-style random move selection, one chain per host
thread) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "pimc.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = ("bead-updates/sec/GB300: batched+adjoint vs plain GPU vs CPU, at E within 2σ "
          "of reference")
UNIT = "bead-updates/s"
SEED = 20261203


# --------------------------------------------------------------------- workloads
PLAIN_STRIDE = 16
# the contact workload's propagator: build_prop_int(12, 1.16, tau)
CONTACT_G0, CONTACT_RANGE = 1.16, 12.0
# per bead update of k_sweep on the first 1216 C4 chains (block 128, ncu
# --set full), by acceptance semantics: DRAM bytes (dram__bytes_read.sum +
# dram__bytes_write.sum) and FP64 flops (dadd + dmul + 2 dfma thread
# instructions) over the launch's bead updates
PER_BEAD = {
    # fused sweep kernel (one launch per sweep)
    ("c4", "physical", "k_sweep"): {"dram_bytes": 188.4, "fp64_flops": 1017.0},   # 3.52 GB, 19.0 G / 18.70 M
    ("c4", "reference", "k_sweep"): {"dram_bytes": 269.7, "fp64_flops": 204.0},   # 4.82 GB, 3.65 G / 17.87 M
    # the swap launch of the split sweep, the kernel compiled for the
    # reference's rules alone, row scans (its bead updates are the swaps'
    # 2(m-1) per attempt; every attempt also reads the N heat-bath candidates)
    ("c4", "reference", "k_sweep_swap_ref"): {"dram_bytes": 1036.0, "fp64_flops": 330.0},  # 3.15 GB, 1.00 G / 3.037 M
}
ROOF_SWEEPS = 2  # sweeps of the per-phase timing pass


def c4_chain_list(n=4096):
    """4096 trapped-gas chains drawn from numpy default_rng(4096)"""
    rng = np.random.default_rng(4096)
    N = rng.integers(8, 513, size=n)
    M = rng.choice([16, 32, 64, 128], size=n)
    beta = rng.uniform(0.5, 4.0, size=n)
    g = rng.uniform(0.0, 2.0, size=n)
    return [dict(N=int(N[i]), M=int(M[i]), beta=float(beta[i]), g=float(g[i])) for i in range(n)]


def workload(name, semantics):
    """(chain params list, mix list, description) of a named workload"""
    from pimc.engine import ChainParams, Mix
    chains, mixes = [], []

    def mix_for(N, M, ell, L, measure_every):
        return Mix(stage_slices=ell, stage_min=2, stage_max=ell, stage_minacc=0.0, stage_maxacc=1.0,
                   swaps_per_sweep=N if N > 1 else 0, swap_slices=ell, swap_min=2, swap_max=ell,
                   swap_minacc=0.0, swap_maxacc=1.0, com_phases=1, com_step=1.0, com_minstep=0.1,
                   com_maxstep=L / 2, adapt=1, measure_every=measure_every)

    if name == "c4":
        for i, c in enumerate(c4_chain_list()):
            ell = min(16, c["M"] // 2)
            chains.append(ChainParams(dim=2, N=c["N"], M=c["M"], L=8.0, T=1.0 / c["beta"], lam=0.5,
                                      harmonic_omega=1.0, interactions=True, pair_g=c["g"],
                                      pair_sigma=0.5, r_a=1.5, semantics=semantics, seed=SEED + i,
                                      energy_capacity=0))
            mixes.append(mix_for(c["N"], c["M"], ell, 8.0, 10))
        desc = ("C4 batched: 4096 trapped-gas chains, N~U{8..512}, M~U{16,32,64,128}, "
                "beta~U[0.5,4], Gaussian pair g~U[0,2] sigma=0.5 (cutoff 3 sigma, cell 1.6), "
                "omega=1, L=8, staging l=min(16,M/2), N swaps + 1 CoM phase per sweep")
    elif name == "c1":
        chains.append(ChainParams(dim=2, N=10, M=20, L=5.0, T=1.0, lam=0.5, harmonic_omega=1.0,
                                  semantics=semantics, seed=SEED, density_nbins=64,
                                  energy_capacity=0))
        mixes.append(mix_for(10, 20, 8, 5.0, 1))
        desc = "C1 plain: 2D trapped ideal bosons N=10, beta=1, M=20, l=8, 64x64 density"
    elif name == "c2":
        chains.append(ChainParams(dim=2, N=64, M=32, L=10.0, T=0.5, lam=0.5, semantics=semantics,
                                  seed=SEED, energy_capacity=0))
        mixes.append(mix_for(64, 32, 16, 10.0, 1))
        desc = "C2 plain: 2D free bosons N=64, beta=2, M=32, periodic [-10,10)^2, l=16"
    elif name == "c3":
        chains.append(ChainParams(dim=2, N=256, M=64, L=8.0, T=0.5, lam=0.5, harmonic_omega=1.0,
                                  interactions=True, pair_g=1.0, pair_sigma=0.5, r_a=1.5,
                                  semantics=semantics, seed=SEED, density_nbins=128,
                                  energy_capacity=0))
        mixes.append(mix_for(256, 64, 16, 8.0, 1))
        desc = "C3 plain: 2D trapped bosons, Gaussian pair g=1 sigma=0.5, N=256, beta=2, M=64"
    elif name == "contact":
        # the C4 list's particle numbers at one temperature and slice count, so
        # that every chain shares one contact table (tau = 1/32)
        for i, c in enumerate(c4_chain_list()[:1024]):
            chains.append(ChainParams(dim=2, N=c["N"], M=64, L=8.0, T=0.5, lam=0.5,
                                      harmonic_omega=1.0, interactions=True, r_a=1.5,
                                      semantics=semantics, seed=SEED + i, energy_capacity=0))
            mixes.append(mix_for(c["N"], 64, 16, 8.0, 10))
        desc = ("contact: 1024 trapped-gas chains, N~U{8..512} (the C4 list), M=64, beta=2, "
                "tabulated contact propagator g0=1.16 (600x600 table over [1e-20, 12], built on "
                "the device), omega=1, L=8, cell 1.6, staging l=16, N swaps + 1 CoM phase")
    elif name == "c5":
        chains.append(ChainParams(dim=2, N=1024, M=64, L=16.0, T=0.25, lam=0.5, harmonic_omega=0.1,
                                  lattice_V0=4.0, lattice_a=1.0, interactions=True, pair_g=1.0,
                                  pair_sigma=0.3, r_a=0.9, semantics=semantics, seed=SEED,
                                  energy_capacity=0))
        mixes.append(mix_for(1024, 64, 16, 16.0, 1))
        desc = ("C5 plain + adjoint: lattice V0=4 a=1 + trap omega=0.1 + Gaussian pair g=1 "
                "sigma=0.3, N=1024, beta=4, M=64")
    else:
        raise SystemExit(f"unknown workload {name}")
    return chains, mixes, desc


# --------------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons while running"""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return ws, rank, local, pg


def reduce_max_sum(pg, tmax, tsum):
    """max of elapsed time and sum of work over ranks (host scalars)"""
    if pg is None:
        return tmax, tsum
    import torch
    dev = "cuda" if torch.cuda.is_available() and pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([tmax], dtype=torch.float64, device=dev)
    s = torch.tensor([tsum], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    pg.all_reduce(s, op=pg.ReduceOp.SUM)
    return float(t.item()), float(s.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def pinned_empty(n):
    """page-locked host buffer (torch only allocates it; numpy views it)"""
    try:
        import torch
        t = torch.empty(n, dtype=torch.float64, pin_memory=True)
        return t.numpy(), t
    except Exception:
        return np.empty(n), None


# --------------------------------------------------------------------- CPU legs
def cpu_oracle_rate(chains, mixes, semantics, budget_s=15.0, max_chains=None, threads=None,
                    contact=None):
    """the CPU oracle (C restatement of the reference's sweep) on a bounded
    sample of the workload's chains: the sampled chains dealt longest-first to
    the host threads, every thread sweeping its own chains in turn (run!
    attempts, N(k+2) per sweep) until budget_s of wall time has passed, so no
    core idles while another finishes; contact = (table, range) gives every
    chain the tabulated contact propagator"""
    from oracle import oracle as O
    O.build()
    threads = threads or os.cpu_count() or 1
    n = len(chains)
    take = max_chains or min(n, 8 * threads)
    idx = np.linspace(0, n - 1, take).astype(int) if n > take else np.arange(n)
    ps, ells = [], []
    for i in idx:
        c, m = chains[i], mixes[i]
        ps.append(O.make_params(dim=c.dim, N=c.N, M=c.M, L=c.L, T=c.T, lam=c.lam,
                                hcoef=0.5 * c.harmonic_omega ** 2, V0=c.lattice_V0,
                                lat_a=c.lattice_a, pair_g=c.pair_g, pair_sigma=c.pair_sigma,
                                interactions=c.interactions, r_a=c.r_a, semantics=semantics,
                                mu=c.mu, contact_table=None if contact is None else contact[0],
                                contact_range=0.0 if contact is None else contact[1]))
        ells.append(m.stage_slices)
    wall, beads, sweeps = O.bench_budget(ps, ells, threads, budget_s, 1.0, SEED)
    sample = (f"{len(idx)} of {n} chains (evenly spaced), dealt longest-first to {threads} host "
              f"threads, each thread sweeping its own chains in turn for {wall:.1f} s of wall "
              f"time ({sweeps:.0f} sweeps of N(k+2) run! attempts in all)")
    return beads / wall, threads, sample


def cpu_contact_table_rate(g0, chain, range_, budget_s=4.0):
    """entries per second of the contact table by adaptive quadrature of the
    reference's integrals on one host core (oracle/contact_table.py), on a
    bounded sample of entries spread over the table"""
    from oracle import contact_table as CT
    tau = 1.0 / (chain.T * chain.M)
    r = CT.grid(range_, 600)
    rng = np.random.default_rng(SEED)
    t0 = time.perf_counter()
    done = 0
    while time.perf_counter() - t0 < budget_s and done < 400:
        i1, i2 = (int(v) for v in rng.integers(0, 600, size=2))
        CT.entry(float(r[i1]), float(r[i2]), g0, tau)
        done += 1
    wall = time.perf_counter() - t0
    rate = done / wall
    return {"entries_per_s": rate, "cores": 1, "kind": "port",
            "full_table_s_estimate": 600 * 601 / 2 / rate,
            "sample": f"{done} random entries in {wall:.1f} s, scipy QUADPACK on the "
                      "reference's integrand (the reference uses QuadGK)"}


# --------------------------------------------------------------------- arms
def run_reference(args):
    ws, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    if args.workload == "contact":
        print(json.dumps({"impl": "reference", "unavailable": (
            "the contact workload's 600x600 table is built on the device (a CPU build by "
            "adaptive quadrature takes hours); its CPU sweep rate is the cpu_baseline of "
            "the engine's line")}))
        return 0
    chains, mixes, desc = workload(args.workload, 0)
    rates = []
    cores = os.cpu_count() or 1
    sample = ""
    # each step a bounded sample; the whole run stays within a few minutes
    budget = max(1.0, min(args.ref_budget, 120.0 / max(args.steps, 1)))
    for _ in range(args.warmup):
        cpu_oracle_rate(chains, mixes, 0, budget_s=0.5)
    for _ in range(args.steps):
        r, cores, sample = cpu_oracle_rate(chains, mixes, 0, budget_s=budget)
        rates.append(r)
    v = float(np.median(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "semantics": "reference (bug-compatible)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "C restatement of PIMC.jl's sweep, not Julia (no Julia "
                                   "toolchain on the box); " + sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import pimc
    from pimc.engine import Engine
    from pimc.shard import shard_of
    ws, rank, local, pg = dist_setup()
    pimc.load()
    sem = 1 if args.semantics == "physical" else 0
    chains, mixes, desc = workload(args.workload, sem)
    if args.chains > 0:
        chains, mixes = chains[:args.chains], mixes[:args.chains]
        desc += f" (first {len(chains)} chains)"
    n_total = len(chains)
    scaling = "weak"
    if ws > 1 and len(chains) > 1:
        # strong scaling: the batch's chains split across the ranks by LPT on
        # the engine's chain cost; every rank runs its shard on its own GPU
        mine = shard_of(chains, rank, ws)
        chains, mixes = [chains[i] for i in mine], [mixes[i] for i in mine]
        scaling = "strong"
    elif ws > 1:
        # a single chain does not shard: independent replicas, own seeds
        for c in chains:
            c.seed = c.seed + 1000003 * rank
    eng = Engine(chains)
    for i, m in enumerate(mixes):
        eng.set_mix(m, chain=i)
    if args.cells is not None or args.crowding is not None:
        eng.set_cells(1 if args.cells is None else args.cells, args.crowding)
    table = None
    if args.workload == "contact":
        t0 = time.perf_counter()
        eng.set_contact_propagator(CONTACT_G0, CONTACT_RANGE)
        table = {"build_s": time.perf_counter() - t0, "entries": 600 * 600,
                 "path": "pimc_set_contact_propagator: composite Gauss-Legendre in FP64 on the "
                         "device, one thread per upper-triangle entry"}
    batched = len(chains) > 1
    run = eng.run_batched if batched else eng.run
    launch = None
    if batched and args.launch:
        f = args.launch.split(":")
        # per phase: CTA size, "w<size>" for one warp per chain, "<size>r<regs>"
        # for the swap kernel compiled for 170 or 255 registers
        pb = f[5].split(",") if len(f) > 5 else ["0", "0", "0"]
        eng.set_launch(block=int(f[1]), sweeps_per_launch=int(f[2]),
                       state_smem_bytes=int(f[3]) if len(f) > 3 else 0,
                       warp_per_chain=f[0] == "warp",
                       split_phases=int(f[4]) if len(f) > 4 else 0,
                       phase_block=[int(b.lstrip("w").split("r")[0]) for b in pb],
                       phase_warp=[int(b.startswith("w")) for b in pb],
                       phase_regs=[int(b.split("r")[1]) if "r" in b else 0 for b in pb])
        launch = dict(eng.launch, tuned=False)
    elif batched and args.tune:
        launch = eng.tune(sweeps_per_trial=1)
        if args.cells is not None:  # an explicit choice outranks the tuner's
            eng.set_cells(args.cells, args.crowding)
            launch = eng.launch
    for _ in range(args.warmup):
        run(1)
    prof = os.environ.get("PIMC_PROFILE", "0") == "1"
    if prof:  # the profiling build: clear the swap counters before the timed sweeps
        import ctypes as C
        pbuf = (C.c_ulonglong * 32)()
        eng.L.pimc_swap_profile(eng.h, pbuf, 1)
    s0 = eng.total_stats()
    barrier(pg)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        run(args.steps)
        wall = time.perf_counter() - t0
    ms = eng.last_run_ms()
    launches = eng.last_run_launches()
    s1 = eng.total_stats()
    swap_profile = None
    if prof:
        eng.L.pimc_swap_profile(eng.h, pbuf, 1)
        v = list(pbuf)
        names = ["heat_bath", "partner_search", "physical_ratio", "bridges", "new_beads",
                 "pair_free_decision", "pair_estimates", "exact_pair_sums", "decision",
                 "accepted_writeback"]
        tot = float(sum(v[:10])) or 1.0
        swap_profile = {"cycle_share": {n: v[k] / tot for k, n in enumerate(names)},
                        "cycles_per_attempt": tot / max(v[16], 1),
                        "counts": dict(zip(["attempts", "n2_eq_n1", "early_accept",
                                            "decided_by_estimate", "exact_sums", "accepted",
                                            "rejected"], v[16:23])),
                        "note": "PIMC_PROFILE build: clock64() cycles of thread 0 per CTA between "
                                "section marks of the swap, summed over CTAs (timed sweeps only)"}
    beads = s1.bead_updates - s0.bead_updates
    tmax, beads_all = reduce_max_sum(pg, ms / 1e3, beads)
    value = beads_all / tmax
    ms_step = tmax * 1e3 / args.steps
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
           "scaling": scaling, "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "gpu_launches": int(launches)}
    state_bytes = sum(8 * (c.dim + 1) * c.N * c.M for c in chains)
    cfg = {"workload": desc, "chains": n_total, "semantics": args.semantics,
           "parallelism": (f"dp{ws}: the chains split across GPUs by LPT on their cost "
                           "(no device collective; host gather of the sums)" if scaling == "strong"
                           else f"dp{ws} (independent replicas per GPU)"),
           "l2": (f"chain state {state_bytes / 1e9:.2f} GB > 129 MB L2"
                  if state_bytes > 129e6 else f"chain state {state_bytes / 1e6:.1f} MB (L2/shared resident)"),
           "bead_updates_per_step": beads / args.steps,
           "neighbour_candidates": {0: "slice scan", 2: "cell lists"}.get(
               (launch["cell_lists"] - 1) if launch and launch.get("cell_lists")
               else (1 if args.cells is None else args.cells),
               "cell lists where they pay (crowding bound "
               f"{0.5 if args.crowding is None else args.crowding}), else slice scan")}
    if batched and launch:
        cfg["launch"] = dict({"tuned": True}, **launch)
    out["config"] = cfg
    # roofline of the dominant kernel.  A split launch shape runs each sweep as
    # three kernels (staging, swaps, the rest): their device times come from
    # a separate pass with CUDA events between the phases, and the kernel
    # with the largest share is the one the roofline describes.  Algorithmic
    # bytes per bead update: 48 B pair-free, 64 B with the pair interaction.
    bpb = np.array([64.0 if c.interactions else 48.0 for c in chains])
    w = np.array([c.N * c.M for c in chains], dtype=float)
    bytes_per_bead = float((bpb * w).sum() / w.sum())
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    split = bool(launch and launch.get("split_phases"))
    if split:
        p0 = eng.total_stats()
        ph_ms = eng.phase_times(ROOF_SWEEPS)
        p1 = eng.total_stats()
        kb = [p1.bead_updates_kind[k] - p0.bead_updates_kind[k] for k in range(4)]
        ph_beads = [kb[0], kb[1], kb[2] + kb[3]]
        top = int(np.argmax(ph_ms))
        # the engine swaps with the kernel compiled for the reference's rules
        # when every chain follows them without a hard core or contact table
        ref_only = all(c.semantics == 0 and c.hardcore_a == 0.0 for c in chains) and table is None
        names = ["k_sweep_stage", "k_sweep_swap_ref" if ref_only else "k_sweep_swap", "k_sweep_rest"]
        kname = names[top]
        launch_s = ph_ms[top] / 1e3 / ROOF_SWEEPS
        beads_per_launch = ph_beads[top] / ROOF_SWEEPS
        kernel_share = {n: float(t / ph_ms.sum()) for n, t in zip(names, ph_ms)}
    else:
        kname = "k_sweep" if batched else "k_sweep (plain)"
        launch_s = (ms / 1e3) / max(launches, 1)
        beads_per_launch = beads / max(launches, 1)
        kernel_share = {kname: 1.0}
    achieved = beads_per_launch * bytes_per_bead / launch_s / 1e9
    # DRAM bytes and FP64 flops per bead update of that kernel: an ncu capture
    # of the same kernel on the first 1216 chains, scaled by the bead updates
    # a full launch performs
    per_bead = PER_BEAD.get((args.workload, args.semantics, kname), {})
    tpb = args.traffic_per_bead if args.traffic_per_bead is not None else per_bead.get("dram_bytes")
    traffic = beads_per_launch * tpb if tpb else None
    out["roofline"] = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm,
                       "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                       "peak_source": ("MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks
                                       else "fallback 6.8 TB/s (of fallback)"),
                       "bytes_per_bead_update": bytes_per_bead,
                       "launch_ms": launch_s * 1e3, "bead_updates_per_launch": beads_per_launch,
                       "kernel_share_of_sweep": kernel_share,
                       "traffic_source": (f"ncu dram__bytes_read+write of {kname} on the first 1216 "
                                          "chains, per bead update, times this launch's bead "
                                          "updates" if tpb else None),
                       "note": "not the binding roof: the sweep is FP64-pipe and latency bound, "
                               "see roofline_fp64"}
    fp64_peak = args.fp64_peak if args.fp64_peak else eng.fp64_peak()
    fpb = args.fp64_flops_per_bead
    measured_fpb = fpb is None and "fp64_flops" in per_bead
    if fpb is None:
        fpb = per_bead.get("fp64_flops", 25.0)
    flops = beads_per_launch * fpb / launch_s / 1e12
    out["roofline_fp64"] = {"bound": "fp64", "kernel": kname, "achieved": flops, "peak": fp64_peak,
                            "unit": "TFLOP/s", "frac": flops / fp64_peak,
                            "flops_per_bead_update": fpb,
                            "flops_source": (f"ncu dadd+dmul+2*dfma thread instructions of {kname} "
                                             "on the first 1216 chains, per bead update"
                                             if measured_fpb else "algorithmic estimate (no pair terms)"),
                            "peak_source": "pimc_fp64_peak: DFMA throughput probe on this GPU (measured)"}
    out["clocks"] = clk.summary()
    if swap_profile is not None:
        out["swap_profile"] = swap_profile
    # plain path: one launch per chain per sweep (no queue, no graph), timed
    # on every PLAIN_STRIDE-th chain of the workload so that it stays short
    if batched and not args.no_plain:
        sub = list(range(0, len(chains), PLAIN_STRIDE))
        pe = Engine([chains[i] for i in sub])
        for k, i in enumerate(sub):
            pe.set_mix(mixes[i], chain=k)
        pe.run_plain(1)
        p0 = pe.total_stats()
        pe.run_plain(1)
        pms = pe.last_run_ms()
        p1 = pe.total_stats()
        out["plain"] = {"value": (p1.bead_updates - p0.bead_updates) / (pms / 1e3),
                        "unit": UNIT, "launches": pe.last_run_launches(),
                        "ms_per_step": pms,
                        "sample": f"every {PLAIN_STRIDE}th chain ({len(sub)} of {len(chains)}), "
                                  "one warm-up sweep, one timed sweep",
                        "path": "one launch per chain per sweep (no queue, no graph)"}
        pe.close()
    # end to end through the C ABI with host buffers: upload the state, sweep,
    # read back the state and the energy sums
    if not args.no_e2e:
        xh, keep = pinned_empty(eng.beads_all_size())
        eng.get_beads_all(xh)

        # a step: the state in from pinned host memory, one sweep, the state
        # and the estimator sums back; a batch does the first three in one
        # call (pimc_batch_run_io)
        def step():
            if batched:
                eng.run_io(xh, 1, chunks=args.io_chunks)
            else:
                eng.set_beads_all(xh)
                run(1)
                eng.get_beads_all(xh)
            eng.energy_sums_all()

        # one untimed step: the legs before this one leave other work's state
        # in the caches and the clocks
        step()
        e0 = eng.total_stats()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        et = time.perf_counter() - t0
        e1 = eng.total_stats()
        # one more step with the three calls apart (host clock; every call
        # returns after its device work)
        tb = []
        for f in (lambda: eng.set_beads_all(xh), lambda: run(1), lambda: eng.get_beads_all(xh),
                  eng.energy_sums_all):
            t1 = time.perf_counter()
            f()
            tb.append((time.perf_counter() - t1) * 1e3)
        emax, ebeads = reduce_max_sum(pg, et, e1.bead_updates - e0.bead_updates)
        nb = 8 * eng.beads_all_size()
        out["e2e"] = {"value": ebeads / emax, "unit": UNIT, "h2d_bytes_per_step": nb,
                      "d2h_bytes_per_step": nb + 8 * 9 * len(chains),
                      "ms_per_step": emax * 1e3 / args.steps,
                      "path": ("pimc_batch_run_io (pinned host buffer in place: the layout "
                               "transposes read and write it over the host link, one sweep of "
                               "every chain in between) + pimc_batch_energy_sums_all") if batched else
                              ("pimc_batch_set_beads_all (pinned host) -> pimc_run -> "
                               "pimc_batch_get_beads_all + pimc_batch_energy_sums_all"),
                      "calls_apart_ms": {"set_beads_all": tb[0], "sweep": tb[1],
                                         "get_beads_all": tb[2], "energy_sums_all": tb[3]}}
    # the adjoint of every chain of the batch in one call (four launches),
    # device time by CUDA events; a step of "batched + adjoint" is one sweep
    # of every chain followed by the adjoint of every chain
    if batched and not args.no_adjoint:
        eng.batch_adjoint()  # makes the handle's adjoint pool
        ams = []
        for _ in range(3):
            eng.batch_adjoint()
            ams.append(eng.last_run_ms())
        a_ms = float(np.median(ams))
        tb = sum(c.N * c.M for c in chains)
        amax, tb_all = reduce_max_sum(pg, a_ms / 1e3, tb)
        out["batched_adjoint"] = {"chains": n_total, "beads": tb_all, "ms_per_call": amax * 1e3,
                                  "bead_gradients_per_s": tb_all / amax, "launches": 4,
                                  "path": "pimc_batch_adjoint: dS/dr of every bead, "
                                          "dS/d(V0, omega, g) and the virial energy of every chain"}
        step_s = ms_step / 1e3 + amax
        out["batched_plus_adjoint"] = {"value": beads_all / args.steps / step_s, "unit": UNIT,
                                       "ms_per_step": step_s * 1e3,
                                       "step": "one sweep of every chain, then the adjoint of "
                                               "every chain (device time)"}
    if args.workload == "c5" or args.adjoint:
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            eng.adjoint(0, want_beads=True)
        at = (time.perf_counter() - t0) / reps
        c = chains[0]
        out["adjoint"] = {"beads": c.N * c.M, "ms_per_call": at * 1e3,
                          "bead_gradients_per_s": c.N * c.M / at}
    contact = eng.contact_table(0) if args.workload == "contact" else None
    if table is not None:
        out["contact_table"] = table
        if rank == 0 and not args.no_cpu:
            out["contact_table"]["cpu"] = cpu_contact_table_rate(CONTACT_G0, chains[0],
                                                                 CONTACT_RANGE)
    if rank == 0 and not args.no_cpu:
        r, cores, sample = cpu_oracle_rate(chains, mixes, sem, budget_s=args.cpu_budget,
                                           contact=contact)
        out["cpu_baseline"] = {"value": r, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "C restatement of PIMC.jl's sweep (same semantics), "
                                         + sample}
    # the energies' side of the metric: a fixed sample of 24 C4 chains run to
    # equilibrium on this GPU and compared per chain with the oracle's run!
    # statistics committed in tests/golden/sweep_stats.json
    if (rank == 0 and args.workload == "c4" and args.semantics == "reference"
            and not args.no_energy_check):
        eng.close()
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from sweep_parity import c4_energy_check
        t0 = time.perf_counter()
        summary, _ = c4_energy_check(semantics=0)
        summary["wall_s"] = time.perf_counter() - t0
        summary["reference"] = ("the oracle (C restatement of the reference's moves) in the "
                                "engine's sweep schedule, tests/golden/sweep_stats.json; the "
                                "reference's rules are not reversible, so the schedule is part "
                                "of what is compared")
        out["energy_check"] = summary
    if rank == 0:
        print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c4", choices=["c1", "c2", "c3", "c4", "c5", "contact"])
    # the library's default (the drop-in keeps the reference's acceptance
    # rules); "physical" adds the pair action to every move
    ap.add_argument("--semantics", default="reference", choices=["physical", "reference"])
    ap.add_argument("--tune", type=int, default=1)
    ap.add_argument("--chains", type=int, default=0,
                    help="keep only the first K chains of the workload (small profiling cases)")
    ap.add_argument("--launch", default=None,
                    help="fixed batched launch shape instead of tuning: "
                         "cta:BLOCK:SPL:STATE_BYTES[:SPLIT[:STAGE,SWAP,REST]] or warp:BLOCK:SPL; "
                         "a phase size written wNNN runs that phase with one warp per chain")
    ap.add_argument("--cells", type=int, default=None, choices=[0, 1, 2],
                    help="neighbour candidates: 0 slice scan, 1 cell lists where they pay "
                         "(the engine's default), 2 cell lists always")
    ap.add_argument("--crowding", type=float, default=None,
                    help="cell-list crowding bound of mode 1 (default 0.5)")
    ap.add_argument("--adjoint", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the batched adjoint timing")
    ap.add_argument("--no-energy-check", action="store_true",
                    help="skip the C4 sample's energies against the oracle's statistics")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--io-chunks", type=int, default=0,
                    help="chunks of chains of the end-to-end step's staged copies, used when "
                         "the host buffer is not page-locked (0: 4)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=6.0)
    ap.add_argument("--ref-budget", type=float, default=8.0)
    ap.add_argument("--traffic-per-bead", type=float, default=None,
                    help="DRAM bytes per bead update of the sweep kernel (ncu)")
    ap.add_argument("--fp64-peak", type=float, default=None, help="TFLOP/s (default: measured)")
    ap.add_argument("--fp64-flops-per-bead", type=float, default=None)
    args = ap.parse_args()
    if args.steps < 1 or args.warmup < 0:
        raise SystemExit("steps >= 1 and warmup >= 0")
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != ws:
        raise SystemExit(f"--gpus {args.gpus} needs {args.gpus} ranks, one per GPU: launch with "
                         f"python -m torch.distributed.run --nproc-per-node {args.gpus} bench.py "
                         f"--gpus {args.gpus} (WORLD_SIZE is {ws})")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
