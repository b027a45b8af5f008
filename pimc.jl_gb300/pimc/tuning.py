"""Persistent choices of the launch-shape tuner.

``pimc_batch_tune`` times candidate launch shapes on a batch's own chains
(seconds for a large batch).  The shape it picks depends on the batch's mix
of chain sizes and on the GPU, not on the chains' positions, so a shape can
be kept and reused by later runs of a batch with the same mix: this module
keys it by a signature of the batch -- the number of chains per (N bucket, M,
pair interaction, acceptance rules), N bucketed by powers of two -- together
with the device name and the library's ABI version, and stores it in a JSON
file.  ``Engine.tune(cache=path)`` looks the signature up first and times
only on a miss.
"""
from __future__ import annotations

import json
import os
from collections import Counter

LAUNCH_KEYS = ("warp_per_chain", "block", "sweeps_per_launch", "state_smem_bytes",
               "split_phases", "phase_block", "phase_warp", "phase_regs", "cell_lists")


def n_bucket(N: int) -> int:
    """the power-of-two bucket of a particle number: 8..15 -> 8, 16..31 -> 16, ..."""
    b = 1
    while b * 2 <= N:
        b *= 2
    return b


def batch_signature(params, device: str, abi: int) -> str:
    """a stable text key of a batch's mix of chain shapes on a device"""
    get = (lambda p, k: p[k]) if params and isinstance(params[0], dict) else getattr
    cnt = Counter()
    for p in params:
        cnt[(n_bucket(int(get(p, "N"))), int(get(p, "M")), int(bool(get(p, "interactions"))),
             int(get(p, "semantics")))] += 1
    buckets = ";".join(f"{n}x{m}p{i}s{s}:{c}" for (n, m, i, s), c in sorted(cnt.items()))
    return f"abi{abi}|{device}|{buckets}"


class TuneCache:
    """launch shapes by batch signature, kept in a JSON file"""

    def __init__(self, path: str):
        self.path = path
        self.data = {}
        if os.path.exists(path):
            with open(path) as f:
                self.data = json.load(f)

    def get(self, signature: str):
        v = self.data.get(signature)
        if v is None or any(k not in v for k in LAUNCH_KEYS):
            return None
        return {k: v[k] for k in LAUNCH_KEYS}

    def put(self, signature: str, launch: dict, ms_per_sweep: float | None = None):
        entry = {k: launch[k] for k in LAUNCH_KEYS}
        for k in ("phase_block", "phase_warp", "phase_regs"):
            entry[k] = [int(x) for x in entry[k]]
        if ms_per_sweep is not None:
            entry["ms_per_sweep"] = float(ms_per_sweep)
        self.data[signature] = entry
        tmp = self.path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(self.data, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)
