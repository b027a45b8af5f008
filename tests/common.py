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
