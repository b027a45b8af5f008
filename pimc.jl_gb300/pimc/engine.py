"""Handle-level wrapper of the C ABI: one object per engine handle.

``Engine`` owns one handle (one or more chains) and exposes every call of
``include/pimc.h`` with numpy buffers.  ``pimc.api`` builds the reference's
Julia-shaped API (System, updates, run, Density, Energy) on top of it.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from ._native import Launch, MoveMix, Params, PimcError, Stats, check, load

SEM_REFERENCE = 0
SEM_PHYSICAL = 1
NOBS = 8  # columns of an observable row (PIMC_NOBS)
REJECT, ACCEPT, SKIP, HARDCORE = 0, 1, 2, 3
OPT_FORCE_WARP_WINDOW = 1
OPT_EXACT_DECISIONS = 2
OPT_CELL_LISTS = 3
OPT_CELL_CROWDING = 4


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def contact_table(g0: float, tau: float, range_: float, n: int = 600) -> np.ndarray:
    """The integral terms T[i1, i2] of the contact-interaction propagator on
    the grid r_i = 1e-20 + i (range_ - 1e-20)/(n - 1), computed on the device
    (prop_rel_interpolate_terms, src/propagator.jl:36-73)"""
    out = np.empty((n, n))
    check(load().pimc_contact_table(float(g0), float(tau), float(range_), int(n), _dp(out)))
    return out


def julia_float(x: float) -> str:
    """x printed as Julia prints a Float64 (the engine's CSV writers use it)"""
    buf = C.create_string_buffer(64)
    check(load().pimc_format_float(float(x), buf, 64))
    return buf.value.decode()


def write_density_csv(path: str, dim: int, nbins: int, L: float, counts, ndata: int):
    """save_density's table (examples/tools/savetools.jl:37-65) from counts
    (nbins^dim, column-major) and the number of bead samples ndata"""
    c = np.ascontiguousarray(np.ravel(counts, order="F"), dtype=np.float64)
    if c.size != nbins ** dim:
        raise PimcError("counts must hold nbins^dim values")
    check(load().pimc_write_density_csv(os.fsencode(path), dim, nbins, float(L), _dp(c), int(ndata)))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


@dataclass
class ChainParams:
    """pimc_params: the System constructor's arguments in engine-known form."""
    dim: int = 2
    N: int = 2
    M: int = 100
    L: float = 4.0
    T: float = 1.0
    lam: float = 1.0
    mu: float = 0.0
    harmonic_omega: float = 0.0
    lattice_V0: float = 0.0
    lattice_a: float = 1.0
    interactions: bool = False
    pair_g: float = 0.0
    pair_sigma: float = 1.0
    r_a: float = 0.0
    hardcore_a: float = 0.0
    semantics: int = SEM_REFERENCE
    seed: int = 20261203
    density_nbins: int = 0
    energy_capacity: int = 0
    retry_cap: int = 0

    def to_c(self) -> Params:
        p = Params()
        for f in ("dim", "N", "M", "L", "T", "lam", "mu", "harmonic_omega", "lattice_V0",
                  "lattice_a", "pair_g", "pair_sigma", "r_a", "hardcore_a", "semantics",
                  "seed", "density_nbins", "energy_capacity", "retry_cap"):
            setattr(p, f, getattr(self, f))
        p.interactions = 1 if self.interactions else 0
        return p


@dataclass
class Mix:
    """pimc_move_mix: the per-sweep move schedule."""
    staging_phases: int = 1
    stage_slices: int = 16
    stage_min: int = 2
    stage_max: int = 16
    stage_minacc: float = 0.6
    stage_maxacc: float = 0.8
    swaps_per_sweep: int = 0
    swap_slices: int = 16
    swap_min: int = 2
    swap_max: int = 16
    swap_minacc: float = 0.6
    swap_maxacc: float = 0.8
    com_phases: int = 1
    com_step: float = 1.0
    com_minstep: float = 0.1
    com_maxstep: float = 2.0
    com_minacc: float = 0.4
    com_maxacc: float = 0.6
    polymer_com_phases: int = 0
    pcom_step: float = 1.0
    pcom_minstep: float = 0.1
    pcom_maxstep: float = 2.0
    pcom_minacc: float = 0.4
    pcom_maxacc: float = 0.6
    adapt: int = 1
    measure_every: int = 0

    def to_c(self) -> MoveMix:
        m = MoveMix()
        for f, _ in MoveMix._fields_:
            setattr(m, f, getattr(self, f))
        return m


@dataclass
class EngineStats:
    attempts: list = field(default_factory=list)
    accepts: list = field(default_factory=list)
    skips: int = 0
    bead_updates: float = 0.0
    sweeps: int = 0
    measurements: int = 0
    stage_slices: int = 0
    swap_slices: int = 0
    com_step: float = 0.0
    pcom_step: float = 0.0
    bead_updates_kind: list = field(default_factory=list)


class Engine:
    """One engine handle holding ``len(params)`` independent chains."""

    def __init__(self, params, mix: Mix | None = None):
        self.L = load()
        plist = params if isinstance(params, (list, tuple)) else [params]
        self.params = list(plist)
        arr = (Params * len(plist))(*[p.to_c() for p in plist])
        h = C.c_void_p()
        if len(plist) == 1:
            check(self.L.pimc_create(arr, C.byref(h)))
        else:
            check(self.L.pimc_batch_create(arr, len(plist), C.byref(h)))
        self.h = h
        if mix is not None:
            self.set_mix(mix)

    def close(self):
        if getattr(self, "h", None):
            self.L.pimc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- state
    def shape(self, chain=0):
        p = self.params[chain]
        return (p.dim, p.N, p.M)

    def set_beads(self, x, chain=0):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape(chain))
        check(self.L.pimc_batch_set_beads(self.h, chain, _dp(x)))

    def get_beads(self, chain=0):
        x = np.empty(self.shape(chain))
        check(self.L.pimc_batch_get_beads(self.h, chain, _dp(x)))
        return x

    def beads_all_size(self) -> int:
        return int(sum(p.dim * p.N * p.M for p in self.params))

    def set_beads_all(self, x_all):
        x_all = np.ascontiguousarray(x_all, dtype=np.float64)
        if x_all.size != self.beads_all_size():
            raise PimcError("x_all has the wrong size")
        check(self.L.pimc_batch_set_beads_all(self.h, _dp(x_all)))

    def get_beads_all(self, out=None):
        out = np.empty(self.beads_all_size()) if out is None else out
        check(self.L.pimc_batch_get_beads_all(self.h, _dp(out)))
        return out

    def energy_sums_all(self):
        n = len(self.params)
        s, s2 = np.zeros((n, 4)), np.zeros((n, 4))
        cnt = np.zeros(n, dtype=np.uint64)
        check(self.L.pimc_batch_energy_sums_all(self.h, _dp(s), _dp(s2),
                                                cnt.ctypes.data_as(C.POINTER(C.c_ulonglong))))
        return s, s2, cnt

    def set_next(self, nxt):
        nxt = np.ascontiguousarray(nxt, dtype=np.int32)
        check(self.L.pimc_set_next(self.h, _ip(nxt)))

    def get_next(self, chain=0):
        n = np.empty(self.params[chain].N, dtype=np.int32)
        check(self.L.pimc_batch_get_next(self.h, chain, _ip(n)))
        return n

    def set_raw(self, x, V, nxt):
        x = np.ascontiguousarray(x, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        nxt = np.ascontiguousarray(nxt, dtype=np.int32)
        check(self.L.pimc_set_raw(self.h, _dp(x), _dp(V), _ip(nxt)))

    def get_links(self):
        p = self.params[0]
        V = np.empty((p.N, p.M))
        check(self.L.pimc_get_links(self.h, _dp(V)))
        return V

    def init_world(self):
        check(self.L.pimc_init_world(self.h))

    # ------------------------------------------------------------- sweeps
    def set_mix(self, mix: Mix, chain: int = -1):
        m = mix.to_c()
        check(self.L.pimc_set_move_mix(self.h, chain, C.byref(m)))

    def run(self, n_sweeps: int):
        check(self.L.pimc_run(self.h, int(n_sweeps)))

    def run_batched(self, n_sweeps: int):
        check(self.L.pimc_batch_run(self.h, int(n_sweeps)))

    def run_plain(self, n_sweeps: int):
        check(self.L.pimc_batch_run_plain(self.h, int(n_sweeps)))

    def run_io(self, x_in, n_sweeps: int, x_out=None, chunks: int = 0):
        """set_beads_all(x_in), run_batched(n_sweeps), get_beads_all(x_out) in
        one call whose copies overlap the sweeps (chunks of chains; 0: 4);
        x_out may be x_in (in place); returns x_out"""
        for a in (x_in,) if x_out is None else (x_in, x_out):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous
                    and a.size == self.beads_all_size()):
                raise PimcError("x_in / x_out must be contiguous float64 arrays of beads_all_size()")
        x_out = x_in if x_out is None else x_out
        check(self.L.pimc_batch_run_io(self.h, _dp(x_in), _dp(x_out), int(n_sweeps), int(chunks)))
        return x_out

    def device_name(self) -> str:
        buf = C.create_string_buffer(256)
        sms = C.c_int()
        check(self.L.pimc_device_info(self.h, buf, 256, C.byref(sms)))
        return buf.value.decode()

    def tune(self, sweeps_per_trial: int = 2, cache: str | None = None) -> dict:
        """time the candidate launch shapes and keep the fastest (chains
        restored).  With cache (a JSON file path), a shape kept there for a
        batch of the same mix of chain shapes on the same GPU is used without
        timing, and a newly timed shape is stored (pimc/tuning.py)."""
        sig = tc = None
        if cache:
            from .tuning import TuneCache, batch_signature
            sig = batch_signature(self.params, self.device_name(), self.L.pimc_abi_version())
            tc = TuneCache(cache)
            hit = tc.get(sig)
            if hit is not None:
                try:
                    self.set_launch(**hit)
                    return dict(self.launch, cached=True)
                except PimcError:
                    pass  # a shape this build no longer accepts: time afresh
        l = Launch()
        check(self.L.pimc_batch_tune(self.h, sweeps_per_trial, C.byref(l)))
        if tc is not None:
            tc.put(sig, self.launch)
        return self.launch

    def set_launch(self, block: int, sweeps_per_launch: int = 1,
                   state_smem_bytes: int = 100 * 1024, warp_per_chain: bool = False,
                   split_phases: int = 0, phase_block=(0, 0, 0), phase_warp=(0, 0, 0),
                   phase_regs=(0, 0, 0), cell_lists: int = 0):
        """cell_lists: 0 keeps the cell-list option (set_cells), 1 + a mode
        of it sets it (1 off, 2 auto, 3 always)"""
        l = Launch(int(bool(warp_per_chain)), block, sweeps_per_launch, state_smem_bytes,
                   int(split_phases), (C.c_int * 3)(*[int(b) for b in phase_block]),
                   (C.c_int * 3)(*[int(w) for w in phase_warp]),
                   (C.c_int * 3)(*[int(r) for r in phase_regs]), int(cell_lists))
        check(self.L.pimc_batch_set_launch(self.h, C.byref(l)))

    @property
    def launch(self) -> dict:
        """the batched launch shape in use"""
        l = Launch()
        check(self.L.pimc_batch_get_launch(self.h, C.byref(l)))
        return {"warp_per_chain": bool(l.warp_per_chain), "block": l.block,
                "sweeps_per_launch": l.sweeps_per_launch, "state_smem_bytes": l.state_smem_bytes,
                "split_phases": l.split_phases, "phase_block": list(l.phase_block),
                "phase_warp": list(l.phase_warp), "phase_regs": list(l.phase_regs),
                "cell_lists": l.cell_lists}

    def phase_times(self, n_sweeps: int = 2):
        """device ms of the staging, swap and remaining phases over n sweeps,
        issued as separate launches with events between them"""
        ms = np.zeros(3)
        check(self.L.pimc_batch_phase_times(self.h, int(n_sweeps), _dp(ms)))
        return ms

    def fp64_peak(self) -> float:
        """measured FP64 FMA throughput of the device, TFLOP/s"""
        v = C.c_double()
        check(self.L.pimc_fp64_peak(self.h, C.byref(v)))
        return v.value

    def last_run_ms(self) -> float:
        v = C.c_double()
        check(self.L.pimc_last_run_ms(self.h, C.byref(v)))
        return v.value

    def last_run_launches(self) -> int:
        v = C.c_longlong()
        check(self.L.pimc_last_run_launches(self.h, C.byref(v)))
        return v.value

    def set_option(self, key: int, value: int):
        check(self.L.pimc_set_option(self.h, key, value))

    def set_cells(self, mode: int, crowding: float | None = None):
        """neighbour candidates from per-slice cell lists: mode 0 off (scan the
        slice), 1 auto (lists except on slices whose 3^dim sum n_c^2 exceeds
        crowding * N^2; default crowding 0.5), 2 always"""
        self.set_option(OPT_CELL_LISTS, int(mode))
        if crowding is not None:
            self.set_option(OPT_CELL_CROWDING, int(round(crowding * 1000)))

    # ------------------------------------------------------------- attempts
    def attempt_staging(self, n, j0, m, normals, uniforms=()):
        nr = np.ascontiguousarray(normals, dtype=np.float64)
        un = np.ascontiguousarray(uniforms, dtype=np.float64)
        res = C.c_int()
        prop = np.zeros((m + 1) * self.params[0].dim)
        check(self.L.pimc_attempt_staging(self.h, n, j0, m, _dp(nr) if nr.size else None, nr.size,
                                          _dp(un) if un.size else None, un.size, C.byref(res),
                                          _dp(prop)))
        return res.value, prop.reshape(m + 1, self.params[0].dim)

    def attempt_swap(self, j0, m, n1, u_pick, normals, uniforms=()):
        nr = np.ascontiguousarray(normals, dtype=np.float64)
        un = np.ascontiguousarray(uniforms, dtype=np.float64)
        res, n2 = C.c_int(), C.c_int()
        prop = np.zeros(2 * (m + 1) * self.params[0].dim)
        check(self.L.pimc_attempt_swap(self.h, j0, m, n1, u_pick, _dp(nr) if nr.size else None,
                                       nr.size, _dp(un) if un.size else None, un.size,
                                       C.byref(res), C.byref(n2), _dp(prop)))
        return res.value, n2.value, prop.reshape(2, m + 1, self.params[0].dim)

    def attempt_com(self, n, step, uniforms):
        un = np.ascontiguousarray(uniforms, dtype=np.float64)
        res = C.c_int()
        check(self.L.pimc_attempt_com(self.h, n, step, _dp(un) if un.size else None, un.size,
                                      C.byref(res)))
        return res.value

    def attempt_polymer_com(self, n, step, uniforms):
        un = np.ascontiguousarray(uniforms, dtype=np.float64)
        res = C.c_int()
        check(self.L.pimc_attempt_polymer_com(self.h, n, step, _dp(un) if un.size else None,
                                              un.size, C.byref(res)))
        return res.value

    # ------------------------------------------------------------- evaluation
    def eval_action(self):
        out = np.zeros(4)
        check(self.L.pimc_eval_action(self.h, _dp(out)))
        return out

    def staging_weights(self, n, j0, m, rp):
        rp = np.ascontiguousarray(rp, dtype=np.float64)
        wi, wu = C.c_double(), C.c_double()
        check(self.L.pimc_eval_staging_weights(self.h, n, j0, m, _dp(rp), C.byref(wi), C.byref(wu)))
        return wi.value, wu.value

    # ------------------------------------------------------------- estimators
    def measure(self):
        check(self.L.pimc_measure(self.h))

    def energies(self, chain=0):
        cnt = C.c_int()
        check(self.L.pimc_get_energies(self.h, chain, None, 0, C.byref(cnt)))
        out = np.zeros((max(cnt.value, 1), 4))
        check(self.L.pimc_get_energies(self.h, chain, _dp(out), cnt.value, C.byref(cnt)))
        return out[: cnt.value]

    def energy_sums(self, chain=0):
        s, s2 = np.zeros(4), np.zeros(4)
        cnt = C.c_ulonglong()
        check(self.L.pimc_get_energy_sums(self.h, chain, _dp(s), _dp(s2), C.byref(cnt)))
        return s, s2, cnt.value

    def observables(self, chain=0):
        """rows of NOBS: E_th, E_v, pair energy, pair virial energy, W^2, A_z,
        sum r^2 / M, 0"""
        cnt = C.c_int()
        check(self.L.pimc_get_observables(self.h, chain, None, 0, C.byref(cnt)))
        out = np.zeros((max(cnt.value, 1), NOBS))
        check(self.L.pimc_get_observables(self.h, chain, _dp(out), cnt.value, C.byref(cnt)))
        return out[: cnt.value]

    def observable_sums(self, chain=0):
        s, s2 = np.zeros(NOBS), np.zeros(NOBS)
        cnt = C.c_ulonglong()
        check(self.L.pimc_get_observable_sums(self.h, chain, _dp(s), _dp(s2), C.byref(cnt)))
        return s, s2, cnt.value

    def set_radial(self, nbins: int, rmax: float = 0.0, chain: int = -1):
        """pair-distance histogram of nbins bins over [0, rmax) (rmax 0: L)"""
        check(self.L.pimc_set_radial(self.h, chain, int(nbins), float(rmax)))
        for i, p in enumerate(self.params):
            if chain < 0 or i == chain:
                p._rdf_nb = int(nbins)

    def radial(self, chain=0):
        """(pair counts per bin, measurements accumulated)"""
        nb = getattr(self.params[chain], "_rdf_nb", 0)
        hist = np.zeros(max(nb, 1))
        nm = C.c_ulonglong()
        check(self.L.pimc_get_radial(self.h, chain, _dp(hist), C.byref(nm)))
        return hist[:nb], nm.value

    def density(self, chain=0):
        p = self.params[chain]
        hist = np.zeros(p.density_nbins ** p.dim)
        nd = C.c_ulonglong()
        check(self.L.pimc_get_density(self.h, chain, _dp(hist), C.byref(nd)))
        return hist, nd.value

    def reset_measurements(self):
        check(self.L.pimc_reset_measurements(self.h))

    # ------------------------------------------------------------- adjoint
    def adjoint(self, chain=0, want_beads=True):
        p = self.params[chain]
        g = np.zeros((p.dim, p.N, p.M)) if want_beads else None
        th, ex = np.zeros(3), np.zeros(4)
        check(self.L.pimc_adjoint(self.h, chain, _dp(g) if want_beads else None, _dp(th), _dp(ex)))
        return g, th, ex

    def batch_adjoint(self, want_beads=False):
        """the adjoint of every chain in one call (pimc_batch_adjoint):
        dS/dtheta [chains][3], extra [chains][4] and, with want_beads, dS/dr
        as a list of per-chain [dim][N][M] arrays"""
        n = len(self.params)
        th, ex = np.zeros((n, 3)), np.zeros((n, 4))
        g = np.zeros(self.beads_all_size()) if want_beads else None
        check(self.L.pimc_batch_adjoint(self.h, _dp(th), _dp(ex), _dp(g) if want_beads else None))
        if not want_beads:
            return None, th, ex
        out, o = [], 0
        for p in self.params:
            k = p.dim * p.N * p.M
            out.append(g[o:o + k].reshape(p.dim, p.N, p.M))
            o += k
        return out, th, ex

    # ------------------------------------------------------------- files
    def write_paths_csv(self, path: str, chain: int = 0):
        """save_paths (examples/tools/savetools.jl:4-35) from the device state"""
        check(self.L.pimc_write_paths_csv(self.h, chain, os.fsencode(path)))

    def save_checkpoint(self, path: str):
        check(self.L.pimc_save_checkpoint(self.h, os.fsencode(path)))

    def load_checkpoint(self, path: str):
        check(self.L.pimc_load_checkpoint(self.h, os.fsencode(path)))

    # ------------------------------------------------------------- contact propagator
    def set_contact_propagator(self, g0: float, range_: float, n: int = 600, chain: int = -1):
        """build_prop_int(range_, g0, tau) on the device as the pair propagator
        of a chain (chain < 0: all), tau the chain's own"""
        check(self.L.pimc_set_contact_propagator(self.h, chain, float(g0), float(range_), int(n)))

    def set_contact_table(self, table, range_: float, chain: int = -1):
        """a caller-made table T[i1, i2] on the grid 1e-20 .. range_"""
        t = np.ascontiguousarray(table, dtype=np.float64)
        if t.ndim != 2 or t.shape[0] != t.shape[1]:
            raise PimcError("the contact table must be square")
        check(self.L.pimc_set_contact_table(self.h, chain, _dp(t), t.shape[0], float(range_)))

    def contact_table(self, chain: int = 0):
        """(table, range) of the chain's contact propagator, or (None, 0.0)"""
        n, rng = C.c_int(), C.c_double()
        check(self.L.pimc_get_contact_table(self.h, chain, None, 0, C.byref(n), C.byref(rng)))
        if n.value == 0:
            return None, 0.0
        out = np.empty((n.value, n.value))
        check(self.L.pimc_get_contact_table(self.h, chain, _dp(out), out.size, C.byref(n),
                                            C.byref(rng)))
        return out, rng.value

    def clear_contact(self, chain: int = -1):
        check(self.L.pimc_clear_contact(self.h, chain))

    def set_beams(self, angles, scale: float, depth: float, helical: bool = False,
                  chain: int = -1):
        """optical lattice depth * normalized_intensity (potentialtools.jl:1-16)"""
        a = np.ascontiguousarray(angles, dtype=np.float64)
        check(self.L.pimc_set_beams(self.h, chain, _dp(a) if a.size else None, a.size,
                                    float(scale), float(depth), int(bool(helical))))

    def set_potential(self, V0, omega, g, chain=0):
        check(self.L.pimc_set_potential(self.h, chain, V0, omega, g))
        p = self.params[chain]
        p.lattice_V0, p.harmonic_omega, p.pair_g = V0, omega, g

    # ------------------------------------------------------------- diagnostics
    @staticmethod
    def _stats(s: Stats) -> EngineStats:
        return EngineStats(list(s.attempts), list(s.accepts), s.skips, s.bead_updates, s.sweeps,
                           s.measurements, s.stage_slices, s.swap_slices, s.com_step, s.pcom_step,
                           list(s.bead_updates_kind))

    def stats(self, chain=0) -> EngineStats:
        s = Stats()
        check(self.L.pimc_get_stats(self.h, chain, C.byref(s)))
        return self._stats(s)

    def total_stats(self) -> EngineStats:
        s = Stats()
        check(self.L.pimc_get_total_stats(self.h, C.byref(s)))
        return self._stats(s)

    def get_state(self) -> bytes:
        n = C.c_size_t()
        check(self.L.pimc_state_size(self.h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        check(self.L.pimc_get_state(self.h, buf, n.value))
        return buf.raw

    def set_state(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        check(self.L.pimc_set_state(self.h, buf, len(blob)))


__all__ = ["Engine", "ChainParams", "Mix", "EngineStats", "PimcError", "SEM_REFERENCE",
           "SEM_PHYSICAL", "REJECT", "ACCEPT", "SKIP", "HARDCORE", "OPT_FORCE_WARP_WINDOW",
           "OPT_EXACT_DECISIONS", "OPT_CELL_LISTS", "OPT_CELL_CROWDING"]
