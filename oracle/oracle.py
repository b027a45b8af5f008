"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of oameye/PIMC.jl's Monte Carlo sweep
(``oracle/pimc_oracle.c``).  Only the tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` use this module, always as the checker or
as the timed CPU reference -- never as part of the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpimc_oracle.so")

SEM_REFERENCE = 0
SEM_PHYSICAL = 1
REJECT, ACCEPT, SKIP, HARDCORE = 0, 1, 2, 3


class Params(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("N", C.c_int), ("M", C.c_int),
        ("L", C.c_double), ("beta", C.c_double), ("tau", C.c_double),
        ("lam", C.c_double), ("mu", C.c_double),
        ("hcoef", C.c_double), ("V0", C.c_double), ("lat_k", C.c_double),
        ("interactions", C.c_int), ("g", C.c_double), ("inv2s2", C.c_double),
        ("nbins", C.c_int), ("rc", C.c_double), ("hardcore_a", C.c_double),
        ("ctr", C.c_int), ("semantics", C.c_int),
        ("ct_tab", C.POINTER(C.c_double)), ("ct_n", C.c_int), ("ct_range", C.c_double),
        ("nbeam", C.c_int), ("beam_helical", C.c_int), ("beam_depth", C.c_double),
        ("beam_scale", C.c_double), ("beam_angle", C.c_double * 16),
    ]


class Rng(C.Structure):
    _fields_ = [("key", C.c_uint32 * 2), ("ctr", C.c_uint32 * 4), ("buf", C.c_uint32 * 4),
                ("pos", C.c_int), ("have_spare", C.c_int), ("spare", C.c_double)]


class Draws(C.Structure):
    _fields_ = [
        ("normals", C.POINTER(C.c_double)), ("n_normals", C.c_long), ("normal_pos", C.c_long),
        ("uniforms", C.POINTER(C.c_double)), ("n_uniforms", C.c_long), ("uniform_pos", C.c_long),
        ("rng", C.POINTER(Rng)), ("exhausted", C.c_int),
    ]


class Update(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("every", C.c_int), ("var", C.c_double), ("minvar", C.c_double),
        ("maxvar", C.c_double), ("minacc", C.c_double), ("maxacc", C.c_double),
        ("adj", C.c_int), ("range", C.c_int), ("queue", C.c_void_p), ("qlen", C.c_int),
        ("qhead", C.c_int), ("qsum", C.c_long), ("tries", C.c_long),
        ("attempts", C.c_long), ("accepts", C.c_long),
    ]


class RunStats(C.Structure):
    _fields_ = [("attempts", C.c_long * 4), ("accepts", C.c_long * 4),
                ("bead_updates", C.c_double), ("measurements", C.c_long)]


def build() -> str:
    """Compile the oracle with its Makefile (gcc; seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(Params)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_set_state.argtypes = [C.c_void_p, dp, ip]
        L.orc_set_raw.argtypes = [C.c_void_p, dp, dp, ip]
        L.orc_get_state.argtypes = [C.c_void_p, dp, dp, ip]
        L.orc_init_world.argtypes = [C.c_void_p, C.POINTER(Draws)]
        L.orc_distance.restype = C.c_double
        L.orc_distance.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_teleport.restype = C.c_double
        L.orc_teleport.argtypes = [C.c_double, C.c_double]
        L.orc_lnK.restype = C.c_double
        L.orc_lnK.argtypes = [C.POINTER(Params), dp, dp, C.c_double]
        L.orc_Vext.restype = C.c_double
        L.orc_Vext.argtypes = [C.POINTER(Params), dp]
        L.orc_lnV.restype = C.c_double
        L.orc_lnV.argtypes = [C.POINTER(Params), dp, dp]
        L.orc_lnU.restype = C.c_double
        L.orc_lnU.argtypes = [C.POINTER(Params), dp, dp]
        L.orc_eval_action.argtypes = [C.c_void_p, dp]
        L.orc_staging_weights.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, dp, dp, dp]
        L.orc_staging.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(Draws), dp]
        L.orc_swap.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                               C.POINTER(Draws), ip, dp]
        L.orc_com.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(Draws)]
        L.orc_polymer_com.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(Draws)]
        L.orc_energy.argtypes = [C.c_void_p, dp]
        L.orc_density.argtypes = [C.c_void_p, C.c_int, dp]
        L.orc_superfluid.argtypes = [C.c_void_p, dp]
        L.orc_radial.argtypes = [C.c_void_p, C.c_int, C.c_double, dp]
        L.orc_rng_init.argtypes = [C.POINTER(Rng), C.c_uint64, C.c_uint64]
        L.orc_rng_uniform.restype = C.c_double
        L.orc_rng_uniform.argtypes = [C.POINTER(Rng)]
        L.orc_rng_normal.restype = C.c_double
        L.orc_rng_normal.argtypes = [C.POINTER(Rng)]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32)]
        L.orc_update_init.argtypes = [C.POINTER(Update), C.c_int, C.c_int, C.c_double,
                                      C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_int, C.c_int]
        L.orc_update_free.argtypes = [C.POINTER(Update)]
        L.orc_run.argtypes = [C.c_void_p, C.c_long, C.POINTER(Update), C.c_int, C.POINTER(Rng),
                              C.c_int, dp, C.c_long, C.POINTER(C.c_long), C.c_int, dp,
                              C.POINTER(C.c_long), C.POINTER(RunStats)]
        L.orc_run_sweeps.argtypes = [C.c_void_p, C.c_long, C.c_int, C.c_int, dp, C.c_double,
                                     C.c_double, C.c_double, C.c_double, C.POINTER(Rng), C.c_int,
                                     dp, C.c_long, C.POINTER(C.c_long), C.c_int, dp,
                                     C.POINTER(C.c_long), C.POINTER(RunStats)]
        L.orc_bench_budget.restype = C.c_double
        L.orc_bench_budget.argtypes = [C.POINTER(Params), C.POINTER(C.c_int), C.c_int, C.c_int,
                                       C.c_double, C.c_double, C.c_uint64, dp, dp]
        L.orc_bench_chains.restype = C.c_double
        L.orc_bench_chains.argtypes = [C.POINTER(Params), C.c_int, C.c_int, C.c_long, C.c_int,
                                       C.c_double, C.c_uint64, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def make_params(dim=2, N=2, M=100, L=4.0, T=1.0, lam=1.0, hcoef=0.0, V0=0.0, lat_a=1.0,
                pair_g=0.0, pair_sigma=1.0, interactions=False, r_a=0.0, hardcore_a=0.0,
                semantics=SEM_REFERENCE, ctr=10000, mu=0.0, contact_table=None,
                contact_range=0.0, beams=None) -> Params:
    """Parameters with the System constructor's derived constants
    (src/system.jl:129-167): tau = beta/M, nbins = floor(2L/r_a), r_a = L/4
    when unset without interactions.  contact_table (n x n, on the grid
    1e-20 .. contact_range) switches lnU to the tabulated contact propagator
    (src/propagator.jl:74-89); the Params object keeps the array alive."""
    p = Params()
    p.dim, p.N, p.M, p.L = dim, N, M, L
    p.beta = 1.0 / T
    p.tau = p.beta / M
    p.lam, p.mu = lam, mu
    p.hcoef, p.V0 = hcoef, V0
    p.lat_k = np.pi / lat_a
    p.interactions = 1 if interactions else 0
    p.g = pair_g
    p.inv2s2 = 1.0 / (2.0 * pair_sigma * pair_sigma)
    ra = r_a if r_a > 0 else L / 4.0
    p.nbins = int(np.floor((2.0 * L) / ra))
    p.rc = 2.0 * L / p.nbins
    p.hardcore_a = hardcore_a
    p.ctr = ctr
    p.semantics = semantics
    if beams is not None:
        # (angles, scale, depth, helical): the optical lattice of potentialtools.jl
        angles, scale, depth, helical = beams
        if not 0 < len(angles) <= 16:
            raise ValueError("between 1 and 16 beam angles")
        p.nbeam = len(angles)
        for k, a in enumerate(angles):
            p.beam_angle[k] = float(a)
        p.beam_scale, p.beam_depth, p.beam_helical = float(scale), float(depth), int(bool(helical))
    if contact_table is not None:
        tab = np.ascontiguousarray(contact_table, dtype=np.float64)
        if tab.ndim != 2 or tab.shape[0] != tab.shape[1] or tab.shape[0] < 2:
            raise ValueError("contact_table must be a square n x n array, n >= 2")
        if not contact_range > 1e-20:
            raise ValueError("contact_range must be positive")
        p._ct_keep = tab
        p.ct_tab = _dp(tab)
        p.ct_n = tab.shape[0]
        p.ct_range = contact_range
    return p


class Draw:
    """Injected normal / uniform streams for one or more moves."""

    def __init__(self, normals=(), uniforms=()):
        self.normals = np.ascontiguousarray(normals, dtype=np.float64)
        self.uniforms = np.ascontiguousarray(uniforms, dtype=np.float64)
        self.s = Draws()
        self.s.normals = _dp(self.normals) if self.normals.size else None
        self.s.n_normals = self.normals.size
        self.s.uniforms = _dp(self.uniforms) if self.uniforms.size else None
        self.s.n_uniforms = self.uniforms.size
        self.s.rng = None

    @property
    def normals_used(self):
        return self.s.normal_pos

    @property
    def uniforms_used(self):
        return self.s.uniform_pos


class Oracle:
    """One chain of the CPU oracle."""

    def __init__(self, params: Params):
        self.p = params
        self.L = lib()
        self.h = self.L.orc_create(C.byref(self.p))
        if not self.h:
            raise ValueError("orc_create rejected the parameters")

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    @property
    def shape(self):
        return (self.p.dim, self.p.N, self.p.M)

    def set_state(self, x, nxt=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape)
        nx = None if nxt is None else np.ascontiguousarray(nxt, dtype=np.int32)
        self.L.orc_set_state(self.h, _dp(x), None if nx is None else _ip(nx))

    def set_raw(self, x, V, nxt):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape)
        V = np.ascontiguousarray(V, dtype=np.float64).reshape(self.p.N, self.p.M)
        nx = np.ascontiguousarray(nxt, dtype=np.int32)
        self.L.orc_set_raw(self.h, _dp(x), _dp(V), _ip(nx))

    def get_state(self):
        x = np.empty(self.shape)
        V = np.empty((self.p.N, self.p.M))
        nx = np.empty(self.p.N, dtype=np.int32)
        self.L.orc_get_state(self.h, _dp(x), _dp(V), _ip(nx))
        return x, V, nx

    def init_world(self, seed=1, stream=0):
        r = Rng()
        self.L.orc_rng_init(C.byref(r), seed, stream)
        d = Draws()
        d.rng = C.pointer(r)
        return self.L.orc_init_world(self.h, C.byref(d))

    def eval_action(self):
        out = np.zeros(4)
        self.L.orc_eval_action(self.h, _dp(out))
        return out

    def staging_weights(self, n, j0, m, rp):
        rp = np.ascontiguousarray(rp, dtype=np.float64)
        wi, wu = np.zeros(1), np.zeros(1)
        self.L.orc_staging_weights(self.h, n, j0, m, _dp(rp), _dp(wi), _dp(wu))
        return float(wi[0]), float(wu[0])

    def staging(self, n, j0, m, draw: Draw):
        rp = np.zeros((m + 1) * self.p.dim)
        rc = self.L.orc_staging(self.h, n, j0, m, C.byref(draw.s), _dp(rp))
        return rc, rp.reshape(m + 1, self.p.dim)

    def swap(self, j0, m, n1, u_pick, draw: Draw):
        n2 = np.zeros(1, dtype=np.int32)
        rp = np.zeros(2 * (m + 1) * self.p.dim)
        rc = self.L.orc_swap(self.h, j0, m, n1, u_pick, C.byref(draw.s), _ip(n2), _dp(rp))
        return rc, int(n2[0]), rp.reshape(2, m + 1, self.p.dim)

    def com(self, n, maxd, draw: Draw):
        return self.L.orc_com(self.h, n, maxd, C.byref(draw.s))

    def polymer_com(self, n, maxd, draw: Draw):
        return self.L.orc_polymer_com(self.h, n, maxd, C.byref(draw.s))

    def energy(self):
        out = np.zeros(4)
        self.L.orc_energy(self.h, _dp(out))
        return out

    def superfluid(self):
        """W^2, A_z, sum r^2 / M of the current configuration"""
        out = np.zeros(3)
        self.L.orc_superfluid(self.h, _dp(out))
        return out

    def radial(self, nb, dr, hist=None):
        if hist is None:
            hist = np.zeros(nb)
        self.L.orc_radial(self.h, nb, dr, _dp(hist))
        return hist

    def density(self, nb, hist=None):
        if hist is None:
            hist = np.zeros(nb ** self.p.dim)
        self.L.orc_density(self.h, nb, _dp(hist))
        return hist

    def run(self, n, updates, seed=7, stream=0, ncycle=0, e_cap=0, dens_nb=0):
        """run!(s, n, updates; Zmeasurements): updates = list of
        (kind, every, var, minvar, maxvar, minacc, maxacc, adj, range)."""
        ups = (Update * len(updates))()
        for i, u in enumerate(updates):
            self.L.orc_update_init(C.byref(ups[i]), *u)
        r = Rng()
        self.L.orc_rng_init(C.byref(r), seed, stream)
        e = np.zeros(max(e_cap, 1) * 4)
        ec = C.c_long(0)
        hist = np.zeros(dens_nb ** self.p.dim) if dens_nb else None
        nd = C.c_long(0)
        st = RunStats()
        rc = self.L.orc_run(self.h, n, ups, len(updates), C.byref(r), ncycle, _dp(e), e_cap,
                            C.byref(ec), dens_nb, None if hist is None else _dp(hist),
                            C.byref(nd), C.byref(st))
        out = {
            "rc": rc,
            "energies": e[: ec.value * 4].reshape(-1, 4),
            "hist": hist, "ndata": nd.value,
            "attempts": list(st.attempts), "accepts": list(st.accepts),
            "bead_updates": st.bead_updates,
            "vars": [ups[i].var for i in range(len(updates))],
        }
        for i in range(len(updates)):
            self.L.orc_update_free(C.byref(ups[i]))
        return out


def run_sweeps(o: Oracle, nsweeps, ell, swaps, com, seed=7, stream=0, measure_every=0, e_cap=0,
               dens_nb=0):
    """nsweeps sweeps in the engine's schedule (orc_run_sweeps); com =
    [step, min, max, minacc, maxacc], its step updated in place"""
    r = Rng()
    o.L.orc_rng_init(C.byref(r), seed, stream)
    step = np.array([float(com[0])])
    e = np.zeros(max(e_cap, 1) * 4)
    ec = C.c_long(0)
    hist = np.zeros(dens_nb ** o.p.dim) if dens_nb else None
    nd = C.c_long(0)
    st = RunStats()
    rc = o.L.orc_run_sweeps(o.h, nsweeps, ell, swaps, _dp(step), com[1], com[2], com[3], com[4],
                            C.byref(r), measure_every, _dp(e), e_cap, C.byref(ec), dens_nb,
                            None if hist is None else _dp(hist), C.byref(nd), C.byref(st))
    com[0] = float(step[0])
    return {"rc": rc, "energies": e[: ec.value * 4].reshape(-1, 4), "hist": hist,
            "ndata": nd.value, "attempts": list(st.attempts), "accepts": list(st.accepts),
            "bead_updates": st.bead_updates}


def distance(a, b, L):
    return lib().orc_distance(a, b, L)


def teleport(x, L):
    return lib().orc_teleport(x, L)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return [int(v) for v in o]


def bench_chains(params: Params, nchains, nthreads, attempts, ell, com_step=1.0, seed=20261203):
    b = np.zeros(1)
    sec = lib().orc_bench_chains(C.byref(params), nchains, nthreads, attempts, ell, com_step,
                                 seed, _dp(b))
    return sec, float(b[0])


def bench_budget(params_list, ells, nthreads, budget_s, com_step=1.0, seed=20261203):
    """time-budgeted CPU rate of a list of chains (orc_bench_budget): the
    chains dealt longest-first to nthreads threads, every thread sweeping its
    own chains in turn until budget_s has passed.  Returns (wall seconds,
    bead updates, sweeps)."""
    n = len(params_list)
    arr = (Params * max(n, 1))(*params_list)
    el = (C.c_int * max(n, 1))(*[int(e) for e in ells])
    b, sw = np.zeros(1), np.zeros(1)
    wall = lib().orc_bench_budget(arr, el, n, int(nthreads), float(budget_s), float(com_step),
                                  int(seed), _dp(b), _dp(sw))
    return wall, float(b[0]), float(sw[0])
