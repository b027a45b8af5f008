"""Build and load the engine's C-ABI library (``include/pimc.h``).

The library is compiled in-tree for sm_103a with nvcc and loaded with ctypes.
There is no fallback: without the library (or without a GPU) every engine call
raises.
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes as C
import os
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
DIST_DIR = os.path.dirname(PKG_DIR)
REPO_DIR = os.path.dirname(DIST_DIR)
CSRC = os.path.join(DIST_DIR, "csrc")
BUILD_DIR = os.path.join(DIST_DIR, "_build")
LIB_DIR = os.path.join(DIST_DIR, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libpimc_gb300.so")
# the bounds-checking build (nvcc -DPIMC_CHECK=1): every window/slice and
# particle index, shared-scratch carve and neighbour-queue push is checked on
# the device, and a miss is reported as PIMC_EDEVICE instead of being
# performed.  load() picks it when the environment sets PIMC_CHECK=1.
LIB_CHECK_PATH = os.path.join(LIB_DIR, "libpimc_gb300_check.so")
# the profiling build (nvcc -DPIMC_PROFILE=1): per-section clock counters of
# the permutation swap (pimc_swap_profile); picked when PIMC_PROFILE=1
LIB_PROF_PATH = os.path.join(LIB_DIR, "libpimc_gb300_prof.so")
INCLUDE = os.path.join(REPO_DIR, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]
SOURCES = ["pimc_sweep.cu", "pimc_swap.cu", "pimc_fused.cu", "pimc_attempt.cu", "pimc_api.cu",
           "pimc_io.cpp"]


class PimcError(RuntimeError):
    """An engine call returned a non-zero status."""


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(verbose: bool = False, check: bool = False, profile: bool = False) -> str:
    """Compile csrc/*.cu for sm_103a into lib/libpimc_gb300.so (parallel TUs);
    check=True builds the bounds-checking variant lib/libpimc_gb300_check.so,
    profile=True the swap-profiling variant lib/libpimc_gb300_prof.so."""
    tag = "_check" if check else ("_prof" if profile else "")
    bdir = BUILD_DIR + tag
    out = LIB_CHECK_PATH if check else (LIB_PROF_PATH if profile else LIB_PATH)
    os.makedirs(bdir, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []
    extra = ["-DPIMC_CHECK=1"] if check else (["-DPIMC_PROFILE=1"] if profile else [])

    def compile_one(src):
        obj = os.path.join(bdir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise PimcError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = out + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise PimcError(f"link failed:\n{r.stderr}")
    os.replace(tmp, out)
    return out


def check_build_requested() -> bool:
    """PIMC_CHECK=1 in the environment selects the bounds-checking build"""
    return os.environ.get("PIMC_CHECK", "0") == "1"


# ------------------------------------------------------------------ structs
class Params(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("N", C.c_int), ("M", C.c_int),
        ("L", C.c_double), ("T", C.c_double), ("lam", C.c_double), ("mu", C.c_double),
        ("harmonic_omega", C.c_double), ("lattice_V0", C.c_double), ("lattice_a", C.c_double),
        ("interactions", C.c_int), ("pair_g", C.c_double), ("pair_sigma", C.c_double),
        ("r_a", C.c_double), ("hardcore_a", C.c_double), ("semantics", C.c_int),
        ("seed", C.c_uint64), ("density_nbins", C.c_int), ("energy_capacity", C.c_int),
        ("retry_cap", C.c_int),
    ]


class MoveMix(C.Structure):
    _fields_ = [
        ("staging_phases", C.c_int),
        ("stage_slices", C.c_int), ("stage_min", C.c_int), ("stage_max", C.c_int),
        ("stage_minacc", C.c_double), ("stage_maxacc", C.c_double),
        ("swaps_per_sweep", C.c_int),
        ("swap_slices", C.c_int), ("swap_min", C.c_int), ("swap_max", C.c_int),
        ("swap_minacc", C.c_double), ("swap_maxacc", C.c_double),
        ("com_phases", C.c_int),
        ("com_step", C.c_double), ("com_minstep", C.c_double), ("com_maxstep", C.c_double),
        ("com_minacc", C.c_double), ("com_maxacc", C.c_double),
        ("polymer_com_phases", C.c_int),
        ("pcom_step", C.c_double), ("pcom_minstep", C.c_double), ("pcom_maxstep", C.c_double),
        ("pcom_minacc", C.c_double), ("pcom_maxacc", C.c_double),
        ("adapt", C.c_int), ("measure_every", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("attempts", C.c_ulonglong * 4), ("accepts", C.c_ulonglong * 4),
        ("skips", C.c_ulonglong), ("bead_updates", C.c_double), ("sweeps", C.c_ulonglong),
        ("measurements", C.c_ulonglong), ("stage_slices", C.c_int), ("swap_slices", C.c_int),
        ("com_step", C.c_double), ("pcom_step", C.c_double),
        ("bead_updates_kind", C.c_double * 4),
    ]


class Launch(C.Structure):
    _fields_ = [("warp_per_chain", C.c_int), ("block", C.c_int),
                ("sweeps_per_launch", C.c_int), ("state_smem_bytes", C.c_int),
                ("split_phases", C.c_int), ("phase_block", C.c_int * 3),
                ("phase_warp", C.c_int * 3), ("phase_regs", C.c_int * 3),
                ("cell_lists", C.c_int)]


# every symbol include/pimc.h declares, with its argument types
_vp, _dp, _ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
_ull = C.POINTER(C.c_ulonglong)
SIGNATURES = {
    "pimc_create": [C.POINTER(Params), C.POINTER(C.c_void_p)],
    "pimc_batch_create": [C.POINTER(Params), C.c_int, C.POINTER(C.c_void_p)],
    "pimc_destroy": [_vp],
    "pimc_num_chains": [_vp, _ip],
    "pimc_set_beads": [_vp, _dp],
    "pimc_get_beads": [_vp, _dp],
    "pimc_set_next": [_vp, _ip],
    "pimc_get_next": [_vp, _ip],
    "pimc_set_raw": [_vp, _dp, _dp, _ip],
    "pimc_get_links": [_vp, _dp],
    "pimc_init_world": [_vp],
    "pimc_batch_set_beads": [_vp, C.c_int, _dp],
    "pimc_batch_get_beads": [_vp, C.c_int, _dp],
    "pimc_batch_get_next": [_vp, C.c_int, _ip],
    "pimc_batch_set_beads_all": [_vp, _dp],
    "pimc_batch_get_beads_all": [_vp, _dp],
    "pimc_batch_energy_sums_all": [_vp, _dp, _dp, _ull],
    "pimc_set_move_mix": [_vp, C.c_int, C.POINTER(MoveMix)],
    "pimc_run": [_vp, C.c_longlong],
    "pimc_batch_run": [_vp, C.c_longlong],
    "pimc_batch_run_plain": [_vp, C.c_longlong],
    "pimc_batch_run_io": [_vp, _dp, _dp, C.c_longlong, C.c_int],
    "pimc_batch_tune": [_vp, C.c_int, C.POINTER(Launch)],
    "pimc_batch_set_launch": [_vp, C.POINTER(Launch)],
    "pimc_batch_get_launch": [_vp, C.POINTER(Launch)],
    "pimc_attempt_staging": [_vp, C.c_int, C.c_int, C.c_int, _dp, C.c_int, _dp, C.c_int, _ip, _dp],
    "pimc_attempt_swap": [_vp, C.c_int, C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp, C.c_int,
                          _ip, _ip, _dp],
    "pimc_attempt_com": [_vp, C.c_int, C.c_double, _dp, C.c_int, _ip],
    "pimc_attempt_polymer_com": [_vp, C.c_int, C.c_double, _dp, C.c_int, _ip],
    "pimc_eval_action": [_vp, _dp],
    "pimc_eval_staging_weights": [_vp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp],
    "pimc_measure": [_vp],
    "pimc_get_energies": [_vp, C.c_int, _dp, C.c_int, _ip],
    "pimc_get_energy_sums": [_vp, C.c_int, _dp, _dp, _ull],
    "pimc_get_density": [_vp, C.c_int, _dp, _ull],
    "pimc_get_observables": [_vp, C.c_int, _dp, C.c_int, _ip],
    "pimc_get_observable_sums": [_vp, C.c_int, _dp, _dp, _ull],
    "pimc_set_radial": [_vp, C.c_int, C.c_int, C.c_double],
    "pimc_get_radial": [_vp, C.c_int, _dp, _ull],
    "pimc_get_params": [_vp, C.c_int, C.POINTER(Params)],
    "pimc_set_beams": [_vp, C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.c_int],
    "pimc_write_paths_csv": [_vp, C.c_int, C.c_char_p],
    "pimc_write_density_csv": [C.c_char_p, C.c_int, C.c_int, C.c_double, _dp, C.c_ulonglong],
    "pimc_save_checkpoint": [_vp, C.c_char_p],
    "pimc_load_checkpoint": [_vp, C.c_char_p],
    "pimc_format_float": [C.c_double, C.c_char_p, C.c_size_t],
    "pimc_reset_measurements": [_vp],
    "pimc_adjoint": [_vp, C.c_int, _dp, _dp, _dp],
    "pimc_adjoint_noalloc": [_vp, C.c_int, _dp, _dp, _dp],
    "pimc_batch_adjoint": [_vp, _dp, _dp, _dp],
    "pimc_set_potential": [_vp, C.c_int, C.c_double, C.c_double, C.c_double],
    "pimc_get_stats": [_vp, C.c_int, C.POINTER(Stats)],
    "pimc_get_total_stats": [_vp, C.POINTER(Stats)],
    "pimc_state_size": [_vp, C.POINTER(C.c_size_t)],
    "pimc_get_state": [_vp, C.c_void_p, C.c_size_t],
    "pimc_set_state": [_vp, C.c_void_p, C.c_size_t],
    "pimc_contact_table": [C.c_double, C.c_double, C.c_double, C.c_int, _dp],
    "pimc_set_contact_propagator": [_vp, C.c_int, C.c_double, C.c_double, C.c_int],
    "pimc_set_contact_table": [_vp, C.c_int, _dp, C.c_int, C.c_double],
    "pimc_get_contact_table": [_vp, C.c_int, _dp, C.c_size_t, _ip, _dp],
    "pimc_clear_contact": [_vp, C.c_int],
    "pimc_fp64_peak": [_vp, _dp],
    "pimc_batch_phase_times": [_vp, C.c_longlong, _dp],
    "pimc_swap_profile": [_vp, _ull, C.c_int],
    "pimc_device_info": [_vp, C.c_char_p, C.c_size_t, _ip],
    "pimc_last_run_ms": [_vp, _dp],
    "pimc_last_run_launches": [_vp, C.POINTER(C.c_longlong)],
    "pimc_set_option": [_vp, C.c_int, C.c_longlong],
    "pimc_last_error": [],
    "pimc_abi_version": [],
}

_lib = None


def load(path: str = None):
    """Load the built library (no fallback: a missing library raises).  The
    default is lib/libpimc_gb300.so, or the bounds-checking build when the
    environment sets PIMC_CHECK=1."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None:
        path = LIB_CHECK_PATH if check_build_requested() else LIB_PATH
        if os.environ.get("PIMC_PROFILE", "0") == "1":
            path = LIB_PROF_PATH
    if not os.path.exists(path):
        raise PimcError(f"engine library {path} is missing; run __graft_entry__.build()")
    L = C.CDLL(path)
    for name, args in SIGNATURES.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.pimc_last_error.restype = C.c_char_p
    _lib = L
    return L


def check(rc: int):
    if rc != 0:
        msg = _lib.pimc_last_error().decode() if _lib else "library not loaded"
        raise PimcError(f"pimc error {rc}: {msg}")
    return rc
