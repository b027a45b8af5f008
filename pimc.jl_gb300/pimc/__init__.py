"""GB300 engine for the PIMC.jl Monte Carlo sweep.

``pimc.api`` mirrors the reference package's Julia API (System, the update
callables, run/apply, Density, Energy); ``pimc.engine.Engine`` is the thin
handle wrapper over the C ABI in ``include/pimc.h``; ``pimc.build()``
compiles the CUDA library for sm_103a.
"""
from ._native import LIB_PATH, PimcError, build, load
from .api import (ContactPropagator, Counter, Density, Energy, GaussianPair, Harmonic,
                  NumbOfSlices, Particle, PolymerCenterOfMass, PotentialSum, RadialDistribution,
                  ReshapeLinear, ReshapeSwapLinear, SingleCenterOfMass, SquareLattice, Step,
                  Superfluid, System, Zero,
                  OpticalLattice, acceptance, apply, build_prop_int, density_filename,
                  determine_nnrange, generate_V, lattice_angles, load_checkpoint, run,
                  save_checkpoint, save_density, save_paths)
from .engine import (ACCEPT, HARDCORE, REJECT, SEM_PHYSICAL, SEM_REFERENCE, SKIP, ChainParams,
                     Engine, Mix, contact_table, julia_float, write_density_csv)

__all__ = [
    "build", "load", "LIB_PATH", "PimcError", "Engine", "ChainParams", "Mix", "System", "Particle",
    "Harmonic", "SquareLattice", "PotentialSum", "Zero", "GaussianPair", "ReshapeLinear",
    "ReshapeSwapLinear", "SingleCenterOfMass", "PolymerCenterOfMass", "Counter", "Step",
    "NumbOfSlices", "acceptance", "run", "apply", "Density", "Energy", "SEM_REFERENCE",
    "SEM_PHYSICAL", "ACCEPT", "REJECT", "SKIP", "HARDCORE", "ContactPropagator",
    "build_prop_int", "determine_nnrange", "contact_table", "RadialDistribution", "Superfluid",
    "save_paths", "save_density", "density_filename", "save_checkpoint", "load_checkpoint",
    "julia_float", "write_density_csv", "OpticalLattice", "generate_V", "lattice_angles",
]
