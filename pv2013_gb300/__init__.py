"""GB300-native lattice Boltzmann engine with the PV2013 solver's hot path:
STL voxelization, boundary classification and the D3Q19/D3Q27 BGK step with
Zou-He and bounce-back boundaries, as sm_103a CUDA kernels behind the C ABI
of include/lbm_gb300.h (liblbm_gb300.so, built in-tree)."""
from . import _capi
from ._capi import LbmError, load
from .engine import (BoundarySpec, Geometry, LatticeModel, PlanePredicate, Reader, Simulation, Snapshot,
                     pv2013_predicates, synth_capsules, synth_cylinder, write_vtu)

__all__ = ["BoundarySpec", "Geometry", "LatticeModel", "LbmError", "PlanePredicate", "Reader", "Simulation",
           "Snapshot", "load", "pv2013_predicates", "synth_capsules", "synth_cylinder", "write_vtu", "_capi"]
