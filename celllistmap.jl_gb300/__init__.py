"""celllistmap_gb300 — CellListMap.jl's cutoff-pair engine on NVIDIA GB300 (sm_103a).

Cell-list construction and the cell-pair map run as CUDA kernels in
``libcelllist_cuda.so`` (C ABI: include/celllistmap_gb300.h).  This package is
the host-side mirror of the reference's API for that path.

The directory name contains a dot, so import it through
``celllistmap_gb300 = load_package()`` from ``__graft_entry__`` or with
importlib (see ``tests/conftest.py``).
"""
from . import _abi
from . import api as _api
from .api import (ArgumentError, BatchedSystems, Box, CUDAError, DimensionMismatch, EnergyAndForces, InPlaceNeighborList,
                  ParticleSystem, device_allocations, neighborlist, neighborlist_, pairwise, pairwise_, update,
                  version)
from . import api as ops  # operator classes live in api; exposed as `ops`
from . import workloads
from . import trajectory
from . import autograd

Count = _api.Count
SumD2 = _api.SumD2
SumD = _api.SumD
SumInvD = _api.SumInvD
SoftEnergy = _api.SoftEnergy
SoftForces = _api.SoftForces
LennardJones = _api.LennardJones
LennardJonesForces = _api.LennardJonesForces
LennardJonesAdjoint = _api.LennardJonesAdjoint
InverseDistanceForces = _api.InverseDistanceForces
WeightedInverseDistance = _api.WeightedInverseDistance
MinimumDistance = _api.MinimumDistance
RadialHistogram = _api.RadialHistogram
NeighborList = _api.NeighborList

__all__ = [
    "ArgumentError", "BatchedSystems", "Box", "CUDAError", "DimensionMismatch", "EnergyAndForces", "InPlaceNeighborList",
    "ParticleSystem", "device_allocations", "neighborlist", "neighborlist_", "pairwise", "pairwise_", "update", "version", "ops",
    "Count", "SumD2", "SumD", "SumInvD", "SoftEnergy", "SoftForces", "LennardJones", "LennardJonesForces", "LennardJonesAdjoint",
    "InverseDistanceForces", "WeightedInverseDistance", "MinimumDistance", "RadialHistogram", "NeighborList",
]


def build(force: bool = False) -> str:
    """Compile libcelllist_cuda.so for sm_103a (nvcc)."""
    from . import build_lib
    return build_lib.build(force=force)
