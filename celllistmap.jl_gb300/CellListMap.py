"""Drop-in for the reference's Python module (test/examples/CellListMap.py:19-58, docs/src/python.md),
running on the GPU library instead of Julia.

    import CellListMap as cl               # with this package directory on sys.path
    i, j, d = cl.neighborlist(coords, 0.05)                            # non-periodic
    i, j, d = cl.neighborlist(coords, 0.05, unitcell=np.array([1, 1, 1]))
    i, j, d = cl.neighborlist_cross(x, y, 0.05, unitcell=np.array([1, 1, 1]))

Inputs are (N, dim) arrays (numpy, or torch tensors, CUDA tensors staying on the device), dim 2 or 3;
`unitcell` is None (non-periodic), a 1-D array of sides (orthorhombic) or a dim x dim matrix whose columns
are the cell vectors (general periodic cell).  Returns numpy arrays: 0-based int64 indices `i` (into x),
`j` (into x, or into y for the cross list) and float64 distances `d`, as the reference's module does.
Pairs are those with d <= cutoff; their order is unspecified, as in the reference.
"""
from __future__ import annotations

import numpy as np

try:
    from . import api as _api
except ImportError:  # imported as a top-level module from this directory
    import importlib.util as _ilu
    import os as _os
    import sys as _sys

    _here = _os.path.dirname(_os.path.abspath(__file__))
    _spec = _ilu.spec_from_file_location("celllistmap_gb300", _os.path.join(_here, "__init__.py"),
                                         submodule_search_locations=[_here])
    _pkg = _sys.modules.get("celllistmap_gb300") or _ilu.module_from_spec(_spec)
    if "celllistmap_gb300" not in _sys.modules:
        _sys.modules["celllistmap_gb300"] = _pkg
        _spec.loader.exec_module(_pkg)
    _api = _pkg.api


def _unitcell(unitcell):
    if unitcell is None:
        return None
    u = np.asarray(unitcell, dtype=np.float64)
    return u if u.ndim == 2 else u.reshape(-1)


def _as_numpy(i, j, d):
    return (np.asarray(i, dtype=np.int64), np.asarray(j, dtype=np.int64), np.asarray(d, dtype=np.float64))


def neighborlist(x, cutoff, unitcell=None):
    """Pairs of one set within the cutoff: 0-based (i, j, d) numpy arrays (test/examples/CellListMap.py:19-38)."""
    i, j, d = _api.neighborlist(xpositions=x, cutoff=float(cutoff), unitcell=_unitcell(unitcell))
    return _as_numpy(i, j, d)


def neighborlist_cross(x, y, cutoff, unitcell=None):
    """Pairs between two sets within the cutoff: 0-based (i into x, j into y, d) numpy arrays
    (test/examples/CellListMap.py:40-58)."""
    i, j, d = _api.neighborlist(xpositions=x, ypositions=y, cutoff=float(cutoff), unitcell=_unitcell(unitcell))
    return _as_numpy(i, j, d)
