"""The drop-in for the reference's Python module (test/examples/CellListMap.py, docs/src/python.md):
`neighborlist(x, cutoff, unitcell=None)` and `neighborlist_cross(x, y, cutoff, unitcell=None)` returning
0-based int64 indices and float64 distances."""
import importlib
import os
import sys

import numpy as np
import pytest

PKG = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "celllistmap.jl_gb300")


def _module():
    if PKG not in sys.path:
        sys.path.insert(0, PKG)
    return importlib.import_module("CellListMap")


def test_module_imports_as_top_level():
    cl = _module()
    assert callable(cl.neighborlist) and callable(cl.neighborlist_cross)
    assert cl.neighborlist.__code__.co_varnames[:3] == ("x", "cutoff", "unitcell")
    assert cl.neighborlist_cross.__code__.co_varnames[:4] == ("x", "y", "cutoff", "unitcell")


def _canon(i, j, d):
    a = np.minimum(i, j)
    b = np.maximum(i, j)
    o = np.lexsort((b, a))
    return a[o], b[o], d[o]


@pytest.mark.gpu
@pytest.mark.parametrize("cell", ["none", "sides", "matrix"])
def test_neighborlist_like_the_reference_module(clm, orc, cell):
    cl = _module()
    rng = np.random.default_rng(12)
    coords = rng.random((20000, 3))
    if cell == "none":
        uc, kw = None, dict(kind="nonperiodic")
    elif cell == "sides":
        uc, kw = np.array([1, 1, 1]), dict(kind="ortho", unitcell=[1.0, 1.0, 1.0])
    else:
        uc = np.matrix("1 0 0; 0 1 0; 0 0 1")  # as in docs/src/python.md
        kw = dict(kind="tri", unitcell=np.eye(3))
    i, j, d = cl.neighborlist(coords, 0.05, unitcell=uc)
    assert i.dtype == np.int64 and j.dtype == np.int64 and d.dtype == np.float64
    assert i.min() >= 0 and max(i.max(), j.max()) < len(coords)  # 0-based
    ref = orc.run("nl", coords, cutoff=0.05, **kw)
    A, B = _canon(i, j, d), _canon(ref["i"], ref["j"], ref["d"])
    np.testing.assert_array_equal(A[0], B[0])
    np.testing.assert_array_equal(A[1], B[1])
    np.testing.assert_array_equal(A[2], B[2])


@pytest.mark.gpu
def test_neighborlist_cross_like_the_reference_module(clm, orc):
    cl = _module()
    rng = np.random.default_rng(13)
    x = rng.random((8000, 3))
    y = rng.random((6000, 3))
    i, j, d = cl.neighborlist_cross(x, y, 0.05, unitcell=np.array([1, 1, 1]))
    ref = orc.run("nl", x, y, kind="ortho", unitcell=[1.0, 1.0, 1.0], cutoff=0.05)
    a = np.lexsort((j, i))
    b = np.lexsort((ref["j"], ref["i"]))
    np.testing.assert_array_equal(i[a], ref["i"][b])
    np.testing.assert_array_equal(j[a], ref["j"][b])
    np.testing.assert_array_equal(d[a], ref["d"][b])
