"""CPU parity of the library's host-side box geometry (csrc/clm_geometry.hpp, what clm_set_box computes:
src/internals/Box.jl:191-270, CellOperations.jl:337-479) with the oracle's restatement, over random
orthorhombic and triclinic cells in 2D and 3D, Float32 and Float64: numbers of cells, cell sizes, the
computing box, the aligned cell and the rotations must be the same bits."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("geom") / "libgeom_probe.so")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-I", os.path.join(ROOT, "celllistmap.jl_gb300", "csrc"), os.path.join(ROOT, "tests", "geometry_probe.cpp"),
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(out)
    lib.geom_probe.restype = C.c_int
    return lib


KINDS = {"ortho": 0, "tri": 1}


def product_box(lib, M, dim, kind, cutoff, lcell, f64):
    Mc = np.ascontiguousarray(np.asarray(M, np.float64).reshape(dim, dim).flatten(order="F"))
    nc = np.zeros(dim, np.int64)
    arrs = [np.zeros(dim) for _ in range(3)] + [np.zeros(dim * dim) for _ in range(3)]
    st = lib.geom_probe(int(f64), dim, KINDS[kind], Mc.ctypes.data_as(C.c_void_p), C.c_double(cutoff), lcell,
                        nc.ctypes.data_as(C.c_void_p), *[a.ctypes.data_as(C.c_void_p) for a in arrs])
    return st, nc, arrs


def random_cells(rng, dim, kind, n):
    for _ in range(n):
        if kind == "ortho":
            yield np.diag(rng.uniform(10.0, 40.0, dim))
        else:
            M = np.diag(rng.uniform(10.0, 40.0, dim))
            M[np.triu_indices(dim, 1)] = rng.uniform(-5.0, 5.0, dim * (dim - 1) // 2)
            if rng.random() < 0.5:  # a general orientation, aligned by the library
                q, r = np.linalg.qr(rng.normal(size=(dim, dim)))
                q = q * np.sign(np.diag(r))
                if np.linalg.det(q) < 0:
                    q[:, 0] = -q[:, 0]
                M = q @ M
            yield M


@pytest.mark.parametrize("f64", [True, False])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_host_geometry_matches_oracle(probe, orc, f64, dim, kind):
    rng = np.random.default_rng(100 + dim + (7 if f64 else 0) + (3 if kind == "tri" else 0))
    checked = 0
    for M in random_cells(rng, dim, kind, 40):
        cutoff = float(rng.uniform(1.0, 4.0))
        lcell = int(rng.integers(1, 4))
        st, nc, (cs, lo, hi, mal, rot, rinv) = product_box(probe, M, dim, kind, cutoff, lcell, f64)
        dtype = np.float64 if f64 else np.float32
        try:
            b = orc.box_info(dim=dim, kind=kind, unitcell=M, cutoff=cutoff, lcell=lcell, dtype=dtype)
        except orc.OracleError as e:
            assert st == e.code  # both refuse the same cells (e.g. planes closer than 2 cutoffs)
            continue
        assert st == 0
        np.testing.assert_array_equal(nc, b["nc"])
        np.testing.assert_array_equal(cs, b["cell_size"])
        np.testing.assert_array_equal(lo, b["computing_box"][0])
        np.testing.assert_array_equal(hi, b["computing_box"][1])
        if kind == "tri":
            np.testing.assert_array_equal(mal.reshape(dim, dim, order="F"), b["aligned_unit_cell"])
            np.testing.assert_array_equal(rot.reshape(dim, dim, order="F"), b["rotation"])
            np.testing.assert_array_equal(rinv.reshape(dim, dim, order="F"), b["inv_rotation"])
        checked += 1
    assert checked >= 20


@pytest.mark.parametrize("f64", [True, False])
@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_host_geometry_random_sweep(probe, orc, f64, kind):
    # the reference's random-cell sweep (test/modules/Testing.jl:162-257): entries in [-10, 10] (negative
    # sides and left-handed cells included), cutoff in [1, 2]; accepted and refused cells and every field agree
    rng = np.random.default_rng(60 + (1 if f64 else 0) + (2 if kind == "tri" else 0))
    dtype = np.float64 if f64 else np.float32
    accepted = 0
    for _ in range(300):
        dim = int(rng.integers(2, 4))
        M = np.diag(-10 + 20 * rng.random(dim)) if kind == "ortho" else -10 + 20 * rng.random((dim, dim))
        cutoff, lcell = float(1 + rng.random()), int(rng.integers(1, 4))
        st, nc, (cs, lo, hi, mal, rot, rinv) = product_box(probe, M, dim, kind, cutoff, lcell, f64)
        try:
            b = orc.box_info(dim=dim, kind=kind, unitcell=np.diag(M) if kind == "ortho" else M, cutoff=cutoff,
                             lcell=lcell, dtype=dtype)
        except orc.OracleError as e:
            assert st == e.code
            continue
        assert st == 0
        np.testing.assert_array_equal(nc, b["nc"])
        np.testing.assert_array_equal(cs, b["cell_size"])
        np.testing.assert_array_equal(lo, b["computing_box"][0])
        np.testing.assert_array_equal(hi, b["computing_box"][1])
        if kind == "tri":
            np.testing.assert_array_equal(mal.reshape(dim, dim, order="F"), b["aligned_unit_cell"])
            np.testing.assert_array_equal(rot.reshape(dim, dim, order="F"), b["rotation"])
        accepted += 1
    assert accepted >= 50


@pytest.mark.parametrize("f64", [False, True])
def test_last_row_pruning_cell(probe, f64):
    """The benchmark's triclinic cell shape aligns to a matrix with exact zeros below the diagonal in its last
    row and a nonzero entry in the middle row: the build's image tests then prune on the last image index
    only (the branch the build-step tests check with this cell)."""
    M = np.array([[10.0, 2.0, 1.0], [0.0, 10.0, 1.5], [0.0, 0.0, 10.0]])
    st, nc, arrs = product_box(probe, M, 3, "tri", 1.5, 1, f64)
    assert st == 0
    mal = arrs[3].reshape(3, 3, order="F")
    assert mal[2, 0] == 0.0 and mal[2, 1] == 0.0
    assert mal[1, 0] != 0.0
