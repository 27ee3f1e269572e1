"""CPU parity of the library's cell-list build steps with the oracle's serial cell list.

tests/build_probe.cpp compiles the per-particle and per-copy steps the build kernels run on the device
(csrc/clm_build_steps.cuh: the device geometry, wrap into the first cell and image tests, the cell keys of
each copy, the gather of the copy coordinates in cell order) for the host and drives them one particle at a
time.  The copies, their cells (with the border-case shift of real particles), their in-cell order, realness
and coordinates must equal the oracle's (src/internals/CellLists.jl:727-1057, Box.jl:499-566) bit for bit, in
Float64 and Float32, for orthorhombic, triclinic and non-periodic boxes in 2D and 3D, and over the
reference's pathological coordinates and random cells (test/modules/Testing.jl:36-60, 162-257).

The pair kernel's decisions are checked the same way (csrc/clm_device.cuh): its stencil lists the
reference's forward and full neighbour cells in the reference's order; its shortcut around the projection
filter keeps only pairs the filter keeps; the self and x-y maps emulated from its pieces give the oracle's
neighbour lists with bit-identical distances; the split form's FP32 distance error stays within the bound
its histogram guard uses, and the bin search and re-decision window decide the bins exactly.  These run
without a GPU; the GPU tests check the kernels themselves.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

KINDS = {"ortho": 0, "tri": 1, "nonperiodic": 2}
DERR_NAN = 1


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    cuda_inc = None
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "include", "cuda_runtime.h")):
            cuda_inc = os.path.join(cand, "include")
            break
    if cxx is None or cuda_inc is None:
        pytest.skip("no C++ compiler or CUDA headers")
    out = str(tmp_path_factory.mktemp("build_steps") / "libbuild_probe.so")
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-I", cuda_inc,
           "-I", os.path.join(ROOT, "celllistmap.jl_gb300", "csrc"), os.path.join(ROOT, "tests", "build_probe.cpp"),
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(out)
    lib.build_probe.restype = C.c_int
    return lib


def kind_of(uc):
    if uc is None:
        return "nonperiodic"
    return "ortho" if np.asarray(uc).ndim == 1 else "tri"


def host_celllist(lib, x, dim, kind, unitcell, cutoff, lcell, dtype):
    """Cell list from the library's build steps run on the host: same fields as the oracle's celllist()."""
    x = np.ascontiguousarray(np.asarray(x, dtype).astype(np.float64)).reshape(-1, dim)
    n = x.shape[0]
    if unitcell is None:
        Mc = np.zeros(dim * dim)
    else:
        uc = np.asarray(unitcell, np.float64)
        M = np.diag(uc) if uc.ndim == 1 else uc.reshape(dim, dim)
        Mc = np.ascontiguousarray(M.flatten(order="F"))
    f64 = int(np.dtype(dtype) == np.float64)
    ncopy, nreal, err = C.c_int64(0), C.c_int64(0), C.c_int(0)
    vp = C.c_void_p

    def call(cap, *arrs):
        return lib.build_probe(f64, dim, KINDS[kind], Mc.ctypes.data_as(vp), C.c_double(cutoff), lcell,
                               x.ctypes.data_as(vp), n, C.c_int64(cap), C.byref(ncopy), C.byref(nreal),
                               *[a.ctypes.data_as(vp) if a is not None else None for a in arrs], C.byref(err))

    st = call(0, None, None, None, None)
    if st:
        return st, None
    m = ncopy.value
    cell, idx = np.zeros(m, np.int64), np.zeros(m, np.int64)
    real, coords = np.zeros(m, np.int8), np.zeros((m, dim), np.float64)
    st = call(m, cell, idx, real, coords)
    assert st == 0, st
    return 0, {"cell": cell, "index": idx, "real": real.astype(bool), "coords": coords,
               "n_cells_with_real": nreal.value, "err": err.value}


def assert_same_celllist(got, ref):
    assert got["err"] == 0
    assert len(got["cell"]) == len(ref["cell"])
    np.testing.assert_array_equal(got["cell"], ref["cell"])
    np.testing.assert_array_equal(got["index"], ref["index"])
    np.testing.assert_array_equal(got["real"], ref["real"])
    np.testing.assert_array_equal(got["coords"], ref["coords"])
    assert got["n_cells_with_real"] == ref["n_cells_with_real"]


CASES = [
    # dim, unitcell, cutoff, lcell, n, span, shift
    (3, [10.0, 12.0, 11.0], 1.5, 1, 3000, 12.0, -1.0),
    (3, [10.0, 12.0, 11.0], 1.5, 2, 3000, 12.0, -1.0),
    (3, [10.0, 12.0, 11.0], 1.5, 3, 1000, 40.0, -20.0),
    (3, [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]], 1.5, 1, 3000, 12.0, -1.0),
    (3, [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]], 1.5, 3, 2000, 12.0, -1.0),
    (3, [[9.0, 0.5, -1.0], [1.0, 11.0, 0.5], [-0.5, 1.5, 12.0]], 2.0, 2, 2000, 30.0, -15.0),
    # the benchmark's cell shape: its aligned cell has zeros below the diagonal in the last row only, so the
    # image tests take their per-s_last pruning (test_geometry.py::test_last_row_pruning_cell)
    (3, [[10.0, 2.0, 1.0], [0.0, 10.0, 1.5], [0.0, 0.0, 10.0]], 1.5, 1, 3000, 12.0, -1.0),
    (3, None, 1.5, 1, 3000, 12.0, -1.0),
    (3, None, 1.5, 2, 2000, 12.0, -1.0),
    (2, [10.0, 12.0], 1.2, 1, 2000, 12.0, -1.0),
    (2, [[10.0, 3.0], [0.0, 11.0]], 1.2, 2, 2000, 12.0, -1.0),
    (2, [[10.0, 3.0], [1.0, 11.0]], 1.2, 1, 2000, 30.0, -15.0),
    (2, None, 1.2, 1, 2000, 12.0, -1.0),
]


def case_id(c):
    dim, uc, cut, lcell, n, span, shift = c
    return f"{dim}d-{kind_of(uc)}-lcell{lcell}-span{span:g}"


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_build_steps_match_oracle(probe, orc, case, dtype):
    dim, uc, cut, lcell, n, span, shift = case
    rng = np.random.default_rng(11 + lcell + dim)
    x = (rng.random((n, dim)) * span + shift).astype(dtype)
    kw = dict(dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    st, got = host_celllist(probe, x, dim, kind_of(uc), uc, cut, lcell, dtype)
    assert st == 0
    assert_same_celllist(got, orc.celllist(x, **kw))


def _pathological(rng, n, sides):
    # test/modules/Testing.jl:36-60: points on faces, +-nextfloat(0), outside the box
    x = sides * rng.random((n, 3))
    tiny, mtiny = np.nextafter(0, 1), np.nextafter(0, -1)
    x[0] = -sides / 2
    x[1] = -sides / 2 + [tiny, tiny, sides[2] * rng.random()]
    x[2] = -sides / 2 + [mtiny, mtiny, sides[2] * rng.random()]
    x[3] = sides / 2 + [tiny, tiny, sides[2] * rng.random()]
    x[4] = sides / 2 + [mtiny, mtiny, sides[2] * rng.random()]
    x[9] = sides
    x[10] = sides + [tiny, tiny, sides[2] * rng.random()]
    x[11] = sides + [mtiny, mtiny, sides[2] * rng.random()]
    x[12] = [tiny, tiny, sides[2] * rng.random()]
    x[13] = [mtiny, mtiny, sides[2] * rng.random()]
    x[14] = 0.0
    x[99] = [sides[0] / 2, -sides[1] / 2, 2 * sides[2]]
    return x


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("lcell", [1, 2])
def test_pathological_coordinates(probe, orc, lcell, dtype):
    rng = np.random.default_rng(5)
    sides = np.array([250.0, 250.0, 250.0])
    x = _pathological(rng, 200, sides).astype(dtype)
    for uc in (sides, np.array([[250.0, 30.0, 10.0], [0.0, 250.0, 20.0], [0.0, 0.0, 250.0]])):
        kind = kind_of(uc)
        st, got = host_celllist(probe, x, 3, kind, uc, 10.0, lcell, dtype)
        assert st == 0
        assert_same_celllist(got, orc.celllist(x, dim=3, kind=kind, unitcell=uc, cutoff=10.0, lcell=lcell,
                                               dtype=dtype))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_particles_on_cell_boundaries(probe, orc, dtype):
    # every particle on a cell face, an edge or a corner of the cell grid (and on the unit-cell faces): the
    # border cases of the cell index and of the image tests
    side, cut = 12.0, 1.5
    g = np.arange(0.0, side + 1e-9, cut / 2)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    x = np.concatenate([pts, pts - side, pts + 0.5 * side]).astype(dtype)
    for lcell in (1, 2, 3):
        for uc in ([side, side, side], [[side, 3.0, 0.0], [0.0, side, 3.0], [0.0, 0.0, side]]):
            kind = kind_of(uc)
            st, got = host_celllist(probe, x, 3, kind, uc, cut, lcell, dtype)
            assert st == 0
            assert_same_celllist(got, orc.celllist(x, dim=3, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell,
                                                   dtype=dtype))


@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_random_cells_sweep(probe, orc, kind):
    # test/modules/Testing.jl:162-257: random cells with entries in [-10, 10] (negative sides, left-handed
    # cells), cutoff in [1, 2], lcell 1..3, 10-20 points far outside the cell; the cells the oracle refuses the
    # library's geometry refuses with the same code
    rng = np.random.default_rng(21 if kind == "ortho" else 22)
    done = 0
    for trial in range(2000):
        dim = int(rng.integers(2, 4))
        lcell = int(rng.integers(1, 4))
        M = np.diag(-10 + 20 * rng.random(dim)) if kind == "ortho" else -10 + 20 * rng.random((dim, dim))
        uc = np.diag(M) if kind == "ortho" else M
        cut = float(1 + rng.random())
        dtype = np.float64 if trial % 2 == 0 else np.float32
        x = (10 * rng.random((int(rng.integers(10, 21)), dim)) - 50).astype(dtype)
        kw = dict(dim=dim, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
        try:
            b = orc.box_info(**kw)
        except orc.OracleError as e:
            st, _ = host_celllist(probe, x, dim, kind, uc, cut, lcell, dtype)
            assert st == e.code
            continue
        if np.prod(b["nc"]) > 200000:
            continue
        st, got = host_celllist(probe, x, dim, kind, uc, cut, lcell, dtype)
        assert st == 0
        assert_same_celllist(got, orc.celllist(x, **kw))
        done += 1
        if done == 150:
            break
    assert done == 150


def test_nan_particle_gets_no_copy(probe):
    # a NaN coordinate is flagged and the particle gets no copy (the library then reports the reference's
    # "Invalid coordinates found (NaN)" error instead of returning the list)
    rng = np.random.default_rng(2)
    x = rng.random((50, 3)) * 10.0
    x[7, 1] = np.nan
    st, got = host_celllist(probe, x, 3, "ortho", [10.0, 10.0, 10.0], 1.0, 1, np.float64)
    assert st == 0
    assert got["err"] & DERR_NAN
    assert 7 not in set(got["index"].tolist())


def test_empty_set(probe):
    st, got = host_celllist(probe, np.zeros((0, 3)), 3, "ortho", [10.0, 10.0, 10.0], 1.0, 1, np.float64)
    assert st == 0
    assert len(got["cell"]) == 0 and got["n_cells_with_real"] == 0


def _cartesian(ranges):
    # Julia's CartesianIndices order: first index fastest
    import itertools
    return [tuple(reversed(t)) for t in itertools.product(*reversed(ranges))]


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("lcell", [1, 2, 3, 5])
def test_stencil_in_the_reference_order(probe, dim, lcell):
    # neighbor_cells_forward / neighbor_cells (src/internals/Box.jl:436-474), element by element
    l = lcell
    full_r = range(-l, l + 1)
    if dim == 3:
        fwd = (_cartesian([range(1, l + 1), full_r, full_r]) + _cartesian([range(0, 1), range(1, l + 1), full_r])
               + _cartesian([range(0, 1), range(0, 1), range(1, l + 1)]))
    else:
        fwd = _cartesian([range(1, l + 1), full_r]) + _cartesian([range(0, 1), range(1, l + 1)])
    full = [t for t in _cartesian([full_r] * dim) if any(t)]
    assert len(fwd) * 2 == len(full)
    o = (C.c_int * 3)()
    for forward, want in ((1, fwd), (0, full)):
        for fixed1 in ((0, 1) if l == 1 else (0,)):
            got = []
            for k in range(len(want)):
                probe.stencil_probe(forward, l, fixed1, dim, k, o)
                got.append(tuple(o[:dim]))
            assert got == want


def band_counts(lib, x, dim, kind, unitcell, cutoff, lcell, dtype):
    x = np.ascontiguousarray(np.asarray(x, dtype).astype(np.float64)).reshape(-1, dim)
    if unitcell is None:
        Mc = np.zeros(dim * dim)
    else:
        uc = np.asarray(unitcell, np.float64)
        Mc = np.ascontiguousarray((np.diag(uc) if uc.ndim == 1 else uc.reshape(dim, dim)).flatten(order="F"))
    out = np.zeros(5, np.int64)
    st = lib.band_probe(int(np.dtype(dtype) == np.float64), dim, KINDS[kind], Mc.ctypes.data_as(C.c_void_p),
                        C.c_double(cutoff), lcell, x.ctypes.data_as(C.c_void_p), x.shape[0],
                        out.ctypes.data_as(C.c_void_p))
    return st, out


BAND_CELLS = [
    (3, [20.0, 20.0, 20.0]),
    (3, [[20.0, 4.0, 2.0], [0.0, 20.0, 3.0], [0.0, 0.0, 20.0]]),
    (3, [[14.0, 9.0, -6.0], [1.0, 15.0, 7.0], [-2.0, 3.0, 16.0]]),
    (3, None),
    (2, [30.0, 25.0]),
    (2, [[30.0, 14.0], [0.0, 25.0]]),
    (2, [[24.0, -11.0], [5.0, 26.0]]),
    (2, None),
]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("lcell", [1, 2, 3])
@pytest.mark.parametrize("cell", BAND_CELLS, ids=lambda c: f"{c[0]}d-{kind_of(c[1])}")
def test_projection_filter_passes_inside_the_band(probe, cell, lcell, dtype):
    # The pair kernel evaluates the reference's projection filter (vicinal_cells.jl:4-75) only for pairs with
    # d2 > rc^2 (1 - 2^-13) (and accepts a pair whose FP32 distance is below that bound: the fma test on the
    # coordinates for Float32 handles, on the cell-relative offsets in the split form for Float64 handles).  The filter keeps every pair well inside the cutoff: |(x_j - x_i).u| <= d < rc, and the
    # particle's projection on the cell-pair axis is at most half the centre distance (lcell 1) or
    # rc sqrt(N)/2 (lcell > 1), inside the margins.  Checked over every pair of the full stencil.
    dim, uc = cell
    rng = np.random.default_rng(40 + lcell + dim)
    n = 6000 if dim == 3 else 3000
    span = 20.0 if dim == 3 else 28.0
    x = (rng.random((n, dim)) * span - 3.0).astype(dtype)
    st, out = band_counts(probe, x, dim, kind_of(uc), uc, 2.0, lcell, dtype)
    assert st == 0
    within, shortcut, banded, rejected, violations = out.tolist()
    assert violations == 0
    assert shortcut > 0.99 * within > 0 and banded > 0 and rejected <= banded


def test_real_particle_border_case(probe):
    # test/internals/CellLists.jl:161-190: Box([1, 1, 1], 0.1, lcell=1); a real particle in cell lcell moves
    # to lcell + 1, one in cell nc - lcell + 1 moves to nc - lcell, per dimension; an image is not moved
    M = np.ascontiguousarray(np.eye(3).flatten(order="F"))
    cart, nc = (C.c_int * 3)(), (C.c_int * 3)()

    def cell(x, real, lcell=1):
        xa = np.ascontiguousarray(x, np.float64)
        li = probe.cell_probe(3, KINDS["ortho"], M.ctypes.data_as(C.c_void_p), C.c_double(0.1), lcell,
                              xa.ctypes.data_as(C.c_void_p), int(real), cart, nc)
        assert li >= 0
        return tuple(cart), tuple(nc)

    h = 0.1  # cell side; cell c (1-based) spans [-0.1 + (c - 1) h, -0.1 + c h)
    centre = lambda c: -0.1 + (c - 0.5) * h  # noqa: E731
    (c1, n1) = cell([centre(1), centre(2), centre(3)], True)
    assert n1 == (13, 13, 13)  # floor(1 / 0.1) + 2 lcell + 1
    assert c1 == (2, 2, 3)
    c2, _ = cell([centre(13), centre(2), centre(3)], True)
    assert c2 == (12, 2, 3)
    c3, _ = cell([centre(1), centre(13), centre(6)], True)
    assert c3 == (2, 12, 6)
    c4, _ = cell([centre(1), centre(13), centre(6)], False)  # images keep their cell
    assert c4 == (1, 13, 6)


def host_map_nl(lib, x, dim, kind, unitcell, cutoff, lcell, dtype):
    """Self-pair neighbour list of the pair kernel's logic emulated on the host (tests/build_probe.cpp
    map_nl): returns (status, i, j, d, lost), `lost` counting exact hits the FP32 pass would drop."""
    x = np.ascontiguousarray(np.asarray(x, dtype).astype(np.float64)).reshape(-1, dim)
    if unitcell is None:
        Mc = np.zeros(dim * dim)
    else:
        uc = np.asarray(unitcell, np.float64)
        Mc = np.ascontiguousarray((np.diag(uc) if uc.ndim == 1 else uc.reshape(dim, dim)).flatten(order="F"))
    lib.map_nl_probe.restype = C.c_int64
    lost, st = C.c_int64(0), C.c_int(0)
    vp = C.c_void_p

    def call(cap, i, j, d):
        return lib.map_nl_probe(int(np.dtype(dtype) == np.float64), dim, KINDS[kind], Mc.ctypes.data_as(vp),
                                C.c_double(cutoff), lcell, x.ctypes.data_as(vp), x.shape[0], C.c_int64(cap),
                                i.ctypes.data_as(vp), j.ctypes.data_as(vp), d.ctypes.data_as(vp), C.byref(lost),
                                C.byref(st))

    e = np.zeros(1, np.int64)
    m = call(0, e, e, e.astype(np.float64))
    if st.value:
        return st.value, None, None, None, None
    i, j, d = np.zeros(m, np.int64), np.zeros(m, np.int64), np.zeros(m, np.float64)
    assert call(m, i, j, d) == m
    return 0, i, j, d, lost.value


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_emulated_map_matches_oracle_neighbor_list(probe, orc, case, dtype):
    # The pair kernel's self-pair logic (cells with real particles, stencil, pair rule, exact test, band and
    # projection filter) driven on the host over the host-built cell list: the same pairs and bit-identical
    # distances as the oracle (src/internals/self.jl:106-184), and no exact hit the FP32 pass would drop.
    dim, uc, cut, lcell, n, span, shift = case
    rng = np.random.default_rng(21 + lcell + dim)
    x = (rng.random((n, dim)) * span + shift).astype(dtype)
    st, i, j, d, lost = host_map_nl(probe, x, dim, kind_of(uc), uc, cut, lcell, dtype)
    assert st == 0 and lost == 0
    ref = orc.run("nl", x, dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    A, B = orc.canonical_pairs(i, j, d), orc.canonical_pairs(ref["i"], ref["j"], ref["d"])
    assert len(A[0]) == len(B[0]) > 0
    for u, v in zip(A, B):
        np.testing.assert_array_equal(u, np.asarray(v, u.dtype))


def test_emulated_map_pathological_and_random_cells(probe, orc):
    # the same emulation over the reference's pathological coordinates (test/modules/Testing.jl:36-60) and
    # its random-cell sweep (test/modules/Testing.jl:162-257: entries in [-10, 10], points far outside)
    rng = np.random.default_rng(8)
    sides = np.array([250.0, 250.0, 250.0])
    xp = _pathological(rng, 500, sides)
    checks = [(xp, 3, uc, 10.0, lcell) for lcell in (1, 2)
              for uc in (sides, np.array([[250.0, 30.0, 10.0], [0.0, 250.0, 20.0], [0.0, 0.0, 250.0]]))]
    done = 0
    for _ in range(600):
        dim = int(rng.integers(2, 4))
        kind = "ortho" if rng.random() < 0.3 else "tri"
        M = np.diag(-10 + 20 * rng.random(dim)) if kind == "ortho" else -10 + 20 * rng.random((dim, dim))
        uc = np.diag(M) if kind == "ortho" else M
        cut, lcell = float(1 + rng.random()), int(rng.integers(1, 4))
        try:
            b = orc.box_info(dim=dim, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell)
        except orc.OracleError:
            continue
        if np.prod(b["nc"]) > 100000:
            continue
        checks.append((10 * rng.random((int(rng.integers(10, 60)), dim)) - 50, dim, uc, cut, lcell))
        done += 1
        if done == 80:
            break
    assert done == 80
    for x, dim, uc, cut, lcell in checks:
        for dtype in (np.float64, np.float32):
            kind = kind_of(uc)
            st, i, j, d, lost = host_map_nl(probe, x, dim, kind, uc, cut, lcell, dtype)
            assert st == 0 and lost == 0
            ref = orc.run("nl", x, dim=dim, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
            A, B = orc.canonical_pairs(i, j, d), orc.canonical_pairs(ref["i"], ref["j"], ref["d"])
            assert len(A[0]) == len(B[0])
            for u, v in zip(A, B):
                np.testing.assert_array_equal(u, np.asarray(v, u.dtype))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_emulated_cross_map_matches_oracle(probe, orc, case, dtype):
    # the kernel's x-y pair logic emulated on the host (tests/build_probe.cpp map_cross) against the oracle's
    # two-set neighbour list (src/internals/cross.jl:8-129): same (i, j) pairs, bit-identical distances
    dim, uc, cut, lcell, n, span, shift = case
    rng = np.random.default_rng(31 + lcell + dim)
    x = (rng.random((n, dim)) * span + shift).astype(dtype)
    y = (rng.random((n // 2 + 7, dim)) * span + shift).astype(dtype)
    if uc is None:
        Mc = np.zeros(dim * dim)
    else:
        u = np.asarray(uc, np.float64)
        Mc = np.ascontiguousarray((np.diag(u) if u.ndim == 1 else u).flatten(order="F"))
    xd, yd = (np.ascontiguousarray(a.astype(np.float64)) for a in (x, y))
    probe.map_cross_probe.restype = C.c_int64
    lost, st = C.c_int64(0), C.c_int(0)
    vp = C.c_void_p

    def call(cap, i, j, d):
        return probe.map_cross_probe(int(np.dtype(dtype) == np.float64), dim, KINDS[kind_of(uc)],
                                     Mc.ctypes.data_as(vp), C.c_double(cut), lcell, xd.ctypes.data_as(vp), len(x),
                                     yd.ctypes.data_as(vp), len(y), C.c_int64(cap), i.ctypes.data_as(vp),
                                     j.ctypes.data_as(vp), d.ctypes.data_as(vp), C.byref(lost), C.byref(st))

    e = np.zeros(1, np.int64)
    m = call(0, e, e, e.astype(np.float64))
    assert st.value == 0 and m > 0
    i, j, d = np.zeros(m, np.int64), np.zeros(m, np.int64), np.zeros(m, np.float64)
    assert call(m, i, j, d) == m and lost.value == 0
    ref = orc.run("nl", x, y, dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    a, b = np.lexsort((j, i)), np.lexsort((ref["j"], ref["i"]))
    np.testing.assert_array_equal(i[a], ref["i"][b])
    np.testing.assert_array_equal(j[a], ref["j"][b])
    np.testing.assert_array_equal(d[a], np.asarray(ref["d"][b], np.float64))


SPLIT_CELLS = [
    (3, [250.0, 250.0, 250.0], 25.0, 20000, 250.0, 0.0),
    (3, [[20.0, 4.0, 2.0], [0.0, 20.0, 3.0], [0.0, 0.0, 20.0]], 2.0, 20000, 20.0, -3.0),
    (2, [30.0, 30.0], 2.0, 5000, 30.0, 0.0),
    (2, [[30.0, 12.0], [0.0, 28.0]], 2.0, 5000, 40.0, -5.0),
]


@pytest.mark.parametrize("lcell", [1, 2, 3])
@pytest.mark.parametrize("cell", SPLIT_CELLS, ids=lambda c: f"{c[0]}d-{kind_of(c[1])}")
def test_split_distance_error_within_bound(probe, cell, lcell):
    # the FP32 distance of the split form (cell-relative FP32 offsets, cell shift fused or not) differs from
    # the exact one by less than the library's bound split_distance_error, over every pair within the cutoff
    dim, uc, cut, n, span, shift = cell
    x = np.ascontiguousarray(np.random.default_rng(50 + lcell).random((n, dim)) * span + shift)
    u = np.asarray(uc, np.float64)
    Mc = np.ascontiguousarray((np.diag(u) if u.ndim == 1 else u).flatten(order="F"))
    worst = C.c_double()
    assert probe.split_error_probe(dim, KINDS[kind_of(uc)], Mc.ctypes.data_as(C.c_void_p), C.c_double(cut), lcell,
                                   x.ctypes.data_as(C.c_void_p), n, C.byref(worst)) == 0
    assert 0.0 < worst.value < 1.0


def test_split_histogram_guard(probe):
    # split-form histograms keep the exact bins only for edges above the FP32 distance error window; the
    # library runs finer edges in the exact form.  The two-set 2 x 2M workload's edges (first 0.1, cutoff 25
    # in a 250 box) stay in the split form.
    M = np.ascontiguousarray(np.diag([250.0] * 3).flatten(order="F"))
    rmin = C.c_double()

    def guard(edges, lcell=1):
        e = np.ascontiguousarray(edges, np.float64)
        return probe.split_bins_probe(3, KINDS["ortho"], M.ctypes.data_as(C.c_void_p), C.c_double(25.0), lcell,
                                      e.ctypes.data_as(C.c_void_p), len(e), C.byref(rmin))

    bins = 10.0 ** np.linspace(np.log10(0.1), np.log10(25.0), 51)
    assert guard(bins) == 1
    assert rmin.value == pytest.approx(np.sqrt(3) * 8 * 25.0 * 2.0 ** -12) and rmin.value < 0.1
    assert guard(np.concatenate([[0.05], bins])) == 0
    assert guard(np.arange(0.0, 26.0)) == 1  # an edge at 0 separates only pairs at distance 0


def test_histogram_bin_search(probe):
    # the kernel's bin of a distance r: searchsortedfirst(edges, r) - 1 (test/examples/pairwise_velocities.jl:
    # 17-24): an r on an edge goes to the lower bin, r <= edges[0] and r > edges[-1] to none
    probe.bin_probe.argtypes = [C.c_void_p, C.c_int, C.c_double]
    edges = np.ascontiguousarray(10.0 ** np.linspace(-1, np.log10(25.0), 51))
    rng = np.random.default_rng(3)
    rs = np.concatenate([edges, np.nextafter(edges, 0), np.nextafter(edges, 30), rng.uniform(0, 30, 2000), [0.0]])
    for r in rs:
        lo = probe.bin_probe(edges.ctypes.data, 50, float(r))
        assert lo == np.searchsorted(edges, r, side="left"), r


def test_split_bin_window_covers_the_error(probe):
    # an FP32 distance within the split form's error bound of the exact one: whenever it falls in another
    # bin than the exact distance, the window sends the pair to the exact decision (edges above the guard's
    # bound; the 2 x 2M workload: cutoff 25 in a 250 box, lcell 1)
    probe.bin_probe.argtypes = [C.c_void_p, C.c_int, C.c_double]
    probe.near_edge_probe.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_void_p]
    edges = np.ascontiguousarray(10.0 ** np.linspace(-1, np.log10(25.0), 51))
    ef = np.ascontiguousarray(edges.astype(np.float32))
    err = np.sqrt(3) * 8 * 25.0 * 2.0 ** -24  # split_distance_error of that geometry
    assert edges[0] > err * 4096
    rng = np.random.default_rng(4)
    lo = C.c_int()
    flagged = 0
    for e in edges:
        for r in e + rng.uniform(-3 * err, 3 * err, 200):
            b_exact = probe.bin_probe(edges.ctypes.data, 50, float(r)) - 1
            for rf in (np.float32(r + err), np.float32(r - err), np.float32(r)):
                near = probe.near_edge_probe(ef.ctypes.data, 50, float(rf), C.byref(lo))
                if lo.value - 1 != b_exact:
                    assert near == 1, (e, r, rf)
                flagged += near
    assert flagged > 0


@pytest.mark.parametrize("dim", [3, 2])
def test_emulated_split_histogram_counts(probe, orc, dim):
    # the split form's binning composed over every x-y pair of a sample with the two-set workload's geometry
    # (box 250, cutoff 25, 50 log-spaced edges from 0.1): the same counts as the oracle's exact histogram
    rng = np.random.default_rng(12 + dim)
    n = 20000 if dim == 3 else 4000
    x = np.ascontiguousarray(rng.random((n, dim)) * 250.0)
    y = np.ascontiguousarray(rng.random((n, dim)) * 250.0)
    edges = np.ascontiguousarray(10.0 ** np.linspace(-1, np.log10(25.0), 51))
    Mc = np.ascontiguousarray(np.diag([250.0] * dim).flatten(order="F"))
    counts = np.zeros(50, np.int64)
    st = C.c_int()
    probe.split_hist_probe.restype = C.c_int64
    vp = C.c_void_p
    m = probe.split_hist_probe(dim, KINDS["ortho"], Mc.ctypes.data_as(vp), C.c_double(25.0), 1, x.ctypes.data_as(vp),
                               n, y.ctypes.data_as(vp), n, edges.ctypes.data_as(vp), 50, counts.ctypes.data_as(vp),
                               C.byref(st))
    assert st.value == 0 and m == counts.sum() > 0
    r = orc.run("rhist", x, y, dim=dim, unitcell=[250.0] * dim, cutoff=25.0, bins=edges, vel_x=np.zeros_like(x),
                vel_y=np.zeros_like(y))
    np.testing.assert_array_equal(counts, r["hist_count"])


def test_noalloc_scratch_slots(probe):
    # the allocation-free entry point's static scratch (128 KiB + 256 B: a 256-byte result area, then one
    # slot per block of an energy, a count, a minimum d2 in the handle dtype and its pair of indices) holds
    # 4096 blocks for Float64 handles and 4681 for Float32 ones; a launch of more blocks is refused
    # (CLM_ERR_CAPACITY), which a GB300 never needs (at most 6 blocks per SM x 152 SMs)
    probe.noalloc_slots_probe.restype = C.c_longlong
    probe.noalloc_slots_probe.argtypes = [C.c_longlong, C.c_int]
    assert probe.noalloc_slots_probe(128 * 1024 + 256, 8) == 4096
    assert probe.noalloc_slots_probe(128 * 1024 + 256, 4) == 4681
    assert probe.noalloc_slots_probe(256, 8) == 0
    assert probe.noalloc_slots_probe(100, 8) == 0
    assert probe.noalloc_slots_probe(256 + 31, 8) == 0 and probe.noalloc_slots_probe(256 + 32, 8) == 1


def test_pair_rule_parts_equal_pair_rule(probe):
    # the pair kernel applies the reference's pair rules (pair_rule) in three parts: pairs of two images
    # dropped in the FP32 distance pass, same-cell slots masked per round, and in the hit queue the
    # lower-index rule of triclinic self pairs of a real copy and an image.  Over every case the parts keep
    # exactly the pairs pair_rule keeps, for the visits the kernel makes (the particle copy is real in
    # triclinic cross pairs; two copies of one particle are never both visited within the cutoff, since
    # the unit-cell check keeps images more than twice the cutoff apart)
    probe.pair_rule_probe.restype = C.c_int
    parts = C.c_int(0)
    n = 0
    codes = [0, 1, 2, 5, ~0, ~1, ~2, ~5]
    for cross in (0, 1):
        for kind in ("ortho", "tri", "nonper"):
            tri, nonper = int(kind == "tri"), int(kind == "nonper")
            for same in (0, 1):
                for slot_j in range(4):
                    for ii in range(4):
                        for ci in codes:
                            for cj in codes:
                                if nonper and (ci < 0 or cj < 0):
                                    continue  # no images without periodic boundaries
                                if (ci if ci >= 0 else ~ci) == (cj if cj >= 0 else ~cj):
                                    continue
                                if cross and tri and ci < 0:
                                    continue  # triclinic cross pairs visit real particle copies only
                                ref = probe.pair_rule_probe(cross, tri, nonper, same, slot_j, ii, ci, cj,
                                                            C.byref(parts))
                                assert parts.value == ref, (cross, kind, same, slot_j, ii, ci, cj)
                                n += 1
    assert n > 3000


@pytest.mark.parametrize("f64", [0, 1])
def test_cell_floor_screen_matches_division(probe, f64):
    """The build's cell index takes floor((x - xmin) / cs) from the product with RN(1 / cs) unless that product
    is within 4 ulp of an integer: it must equal the floor of the IEEE quotient everywhere, in particular for
    numerators a few ulp around multiples of the cell size (where the product and the quotient can round to
    different sides of an integer) and for random cell sizes."""
    dt = np.float64 if f64 else np.float32
    rng = np.random.default_rng(7)
    lib = probe
    lib.cell_floor_probe.restype = C.c_int64
    for cs in [2.5, 0.1, 1.0 / 3.0, 7.77, 0.0123456, 1234.5] + list(rng.uniform(0.01, 100.0, 20)):
        cs = float(dt(cs))
        k = np.arange(-3, 200, dtype=np.float64)
        base = (k * cs).astype(dt)
        vals = [base]
        up, dn = base.copy(), base.copy()
        for _ in range(8):
            up = np.nextafter(up, dt(np.inf))
            dn = np.nextafter(dn, dt(-np.inf))
            vals += [up.copy(), dn.copy()]
        vals.append(rng.uniform(-3 * cs, 200 * cs, 5000).astype(dt))
        a = np.ascontiguousarray(np.concatenate(vals).astype(np.float64))
        assert lib.cell_floor_probe(f64, a.ctypes.data_as(C.c_void_p), a.size, C.c_double(cs)) == 0, cs


@pytest.mark.parametrize("f64", [0, 1])
def test_image_tests_on_order_keys(probe, f64):
    """The build tests whether image k of a wrapped position lies in the computing box along each axis by
    comparing the position's order key (its bit pattern, magnitude inverted for negative values) with two
    thresholds found on the host, instead of the sum p + shift and two compares.  For every image and axis of
    periodic cells (orthorhombic and triclinic, 2D and 3D, lcell 1 to 3, random triclinic cells) the key test
    must agree with the sum and compares: at random positions across and around the box, at the keys around
    each threshold, and at +-0, +-inf and NaN."""
    dt = np.float64 if f64 else np.float32
    rng = np.random.default_rng(11)
    lib = probe
    lib.image_key_probe.restype = C.c_int64
    cells = [(dim, uc, cut, lcell) for dim, uc, cut, lcell, *_ in CASES if uc is not None]
    for _ in range(12):
        dim = int(rng.integers(2, 4))
        M = np.diag(rng.uniform(5.0, 20.0, dim)) + np.triu(rng.uniform(-3.0, 3.0, (dim, dim)), 1)
        if rng.random() < 0.5:
            M += np.tril(rng.uniform(-1.0, 1.0, (dim, dim)), -1)
        cells.append((dim, M.tolist(), float(rng.uniform(0.5, 2.5)), int(rng.integers(1, 4))))
    n_checked = 0
    for dim, uc, cut, lcell in cells:
        u = np.asarray(uc, np.float64)
        M = np.diag(u) if u.ndim == 1 else u.reshape(dim, dim)
        kind = 0 if u.ndim == 1 else 1
        Mc = np.ascontiguousarray(M.flatten(order="F"))
        span = float(np.abs(M).sum(axis=1).max()) + 3 * cut
        v = [rng.uniform(-span, span, 4000), rng.uniform(-cut, cut, 1000), rng.uniform(-1e-6, 1e-6, 200)]
        v = np.ascontiguousarray(np.concatenate(v).astype(dt).astype(np.float64))
        bad = lib.image_key_probe(f64, dim, kind, Mc.ctypes.data_as(C.c_void_p), C.c_double(cut), lcell,
                                  v.ctypes.data_as(C.c_void_p), C.c_int64(v.size))
        assert bad == 0, (dim, uc, cut, lcell, bad)
        n_checked += 1
    assert n_checked >= 20


def test_wrap_quotient_matches_division(probe):
    """The Float64 wrap solve divides by det(M) through quot_rn: RN(a / b) from y = RN(1 / b) with one
    correction step, kept only when the remainder proves it is the rounded quotient.  It must equal the IEEE
    quotient bit for bit: random quotients over many binades, exact multiples, powers of two (always left to
    the division), numerators a few ulp from multiples of b, signed zeros, subnormals, huge values, inf and
    NaN.  The fast path must also take the great majority of ordinary pairs."""
    rng = np.random.default_rng(5)
    lib = probe
    lib.quot_probe.restype = C.c_int64
    n = 200000
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-30, 30, n).astype(np.float64))
    b *= np.where(rng.random(n) < 0.2, -1.0, 1.0)
    a = rng.uniform(-1.0, 1.0, n) * np.exp2(rng.integers(-40, 40, n).astype(np.float64))
    fb = C.c_int64(0)
    vp = C.c_void_p
    assert lib.quot_probe(a.ctypes.data_as(vp), b.ctypes.data_as(vp), n, C.byref(fb)) == 0
    assert fb.value < n // 100, fb.value
    # positions against a box determinant, as the solve sees them
    det = np.array([1000.0, 1234.5678, 1.0 / 3.0, 8.0, 1e-3, 7.0e5, -512.25])
    k = rng.integers(-50000, 50000, 20000).astype(np.float64)
    cases_a, cases_b = [], []
    for d in det:
        base = k * d
        for s in range(-3, 4):
            cases_a.append(base + s * np.spacing(np.abs(base)))
            cases_b.append(np.full(base.size, d))
        cases_a.append(rng.uniform(-3 * abs(d), 3 * abs(d), 20000))
        cases_b.append(np.full(20000, d))
    sp = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, 5e-324, -5e-324, 2.2250738585072014e-308,
                   1.7976931348623157e308, -1.7976931348623157e308, np.inf, -np.inf, np.nan, 1e-300, 1e300,
                   0.1, 1.0 / 3.0, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)])
    aa, bb = np.meshgrid(sp, sp)
    cases_a.append(aa.ravel())
    cases_b.append(bb.ravel())
    a = np.ascontiguousarray(np.concatenate(cases_a))
    b = np.ascontiguousarray(np.concatenate(cases_b))
    assert lib.quot_probe(a.ctypes.data_as(vp), b.ctypes.data_as(vp), a.size, C.byref(fb)) == 0


@pytest.mark.parametrize("f64", [0, 1])
def test_cell_index_bits_match_division(probe, f64):
    """cell_of takes floor(RN((x - xmin) / cs)) from the bit pattern of the product with RN(1 / cs) when that
    product lies in (0, 2^31) and at least 5 ulp from every integer, else from cell_floor; with the range
    test [-1, nc) it must equal the IEEE floor of the quotient everywhere: numerators a few ulp around
    multiples of the cell size (the last cell, the half cell), zeros of both signs, negative, subnormal,
    tiny, huge, inf and NaN numerators, and random ones.  The bit screen must decide nearly all of the
    random numerators."""
    dt = np.float64 if f64 else np.float32
    rng = np.random.default_rng(13)
    lib = probe
    lib.cell_index_probe.restype = C.c_int64
    fast = C.c_int64(0)
    for cs in [2.5, 0.1, 1.0 / 3.0, 7.77, 0.0123456, 1234.5] + list(rng.uniform(0.01, 100.0, 12)):
        cs = float(dt(cs))
        nc = int(rng.integers(3, 400))
        k = np.arange(-3, nc + 3, dtype=np.float64)
        base = np.concatenate([(k * cs).astype(dt), ((k + 0.5) * cs).astype(dt)])
        vals = [base]
        up, dn = base.copy(), base.copy()
        for _ in range(8):
            up = np.nextafter(up, dt(np.inf))
            dn = np.nextafter(dn, dt(-np.inf))
            vals += [up.copy(), dn.copy()]
        tiny = np.finfo(dt).smallest_subnormal
        vals.append(np.array([0.0, -0.0, tiny, -tiny, 1e-30, -1e-30, np.inf, -np.inf, np.nan, 1e30, -1e30,
                              float(np.finfo(dt).max)], dt))
        a = np.ascontiguousarray(np.concatenate(vals).astype(np.float64))
        assert lib.cell_index_probe(f64, a.ctypes.data_as(C.c_void_p), a.size, C.c_double(cs), nc,
                                    C.byref(fast)) == 0, cs
        r = np.ascontiguousarray(rng.uniform(0.0, nc * cs, 20000).astype(dt).astype(np.float64))
        assert lib.cell_index_probe(f64, r.ctypes.data_as(C.c_void_p), r.size, C.c_double(cs), nc,
                                    C.byref(fast)) == 0, cs
        assert fast.value > 0.99 * r.size, (cs, fast.value)


def test_float_pair_from_bits(probe):
    """The gather splits each Float64 copy coordinate into a float pair for the FP32 offsets: hi = (float)q,
    lo = (float)(q - hi).  float_pair takes both from q's bit pattern with integer operations: it must equal
    the conversions bit for bit on random values over every binade the fast path takes and beyond it, on
    round-to-nearest-even ties (29 dropped bits exactly half, kept bits odd and even), on carries into the
    exponent, on floats themselves, on the limits of the fast range, and on zeros, subnormals, huge values,
    inf and NaN."""
    rng = np.random.default_rng(17)
    lib = probe
    lib.float_pair_probe.restype = C.c_int64
    n = 200000
    q = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-140, 140, n).astype(np.float64))
    q *= np.where(rng.random(n) < 0.5, -1.0, 1.0)
    # bit patterns built to hit the rounding cases: the dropped 29 bits at, just below and just above half,
    # all ones (a carry through the 23 kept bits into the exponent), kept bits odd or even
    e = rng.integers(1023 - 80, 1023 + 130, 4000).astype(np.uint64)
    top = rng.integers(0, 1 << 23, 4000).astype(np.uint64)
    cases = []
    for rem in (0x10000000, 0x0FFFFFFF, 0x10000001, 0x1FFFFFFF, 0, 1):
        for t in (top, top | np.uint64(1), top & ~np.uint64(1), np.full(4000, (1 << 23) - 1, np.uint64)):
            bits = (e << np.uint64(52)) | (t << np.uint64(29)) | np.uint64(rem)
            cases.append(bits.view(np.float64))
            cases.append((bits | np.uint64(1 << 63)).view(np.float64))
    edges = [np.exp2(float(k)) for k in (-74, -75, -73, 125, 126, 127, -126, -149, -150)]
    sp = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf,
                   -np.inf, np.nan, 1e-30, 3.4028234663852886e38, 3.4028235677973366e38, 1.0, -1.0, 0.1, 109.4]
                  + edges + [np.nextafter(x, 0.0) for x in edges] + [np.nextafter(x, np.inf) for x in edges])
    fl = rng.uniform(-200, 200, 5000).astype(np.float32).astype(np.float64)
    allq = np.ascontiguousarray(np.concatenate([q, sp, fl] + cases))
    assert lib.float_pair_probe(allq.ctypes.data_as(C.c_void_p), allq.size) == 0


def test_shaped_wrap_matches_general(probe):
    """Float64 3D cells with exact zeros in the input matrix (orthorhombic: diagonal with R the identity;
    upper-triangular triclinic cells such as the benchmark's) wrap with the zero terms skipped.  That is
    exact when every input is finite and no shortened sum is zero, and otherwise the particle takes the full
    sums.  The shaped wrap must equal the general one bit for bit, signed zeros included: random positions
    inside and far outside the box, lattice points and box corners (zero fractional coordinates, the
    fallback), signed zeros, points a few ulp off multiples of the cell vectors, huge and non-finite
    coordinates."""
    rng = np.random.default_rng(19)
    lib = probe
    lib.wrap_shape_probe.restype = C.c_int64
    cells = [(0, [10.0, 12.0, 11.0]), (0, [109.43846059, 109.43846059, 109.43846059]),
             (1, [[109.43846059, 21.88769212, 10.94384606], [0.0, 109.43846059, 16.41576909],
                  [0.0, 0.0, 109.43846059]]),
             (1, [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]]),
             (1, [[10.0, -2.0, 1.0], [0.0, 11.0, -1.5], [0.0, 0.0, 12.0]]),
             (1, [[12.0, 0.0, 0.0], [0.0, 10.0, 0.0], [0.0, 0.0, 11.0]]),
             # negative sides (a triclinic cell with a negative diagonal fails the cell check)
             (0, [-10.0, 12.0, -11.0])]
    for _ in range(6):
        M = np.diag(rng.uniform(5.0, 20.0, 3)) + np.triu(rng.uniform(-3.0, 3.0, (3, 3)), 1)
        cells.append((1, M.tolist()))
        cells.append((0, list(rng.uniform(5.0, 30.0, 3))))
    seen = set()
    shape = C.c_int(0)
    for kind, uc in cells:
        u = np.asarray(uc, np.float64)
        M = np.diag(u) if u.ndim == 1 else u
        Mc = np.ascontiguousarray(M.flatten(order="F"))
        pts = [rng.uniform(-2.0, 3.0, (20000, 3)) @ M.T, rng.uniform(-1e6, 1e6, (2000, 3)),
               (rng.integers(-3, 4, (3000, 3)).astype(np.float64)) @ M.T,
               (rng.integers(-3, 4, (2000, 3)).astype(np.float64) * 0.5) @ M.T]
        lat = (rng.integers(-3, 4, (2000, 3)).astype(np.float64)) @ M.T
        for s in (-2, -1, 1, 2):
            pts.append(lat + s * np.spacing(np.abs(lat) + 1e-300))
        sp = np.array([0.0, -0.0, 1e-300, -1e-300, 5e-324, 1e300, -1e300, np.inf, -np.inf])
        g3 = np.array(np.meshgrid(sp, sp, sp)).reshape(3, -1).T
        pts.append(g3)
        x = np.ascontiguousarray(np.concatenate(pts))
        bad = lib.wrap_shape_probe(kind, Mc.ctypes.data_as(C.c_void_p), C.c_double(1.5),
                                   x.ctypes.data_as(C.c_void_p), x.shape[0], C.byref(shape))
        assert bad == 0, (kind, uc, bad)
        seen.add(shape.value)
    assert seen == {1, 2}, seen


@pytest.mark.parametrize("f64", [0, 1])
def test_image_threshold_search(probe, f64):
    """The image tests' thresholds: the smallest order key q with RN(value(q) + s) >= b, found by bisection
    after a bracket of 4 keys around RN(b - s).  On arbitrary shifts and bounds it must be exactly the first
    passing key: ordinary values, b - s near zero where the threshold lies many keys from RN(b - s) (the
    bracket fails and the full bisection runs), s much larger or smaller than b, equal values, signed
    zeros and subnormals."""
    rng = np.random.default_rng(23)
    lib = probe
    lib.first_key_probe.restype = C.c_int64
    dt = np.float64 if f64 else np.float32
    n = 20000
    s = rng.uniform(-100, 100, n)
    b = rng.uniform(-100, 100, n)
    s2 = rng.uniform(-100, 100, n)
    b2 = s2 + rng.uniform(-1e-6, 1e-6, n) * np.abs(s2)  # b - s near zero
    s3 = rng.uniform(-1, 1, n) * np.exp2(rng.integers(-60, 60, n).astype(np.float64))
    b3 = rng.uniform(-1, 1, n) * np.exp2(rng.integers(-60, 60, n).astype(np.float64))
    tiny = float(np.finfo(dt).smallest_subnormal)
    sp = np.array([0.0, -0.0, 1.0, -1.0, tiny, -tiny, 5.0, -5.0, 1e-30, 1e30, 1234.5678])
    ss, bb = np.meshgrid(sp, sp)
    S = np.concatenate([s, s2, s2, s3, ss.ravel()]).astype(dt).astype(np.float64)
    B = np.concatenate([b, b2, s2, b3, bb.ravel()]).astype(dt).astype(np.float64)
    S, B = np.ascontiguousarray(S), np.ascontiguousarray(B)
    assert lib.first_key_probe(f64, S.ctypes.data_as(C.c_void_p), B.ctypes.data_as(C.c_void_p), S.size) == 0
