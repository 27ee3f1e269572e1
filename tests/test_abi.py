"""CPU tests of the C-ABI boundary: the library builds for sm_103a, loads, and exports every
symbol declared in include/celllistmap_gb300.h.  No compute call is made (no GPU here)."""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "celllistmap_gb300.h")).read()
    return sorted(set(re.findall(r"\b(clm_[a-z_]+)\s*\(", src)))


def test_header_declares_the_python_binding_table(clm):
    assert declared_symbols() == sorted(clm._abi.EXPORTS)


def test_library_exports_every_declared_symbol(clm):
    path = clm._abi.lib_path()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_julia_binding_covers_every_declared_symbol():
    # the reference-side binding (the ccall stubs of a CellListMap.jl package extension) names every entry
    # point of the header
    src = open(os.path.join(ROOT, "celllistmap.jl_gb300", "julia", "CellListMapGB300Ext.jl")).read()
    bound = set(re.findall(r"ccall\(\(:(clm_[a-z_0-9]+)\s*,", src))
    assert sorted(bound) == declared_symbols()


def test_version_string(clm):
    lib = clm._abi.load()
    assert b"sm_103a" in lib.clm_version()


def test_create_rejects_bad_arguments_without_touching_the_gpu(clm):
    lib = clm._abi.load()
    h = ctypes.c_void_p()
    assert lib.clm_create(7, 3, 1, ctypes.byref(h)) == 1   # bad dtype
    assert lib.clm_create(1, 4, 1, ctypes.byref(h)) == 1   # bad dim
    assert lib.clm_create(1, 3, 3, ctypes.byref(h)) == 1   # bad nsets
    assert lib.clm_destroy(None) == 1


def test_python_front_end_reports_missing_library(tmp_path, clm):
    saved = clm._abi._lib
    clm._abi._lib = None
    try:
        with pytest.raises(ImportError):
            clm._abi.load(str(tmp_path / "missing.so"))
    finally:
        clm._abi._lib = saved


def test_dimension_and_argument_checks_happen_on_the_host(clm):
    api = clm._api if hasattr(clm, "_api") else clm.api
    with pytest.raises(clm.ArgumentError):
        api._get_dim([1.0, 1.0, 1.0, 1.0], [[0.0, 0.0, 0.0, 0.0]])
    with pytest.raises(clm.ArgumentError):
        api._get_dim([1.0, 1.0, 1.0], [[0.0, 0.0]])
    assert api._promote_dtype([1, 1, 1], 2, None) == "float64"
    import numpy as np
    assert api._promote_dtype(np.array([1.0, 1.0], np.float32), np.float32(0.1), None) == np.float32


def test_dimension_inference_like_the_reference(clm):
    # get_dim cases of test/internals/auxiliary_functions.jl:12-31 (positions as lists of points; the
    # untyped-empty-vector case has no Python counterpart: [] and an empty (0, dim) array are both accepted)
    import numpy as np
    api = clm._api if hasattr(clm, "_api") else clm.api
    assert api._get_dim([1, 2], [[1, 2], [3, 4]]) == 2
    assert api._get_dim([1, 2], [[1, 2], [3, 4]], [[1, 2], [3, 4]]) == 2
    assert api._get_dim([1, 2, 3], [[1, 2, 3], [3, 4, 5]]) == 3
    assert api._get_dim([1, 2, 3], [[1, 2, 3], [3, 4, 5]], [[1, 2, 3], [3, 4, 5]]) == 3
    assert api._get_dim([1, 2], np.zeros((0, 2))) == 2
    assert api._get_dim([], [[1.0, 2.0]]) == 2
    assert api._get_dim(None, [[1.0, 2.0]]) == 2
    for args, msg in ((([1, 2], [[1, 2, 3]]), "Incompatible dimensions"), (([1, 2, 3, 4], [[1, 2, 3, 4]]), "2 or 3"),
                      ((None, [[]]), "Could not infer")):
        with pytest.raises(clm.ArgumentError, match=msg):
            api._get_dim(*args)


def test_type_promotion_like_the_reference(clm):
    # _promote_types cases of test/internals/Box.jl:11-28,124-131 (0.1f0 -> np.float32(0.1), a Float32
    # vector -> a float32 array, nothing -> None): integers yield to any float type, integers alone give
    # Float64, Float32 with Float64 gives Float64
    import numpy as np
    api = clm._api if hasattr(clm, "_api") else clm.api
    f32 = np.float32
    cases = [
        ([1, 1, 1], 0.1, np.float64),
        ([1, 1, 1], f32(0.1), np.float32),
        ([1.0, 1, 1], f32(0.1), np.float64),
        (np.array([1, 1, 1], f32), f32(0.1), np.float32),
        ([10, 10, 10.0], 1, np.float64),
        (np.array([10, 10, 10], f32), 1, np.float32),
        ([10, 10, 10], 1, np.float64),
        (None, f32(1.0), np.float32),
        (np.array([1, 1, 1], f32), None, np.float32),
        (np.array([1, 1, 1], f32), 1.0, np.float64),
        ([1.0, 1.0, 1.0], f32(1.0), np.float64),
        ([1, 1, 1], 1, np.float64),
    ]
    for unitcell, cutoff, want in cases:
        assert api._promote_dtype(unitcell, cutoff, None) == want, (unitcell, cutoff)


def _build_c_driver(clm, tmp_path):
    """Compile tests/abi_driver.c (plain C99 against the header) and link it to the library."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(clm._abi.lib_path())
    exe = str(tmp_path / "abi_driver")
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "abi_driver.c"), "-L", libdir, "-lcelllist_cuda", "-Wl,-rpath," + libdir,
           "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_client_compiles_and_links(clm, tmp_path):
    # the header is plain C and every entry point the C client calls resolves in the shared library
    assert os.path.exists(_build_c_driver(clm, tmp_path))


@pytest.mark.gpu
def test_c_client_known_answers(clm, tmp_path):
    import subprocess
    exe = _build_c_driver(clm, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi driver ok" in r.stdout


def test_operator_parameters_are_checked_on_the_host(clm):
    """Operator arguments are validated before any device work (stand-in system: sizes only)."""
    import numpy as np

    class Sys:
        n_x, n_y, nsets, dim, dtype = 5, 3, 1, 3, np.float64

    p, keep = clm.WeightedInverseDistance(np.ones(5), 9.8).params(Sys)
    assert p.p[0] == 9.8 and p.weights_x == keep[0].ctypes.data and not p.weights_y
    with pytest.raises(clm.DimensionMismatch):
        clm.WeightedInverseDistance(np.ones(4)).params(Sys)
    Sys.nsets = 2
    with pytest.raises(clm.ArgumentError):
        clm.WeightedInverseDistance(np.ones(5)).params(Sys)  # two sets need weights_y
    with pytest.raises(clm.DimensionMismatch):
        clm.WeightedInverseDistance(np.ones(5), weights_y=np.ones(2)).params(Sys)
    p, keep = clm.WeightedInverseDistance(np.ones(5), 1.0, np.ones(3)).params(Sys)
    assert p.weights_y == keep[1].ctypes.data
    Sys.nsets = 1
    eps = np.ones((2, 2))
    with pytest.raises(clm.ArgumentError):  # type index outside the tables
        clm.LennardJones(types_x=np.array([0, 1, 2, 0, 1]), eps_table=eps, sig_table=eps).params(Sys)
    with pytest.raises(clm.DimensionMismatch):
        clm.LennardJones(types_x=np.array([0, 1]), eps_table=eps, sig_table=eps).params(Sys)


def test_operator_ids_agree_across_header_python_and_oracle(clm, orc):
    """The operator ids of include/celllistmap_gb300.h, the Python binding table and the oracle's table
    are the same numbers."""
    src = open(os.path.join(ROOT, "include", "celllistmap_gb300.h")).read()
    ids = {name.lower(): int(v) for name, v in re.findall(r"CLM_OP_([A-Z0-9_]+)\s*=\s*(\d+)", src)}
    assert ids and ids == {k: v for k, v in clm._abi.OP.items()}
    assert {k: v for k, v in orc.OPS.items()} == ids
