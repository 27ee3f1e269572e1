"""Trajectory ingestion (DCD and PDB readers of the package): round trips through the writer, both byte
orders, unit-cell records, and the cell matrix of the CHARMM cell record."""
import math
import os

import numpy as np
import pytest


@pytest.mark.parametrize("endian", ["<", ">"])
@pytest.mark.parametrize("with_cell", [False, True])
def test_dcd_round_trip(clm, tmp_path, endian, with_cell):
    rng = np.random.default_rng(4)
    frames = [rng.random((57, 3)).astype(np.float32) * 30 for _ in range(3)]
    cells = [[30.0, 0.0, 31.0, 0.0, 0.0, 32.0 + k] for k in range(3)] if with_cell else None
    p = os.path.join(tmp_path, "t.dcd")
    clm.trajectory.write_dcd(p, frames, cells, endian=endian)
    t = clm.trajectory.read_dcd(p)
    assert t.natoms == 57 and len(t.frames) == 3
    for a, b in zip(t.frames, frames):
        np.testing.assert_array_equal(a, b)
    if with_cell:
        np.testing.assert_array_equal(t.unitcell(2), np.diag([30.0, 31.0, 34.0]))
    else:
        assert t.cells[0] is None


def test_dcd_cell_matrix_angles(clm):
    # cosines (NAMD) and degrees give the same matrix; a along x, b in the xy plane
    a, b, c = 10.0, 11.0, 12.0
    al, be, ga = 70.0, 80.0, 60.0
    Mc = clm.trajectory.cell_matrix_from_dcd([a, math.cos(math.radians(ga)), b, math.cos(math.radians(be)),
                                              math.cos(math.radians(al)), c])
    Md = clm.trajectory.cell_matrix_from_dcd([a, ga, b, be, al, c])
    np.testing.assert_allclose(Mc, Md, rtol=1e-12)
    va, vb, vc = Md[:, 0], Md[:, 1], Md[:, 2]
    assert np.isclose(np.linalg.norm(vb), b) and np.isclose(np.linalg.norm(vc), c)
    assert np.isclose(np.degrees(np.arccos(vb @ vc / (b * c))), al)
    assert np.isclose(np.degrees(np.arccos(va @ vc / (a * c))), be)
    assert np.isclose(np.degrees(np.arccos(va @ vb / (a * b))), ga)


def test_dcd_rejects_garbage(clm, tmp_path):
    p = os.path.join(tmp_path, "bad.dcd")
    open(p, "wb").write(b"\x00" * 100)
    with pytest.raises(ValueError):
        clm.trajectory.read_dcd(p)


def test_pdb_reader(clm, tmp_path):
    p = os.path.join(tmp_path, "x.pdb")
    open(p, "w").write("CRYST1   21.000   21.000   21.000  90.00  90.00  90.00 P 1           1\n"
                       "ATOM      1  AR  ARG A   1       1.000   2.500  -3.250  1.00  0.00\n"
                       "HETATM    2  AR  ARG A   2      10.125  20.000   0.000  1.00  0.00\n")
    x, cryst = clm.trajectory.read_pdb(p)
    np.testing.assert_array_equal(x, [[1.0, 2.5, -3.25], [10.125, 20.0, 0.0]])
    assert cryst == [21.0, 21.0, 21.0, 90.0, 90.0, 90.0]
