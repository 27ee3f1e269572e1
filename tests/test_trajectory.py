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


class _BitWriter:
    def __init__(self):
        self.bits = []

    def put(self, value, n):
        self.bits += [(value >> (n - 1 - k)) & 1 for k in range(n)]

    def triplet(self, digits, radix, nbits):
        v = (digits[0] * radix[1] + digits[1]) * radix[2] + digits[2]
        while nbits > 8:
            self.put(v & 0xFF, 8)
            v >>= 8
            nbits -= 8
        self.put(v, nbits)

    def data(self):
        bits = self.bits + [0] * (-len(self.bits) % 8)
        return bytes(int("".join(map(str, bits[k:k + 8])), 2) for k in range(0, len(bits), 8))


def _xtc_frame(xyz_nm, box_nm, precision, runs=(), smallidx=20):
    """One XTC frame written the simple way: every atom a full triplet, except the atoms listed in `runs`
    (start index, length), which are packed as a run of small differences after their first atom."""
    import struct
    q = np.rint(np.asarray(xyz_nm, np.float64) * precision).astype(np.int64)
    n = len(q)
    mn, mx = q.min(axis=0), q.max(axis=0)
    radix = [int(mx[k] - mn[k] + 1) for k in range(3)]
    nbits = (radix[0] * radix[1] * radix[2]).bit_length()
    large = any(r > 0xFFFFFF for r in radix)  # then each component is stored with its own width
    w = _BitWriter()

    def first(digits):
        if large:
            for k in range(3):
                w.put(digits[k], radix[k].bit_length())
        else:
            w.triplet(digits, radix, nbits)
    run_at = dict(runs)
    i, current = 0, 0

    def run_flag(length):
        # the run length carries over to the next group unless a flag bit announces a new one
        nonlocal current
        if length == current:
            w.put(0, 1)
        else:
            w.put(1, 1)
            w.put(3 * length + 1, 5)                   # radix index unchanged: run % 3 == 1
            current = length

    while i < n:
        length = run_at.get(i, 0)
        if length == 0:
            first([int(q[i, k] - mn[k]) for k in range(3)])
            run_flag(0)
            i += 1
            continue
        # output order a_i, a_{i+1}, ...: the full triplet carries a_{i+1}, the first small difference a_i
        size = _MAGIC[smallidx]
        half = size // 2
        first([int(q[i + 1, k] - mn[k]) for k in range(3)])
        run_flag(length)
        prev = q[i + 1]
        for k, a in enumerate([i] + list(range(i + 2, i + 1 + length))):
            w.triplet([int(q[a, c] - prev[c] + half) for c in range(3)], [size] * 3, smallidx)
            prev = q[a]
        i += 1 + length
    block = w.data()
    head = struct.pack(">3i", 1995, n, 7) + struct.pack(">f", 0.5) + \
        struct.pack(">9f", *np.asarray(box_nm, np.float32).ravel()) + struct.pack(">i", n)
    head += struct.pack(">f", precision) + struct.pack(">3i", *mn) + struct.pack(">3i", *mx) + \
        struct.pack(">i", smallidx) + struct.pack(">i", len(block))
    return head + block + b"\0" * (-len(block) % 4)


_MAGIC = {20: 101, 21: 128}


def test_xtc_magic_table(clm):
    t = clm.trajectory._XTC_MAGIC_TABLE
    assert t[:9] == [0] * 9 and t[9:15] == [8, 10, 12, 16, 20, 25] and t[20] == 101 and t[72] == 1 << 24
    assert all(t[i] ** 3 <= 1 << i < (t[i] + 1) ** 3 for i in range(9, 73) if i not in (37, 57, 69))


@pytest.mark.parametrize("runs", [(), ((3, 2), (10, 1))])
def test_xtc_synthetic_frames(clm, tmp_path, runs):
    rng = np.random.default_rng(9)
    box = np.array([[3.0, 0, 0], [0.5, 3.1, 0], [0.2, 0.3, 2.9]])
    x = rng.random((14, 3)) * 3.0
    for start, length in runs:                         # the run's atoms sit next to their first atom
        for a in [start] + list(range(start + 2, start + 1 + length)):
            x[a] = x[start + 1] + rng.uniform(-0.03, 0.03, 3)
    p = os.path.join(tmp_path, "t.xtc")
    with open(p, "wb") as f:
        f.write(_xtc_frame(x, box, 1000.0, runs) + _xtc_frame(x[::-1], box, 1000.0))
    frames = clm.trajectory.read_xtc(p)
    assert len(frames) == 2 and frames[0].step == 7 and frames[0].precision == 1000.0
    want = np.rint(x * 1000).astype(np.float32) * np.float32(1.0 / 1000)
    np.testing.assert_allclose(frames[0].positions, want.astype(np.float64) * 10, rtol=0, atol=1e-5)
    np.testing.assert_allclose(frames[1].positions, want[::-1].astype(np.float64) * 10, rtol=0, atol=1e-5)
    np.testing.assert_allclose(frames[0].unitcell, box.T * 10, rtol=1e-6)
    with open(p, "rb") as f:
        data = f.read()
    with open(p, "wb") as f:
        f.write(data[:60])
    with pytest.raises(ValueError):
        clm.trajectory.read_xtc(p)
    with open(p, "wb") as f:
        f.write(b"\0\0\0\1" + data[4:])
    with pytest.raises(ValueError):
        clm.trajectory.read_xtc(p)


def test_xtc_large_coordinate_range(clm, tmp_path):
    # a range above 2^24 stored integers (here 40,000 nm at precision 1000) switches the format to one
    # field per component
    rng = np.random.default_rng(10)
    x = rng.random((30, 3)) * np.array([40000.0, 3.0, 20000.0])
    x[4] = x[5] + rng.uniform(-0.03, 0.03, 3)  # atom 4 is packed as a small difference from atom 5
    box = np.diag([40000.0, 3.0, 20000.0])
    p = os.path.join(tmp_path, "big.xtc")
    with open(p, "wb") as f:
        f.write(_xtc_frame(x, box, 1000.0, ((4, 1),)))
    (fr,) = clm.trajectory.read_xtc(p)
    want = (np.rint(x * 1000).astype(np.float32) * np.float32(1.0 / 1000)).astype(np.float64) * 10
    np.testing.assert_allclose(fr.positions, want, rtol=1e-6, atol=0)


def test_xtc_small_frame_uncompressed(clm, tmp_path):
    import struct
    x = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]], np.float32)
    data = struct.pack(">3i", 1995, 2, 0) + struct.pack(">f", 0.0) + struct.pack(">9f", 2, 0, 0, 0, 2, 0, 0, 0, 2) + \
        struct.pack(">i", 2) + struct.pack(">6f", *x.ravel())
    p = os.path.join(tmp_path, "m.xtc")
    with open(p, "wb") as f:
        f.write(data)
    (fr,) = clm.trajectory.read_xtc(p)
    np.testing.assert_array_equal(fr.positions, x.astype(np.float64) * 10)
    np.testing.assert_array_equal(fr.unitcell, np.diag([20.0, 20.0, 20.0]))
