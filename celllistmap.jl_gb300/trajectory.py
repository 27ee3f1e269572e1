"""Trajectory ingestion for the pair engine: CHARMM/NAMD DCD frames, GROMACS XTC frames and PDB coordinates.

The reference reads its NAMD and GROMACS test trajectories with Chemfiles (test/applications/namd/
ParticleSystem_vs_NAMD.jl:21-26, test/applications/gromacs/compare_with_gromacs.jl:15-24) and its argon
fixture with PDBTools (src/CellListMap.jl:61).  Neither is available here, so this module reads the
formats directly:

* DCD: Fortran unformatted records (4-byte length markers, either byte order).  Header record ``CORD``
  with 20 control integers (frame count, ``icntrl[10]`` = unit-cell flag, ``icntrl[8]`` = fixed atoms),
  a title record, the atom count, then per frame an optional unit-cell record of 6 doubles
  (a, gamma, b, beta, alpha, c in the CHARMM order; angles in degrees or as cosines) and three float32
  records x, y, z.
* XTC: XDR (big-endian) frames of the GROMACS compressed-coordinate format (Green et al., the
  ``xdr3dfcoord`` scheme): integer coordinates at a stored precision, the first atom of every group
  packed as a mixed-radix triplet over the frame's bounding range, runs of nearby atoms packed as small
  differences whose radix follows the "magic" table of sizes ~2^(i/3).  Positions and box come back in
  Angstrom, as Chemfiles returns them.
* PDB: fixed columns 31-54 of ATOM/HETATM records, parsed as Float64 and the CRYST1 box.

Frames come back as (n, 3) float32 arrays, which is the memory layout the C ABI takes.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass
from typing import List, Optional

import numpy as np


@dataclass
class DCDTrajectory:
    natoms: int
    frames: List[np.ndarray]             # (natoms, 3) float32 each
    cells: List[Optional[np.ndarray]]    # per frame: (a, gamma, b, beta, alpha, c) or None
    title: str = ""

    def unitcell(self, k: int = 0) -> Optional[np.ndarray]:
        """3x3 unit-cell matrix (columns are the cell vectors) of frame k, or None without a cell record."""
        c = self.cells[k]
        return None if c is None else cell_matrix_from_dcd(c)


def _records(data: bytes):
    """Splits a Fortran unformatted file into records; detects the byte order from the first marker."""
    for endian in ("<", ">"):
        (n,) = struct.unpack_from(endian + "i", data, 0)
        if n == 84 and data[4:8] == b"CORD":
            break
    else:
        raise ValueError("not a DCD file (no 84-byte CORD header record)")
    pos, recs = 0, []
    while pos < len(data):
        (n,) = struct.unpack_from(endian + "i", data, pos)
        if n < 0 or pos + 8 + n > len(data):
            raise ValueError("truncated or corrupt DCD record")
        (n2,) = struct.unpack_from(endian + "i", data, pos + 4 + n)
        if n != n2:
            raise ValueError("corrupt DCD record (length markers differ)")
        recs.append(data[pos + 4:pos + 4 + n])
        pos += 8 + n
    return endian, recs


def read_dcd(path: str) -> DCDTrajectory:
    data = open(path, "rb").read()
    endian, recs = _records(data)
    hdr = recs[0]
    icntrl = struct.unpack_from(endian + "20i", hdr, 4)
    if icntrl[8] != 0:
        raise ValueError("DCD files with fixed atoms are not supported")
    has_cell = icntrl[10] != 0
    title = recs[1][4:].decode("latin-1", errors="replace").strip() if len(recs[1]) > 4 else ""
    (natoms,) = struct.unpack_from(endian + "i", recs[2])
    per = 3 + (1 if has_cell else 0)
    body = recs[3:]
    if len(body) % per:
        raise ValueError("DCD frame records are incomplete")
    frames, cells = [], []
    for f in range(len(body) // per):
        r = body[f * per:(f + 1) * per]
        cell = None
        if has_cell:
            cell = np.array(struct.unpack_from(endian + "6d", r[0]), dtype=np.float64)
            r = r[1:]
        xyz = [np.frombuffer(rr, dtype=endian + "f4") for rr in r]
        if any(v.size != natoms for v in xyz):
            raise ValueError("DCD coordinate record size does not match the atom count")
        frames.append(np.stack(xyz, axis=1).astype(np.float32))
        cells.append(cell)
    return DCDTrajectory(natoms, frames, cells, title)


def cell_matrix_from_dcd(c) -> np.ndarray:
    """Unit-cell matrix from a DCD cell record (a, gamma, b, beta, alpha, c).  Angles given as cosines
    (|value| <= 1, as NAMD writes them) or in degrees.  a along x, b in the xy plane."""
    a, g, b, be, al, cc = [float(v) for v in c]

    def cosine(v):
        return v if abs(v) <= 1.0 else math.cos(math.radians(v))

    cg, cb, ca = cosine(g), cosine(be), cosine(al)
    sg = math.sqrt(max(0.0, 1.0 - cg * cg))
    ax = np.array([a, 0.0, 0.0])
    bx = np.array([b * cg, b * sg, 0.0])
    cx = cc * cb
    cy = cc * (ca - cb * cg) / sg if sg > 0 else 0.0
    cz = math.sqrt(max(0.0, cc * cc - cx * cx - cy * cy))
    M = np.stack([ax, bx, np.array([cx, cy, cz])], axis=1)
    M[np.abs(M) < 1e-12 * max(a, b, cc)] = 0.0
    return M


def write_dcd(path: str, frames, cells=None, endian: str = "<") -> None:
    """Writes frames (each (natoms, 3)) as a DCD file; `cells` (one 6-vector per frame) adds cell records."""
    frames = [np.asarray(f, dtype=np.float32) for f in frames]
    natoms = frames[0].shape[0]

    def rec(b: bytes) -> bytes:
        return struct.pack(endian + "i", len(b)) + b + struct.pack(endian + "i", len(b))

    icntrl = [0] * 20
    icntrl[0] = len(frames)
    icntrl[10] = 1 if cells is not None else 0
    icntrl[19] = 24
    out = [rec(b"CORD" + struct.pack(endian + "20i", *icntrl)),
           rec(struct.pack(endian + "i", 1) + b"celllistmap-gb300".ljust(80)),
           rec(struct.pack(endian + "i", natoms))]
    for k, f in enumerate(frames):
        if cells is not None:
            out.append(rec(struct.pack(endian + "6d", *[float(v) for v in cells[k]])))
        for d in range(3):
            out.append(rec(np.ascontiguousarray(f[:, d]).astype(endian + "f4").tobytes()))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


def read_pdb(path: str):
    """Coordinates (n, 3) float64 of ATOM/HETATM records and the CRYST1 sides/angles (or None)."""
    xyz, cryst = [], None
    with open(path) as f:
        for line in f:
            if line.startswith("ATOM") or line.startswith("HETATM"):
                xyz.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
            elif line.startswith("CRYST1"):
                try:
                    cryst = [float(line[6:15]), float(line[15:24]), float(line[24:33]),
                             float(line[33:40]), float(line[40:47]), float(line[47:54])]
                except ValueError:   # hand-written files that ignore the fixed columns
                    cryst = [float(v) for v in line.split()[1:7]]
    return np.array(xyz, dtype=np.float64).reshape(-1, 3), cryst


# --------------------------------------------------------------------------------------------- XTC

XTC_MAGIC = 1995
_XTC_FIRST_SMALL = 9     # the smallest usable index of the magic table


def _xtc_magic_table():
    """Radix of a packed small difference per index: floor(2^(i/3)) for i >= 9, zero below.

    The format fixes three entries that differ from that rule (5060 at 37, 2^19 - 1 at 57 and
    2^23 - 1 at 69); they are kept so that files written with them decode the same way.
    """
    table = [0] * _XTC_FIRST_SMALL
    for i in range(_XTC_FIRST_SMALL, 73):
        target, m = 1 << i, 1 << (i // 3)          # integer cube root of 2^i, from below
        while (m + 1) ** 3 <= target:
            m += 1
        table.append(m)
    table[37], table[57], table[69] = 5060, (1 << 19) - 1, (1 << 23) - 1
    return table


_XTC_MAGIC_TABLE = _xtc_magic_table()


class _BitStream:
    """Reads unsigned integers of any width from a byte string, most significant bit first."""

    def __init__(self, data: bytes):
        self.value = int.from_bytes(data, "big")
        self.nbits = 8 * len(data)
        self.pos = 0

    def take(self, n: int) -> int:
        if n == 0:
            return 0
        if self.pos + n > self.nbits:
            raise ValueError("truncated XTC coordinate block")
        self.pos += n
        return (self.value >> (self.nbits - self.pos)) & ((1 << n) - 1)

    def triplet(self, nbits: int, radix) -> List[int]:
        """Three digits of a mixed-radix number stored in `nbits` bits as little-endian 8-bit groups
        (the last, possibly shorter, group is the most significant)."""
        v, shift = 0, 0
        while nbits > 8:
            v |= self.take(8) << shift
            shift += 8
            nbits -= 8
        v |= self.take(nbits) << shift
        c2 = v % radix[2]
        v //= radix[2]
        c1 = v % radix[1]
        return [v // radix[1], c1, c2]


@dataclass
class XTCFrame:
    step: int
    time: float
    positions: np.ndarray        # (natoms, 3) float64, Angstrom
    unitcell: np.ndarray         # (3, 3) float64, Angstrom; columns are the cell vectors
    precision: float


def _xtc_decode_block(data: bytes, natoms: int, minint, maxint, smallidx: int, inv_prec: np.float32):
    radix = [int(maxint[k]) - int(minint[k]) + 1 for k in range(3)]
    if any(r <= 0 for r in radix):
        raise ValueError("corrupt XTC frame (empty coordinate range)")
    large = any(r > 0xFFFFFF for r in radix)
    bits_each = [r.bit_length() for r in radix]
    bits_all = (radix[0] * radix[1] * radix[2]).bit_length()
    table = _XTC_MAGIC_TABLE
    if not (_XTC_FIRST_SMALL <= smallidx < len(table)):
        raise ValueError("corrupt XTC frame (small-difference index out of range)")
    smaller = table[max(_XTC_FIRST_SMALL, smallidx - 1)] // 2
    smallnum = table[smallidx] // 2
    bs = _BitStream(data)
    out = np.empty((natoms, 3), dtype=np.int64)
    nout, run = 0, 0

    def emit(c):
        nonlocal nout
        if nout >= natoms:
            raise ValueError("corrupt XTC frame (more coordinates than atoms)")
        out[nout] = c
        nout += 1

    i = 0
    while i < natoms:
        if large:
            first = [bs.take(bits_each[k]) for k in range(3)]
        else:
            first = bs.triplet(bits_all, radix)
        first = [first[k] + int(minint[k]) for k in range(3)]
        i += 1
        step_idx = 0
        if bs.take(1):
            run = bs.take(5)
            step_idx = run % 3 - 1
            run -= run % 3
        if run > 0:
            # each following atom is a small difference from the one decoded before it; the first two
            # atoms of a run are stored in swapped order (for water, the oxygen is packed second)
            prev = first
            size_small = [table[smallidx]] * 3
            for k in range(0, run, 3):
                d = bs.triplet(smallidx, size_small)
                cur = [d[c] + prev[c] - smallnum for c in range(3)]
                i += 1
                if k == 0:
                    emit(cur)
                    emit(first)
                else:
                    emit(cur)
                prev = cur
        else:
            emit(first)
        smallidx += step_idx
        if not (_XTC_FIRST_SMALL <= smallidx < len(table)):
            raise ValueError("corrupt XTC frame (small-difference index out of range)")
        if step_idx < 0:
            smallnum = smaller
            smaller = table[smallidx - 1] // 2 if smallidx > _XTC_FIRST_SMALL else 0
        elif step_idx > 0:
            smaller = smallnum
            smallnum = table[smallidx] // 2
    if nout != natoms:
        raise ValueError("corrupt XTC frame (%d coordinates for %d atoms)" % (nout, natoms))
    return (out.astype(np.float32) * inv_prec).astype(np.float32)


def read_xtc(path: str, max_frames: Optional[int] = None) -> List[XTCFrame]:
    """Frames of a GROMACS XTC file: positions and unit cell in Angstrom (the file stores nm)."""
    with open(path, "rb") as fh:
        data = fh.read()
    frames: List[XTCFrame] = []
    pos = 0

    def unpack(fmt: str):
        nonlocal pos
        size = struct.calcsize(fmt)
        if pos + size > len(data):
            raise ValueError("truncated XTC frame")
        vals = struct.unpack_from(fmt, data, pos)
        pos += size
        return vals

    while pos < len(data) and (max_frames is None or len(frames) < max_frames):
        magic, natoms, step = unpack(">3i")
        if magic != XTC_MAGIC:
            raise ValueError("not an XTC frame (magic %d)" % magic)
        (time,) = unpack(">f")
        box = np.array(unpack(">9f"), dtype=np.float32).reshape(3, 3)   # rows are the cell vectors
        (natoms2,) = unpack(">i")
        if natoms2 != natoms or natoms < 0:
            raise ValueError("corrupt XTC frame (atom counts differ)")
        if natoms <= 9:
            xyz = np.array(unpack(">%df" % (3 * natoms)), dtype=np.float32).reshape(natoms, 3)
            precision = 0.0
        else:
            (precision,) = unpack(">f")
            minint = unpack(">3i")
            maxint = unpack(">3i")
            (smallidx,) = unpack(">i")
            (nbytes,) = unpack(">i")
            padded = (nbytes + 3) & ~3
            if nbytes < 0 or pos + padded > len(data):
                raise ValueError("truncated XTC coordinate block")
            block = data[pos:pos + nbytes]
            pos += padded
            inv_prec = np.float32(1.0) / np.float32(precision)
            xyz = _xtc_decode_block(block, natoms, minint, maxint, smallidx, inv_prec)
        frames.append(XTCFrame(step=step, time=float(time),
                               positions=xyz.astype(np.float64) * 10.0,
                               unitcell=box.T.astype(np.float64) * 10.0,
                               precision=float(precision)))
    return frames
