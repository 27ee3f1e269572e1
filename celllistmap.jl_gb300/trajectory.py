"""Trajectory ingestion for the pair engine: CHARMM/NAMD DCD frames and PDB coordinates.

The reference reads its NAMD test trajectories with Chemfiles (test/applications/namd/
ParticleSystem_vs_NAMD.jl:21-26) and its argon fixture with PDBTools (src/CellListMap.jl:61).  Neither
is available here, so this module reads the two formats directly:

* DCD: Fortran unformatted records (4-byte length markers, either byte order).  Header record ``CORD``
  with 20 control integers (frame count, ``icntrl[10]`` = unit-cell flag, ``icntrl[8]`` = fixed atoms),
  a title record, the atom count, then per frame an optional unit-cell record of 6 doubles
  (a, gamma, b, beta, alpha, c in the CHARMM order; angles in degrees or as cosines) and three float32
  records x, y, z.
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
                cryst = [float(line[6:15]), float(line[15:24]), float(line[24:33]),
                         float(line[33:40]), float(line[40:47]), float(line[47:54])]
    return np.array(xyz, dtype=np.float64).reshape(-1, 3), cryst
