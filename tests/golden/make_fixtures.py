"""Generate the committed test fixtures from the reference's own test data.

Run once in a checkout where the reference tree is available:

    python tests/golden/make_fixtures.py /path/to/CellListMap.jl

It reads
  * test/applications/gromacs/argon/cubic.pdb  (the reference's ``argon_pdb_file``,
    src/CellListMap.jl:61): 100 argon atoms, fixed-column PDB coordinates parsed as
    Float64, as PDBTools does;
  * test/applications/namd/{o1..o6,t1,t2}.dcd: one frame each of a Neon system,
    CHARMM DCD with float32 coordinates (read by Chemfiles in
    test/applications/namd/ParticleSystem_vs_NAMD.jl:21-26);
  * test/applications/gromacs/argon/{minimal,cubic,dodecahedron,octahedron}.xtc: the first
    frame of each GROMACS run (read by Chemfiles in
    test/applications/gromacs/compare_with_gromacs.jl:15-24), positions and box in Angstrom;
and writes
  * tests/golden/argon_cubic.npy   (100 x 3 float64)
  * tests/golden/namd_frames.npz   (one (n, 3) float32 array per frame)
  * tests/golden/gromacs_argon.npz (``<name>_x``: (n, 3) float64, ``<name>_cell``: 3 x 3 float64 with
    the cell vectors as columns, per run)
Only coordinates are extracted.  The expected values these fixtures are checked
against are quoted, with their source lines, in tests/test_oracle_kat.py.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _trajectory():
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import __graft_entry__ as ge
    return ge.load_package().trajectory


def read_pdb_coords(path):
    return _trajectory().read_pdb(path)[0]


def read_dcd_first_frame(path):
    return _trajectory().read_dcd(path).frames[0]


def main(ref_root):
    pdb = os.path.join(ref_root, "test", "applications", "gromacs", "argon", "cubic.pdb")
    np.save(os.path.join(HERE, "argon_cubic.npy"), read_pdb_coords(pdb))
    frames = {}
    for name in ["o1", "o2", "o3", "o4", "o5", "o6", "t1", "t2"]:
        frames[name] = read_dcd_first_frame(os.path.join(ref_root, "test", "applications", "namd", name + ".dcd"))
    np.savez_compressed(os.path.join(HERE, "namd_frames.npz"), **frames)
    trj = _trajectory()
    gromacs = {}
    for name in ["minimal", "cubic", "dodecahedron", "octahedron"]:
        base = os.path.join(ref_root, "test", "applications", "gromacs", "argon", name)
        frame = trj.read_xtc(base + ".xtc")[0]
        # the decoded frame is the PDB the run started from, up to lattice translations (GROMACS puts the
        # atoms in the box): a check of the XTC decoder on the reference's own files
        start = trj.read_pdb(base + ".pdb")[0]
        frac = np.linalg.solve(frame.unitcell, (frame.positions - start).T).T
        assert np.abs(frac - np.rint(frac)).max() < 1e-6, name
        gromacs[name + "_x"] = frame.positions
        gromacs[name + "_cell"] = frame.unitcell
    np.savez_compressed(os.path.join(HERE, "gromacs_argon.npz"), **gromacs)
    print("wrote fixtures:", sorted(frames), "argon", read_pdb_coords(pdb).shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path to the CellListMap.jl source tree>")
    main(sys.argv[1])
