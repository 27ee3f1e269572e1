"""Batches of independent systems (one build and one launch per kernel for all systems) against the
oracle run system by system.

Bar: neighbour lists bit-exact per system as sorted (i, j) sets with d bit-exact (exact form); counts
exact; soft energies and forces within 1e-12 (Float64) / 1e-5 (Float32) relative to the oracle's sum of
|u| (energies) or max |F| (forces).  Systems whose cell fails the reference's check report
CLM_ERR_CELL_TOO_SMALL and NaN sums without disturbing the others.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RC = 6.0


def make_batch(nsys=40, nmin=64, nmax=3000, rho=0.1, seed=11, tri=False, dtype=np.float64):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nsys)).astype(np.int64)
    sizes[0] = 100  # side 10 < 2 cutoff: fails the unit-cell check
    pos, cells = [], []
    for n in sizes:
        L = (n / rho) ** (1.0 / 3.0)
        if tri:
            M = np.array([[L, 0.2 * L, 0.1 * L], [0.0, L, 0.15 * L], [0.0, 0.0, L]])
            x = rng.random((n, 3)) @ M.T
            cells.append(M)
        else:
            x = rng.random((n, 3)) * L
            cells.append([L, L, L])
        pos.append(x.astype(dtype))
    return pos, np.array(cells)


def cell_ok(cell):
    """The reference's unit-cell check: every distance between opposite cell faces exceeds 2 cutoff."""
    cell = np.asarray(cell, np.float64)
    M = np.diag(cell) if cell.ndim == 1 else cell
    a, b, c = M[:, 0], M[:, 1], M[:, 2]
    V = abs(np.dot(a, np.cross(b, c)))
    return min(V / np.linalg.norm(np.cross(b, c)), V / np.linalg.norm(np.cross(c, a)),
               V / np.linalg.norm(np.cross(a, b))) > 2 * RC


def oracle_system(orc, x, cell, op, dtype, params=(), lcell=1):
    cell = np.asarray(cell)
    kind = "ortho" if cell.ndim == 1 else "tri"
    return orc.run(op, x, dim=3, kind=kind, unitcell=cell, cutoff=RC, lcell=lcell, dtype=dtype, params=params)


def check_batch(orc, clm, bs, pos, cells, dtype, exact_d=True, forces=False, lcell=1):
    """lcell: the batch's cells per cutoff; the oracle runs with the same one (which copy of a pair, real
    or image, is met depends on the computing box, and d is that copy's distance)."""
    tol = 1e-12 if dtype == np.float64 else 1e-5
    ops = [clm.NeighborList(), clm.SoftEnergy()]
    if forces:
        ops.append(clm.SoftForces())
    res = bs.run(*ops)
    nls, energies = res[0], res[1]
    status = bs.status()
    off = bs.offsets
    for s, (x, cell) in enumerate(zip(pos, cells)):
        if not cell_ok(cell):
            assert status[s] == 2, (s, status[s])
            assert np.isnan(energies[s])
            continue
        assert status[s] == 0
        ref = oracle_system(orc, x, cell, "nl", dtype, lcell=lcell)
        gi, gj, gd = nls[s]
        A = orc.canonical_pairs(gi, gj, gd)
        B = orc.canonical_pairs(ref["i"], ref["j"], ref["d"])
        np.testing.assert_array_equal(A[0], B[0])
        np.testing.assert_array_equal(A[1], B[1])
        if exact_d:
            np.testing.assert_array_equal(np.asarray(A[2], np.float64), np.asarray(B[2], np.float64))
        else:
            np.testing.assert_allclose(np.asarray(A[2], np.float64), B[2], rtol=2e-6, atol=2e-6 * RC)
        e = oracle_system(orc, x, cell, "soft_energy", dtype, params=[RC])
        d = np.asarray(ref["d"], np.float64)
        scale = np.sum((RC - d) ** 2) + 1e-300
        assert abs(energies[s] - e["scalar"]) <= tol * scale, (s, energies[s], e["scalar"])
        if forces:
            fr = oracle_system(orc, x, cell, "soft_forces", dtype, params=[RC])
            f = np.asarray(res[2].forces[off[s]:off[s + 1]], np.float64)
            fs = np.abs(fr["forces_x"]).max() + 1e-300
            assert np.abs(f - fr["forces_x"]).max() <= tol * fs
            assert abs(res[2].energy[s] - fr["scalar"]) <= tol * scale


@pytest.mark.parametrize("tri", [False, True])
def test_batch_f64_exact(orc, clm, tri):
    pos, cells = make_batch(tri=tri)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    check_batch(orc, clm, bs, pos, cells, np.float64, forces=True)


def test_batch_f32(orc, clm):
    pos, cells = make_batch(nsys=24, dtype=np.float32, seed=5)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC, dtype=np.float32)
    check_batch(orc, clm, bs, pos, cells, np.float32, forces=True)


def test_batch_split_form(orc, clm):
    pos, cells = make_batch(nsys=24, seed=6)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC, precision="split")
    # the split form keeps the pair set exact; sums carry FP32 pair arithmetic (1e-5 of sum |u|)
    res = bs.run(clm.NeighborList(), clm.SoftEnergy())
    for s, (x, cell) in enumerate(zip(pos, cells)):
        if not cell_ok(cell):
            continue
        ref = oracle_system(orc, x, cell, "nl", np.float64)
        A = orc.canonical_pairs(*res[0][s])
        B = orc.canonical_pairs(ref["i"], ref["j"], ref["d"])
        np.testing.assert_array_equal(A[0], B[0])
        np.testing.assert_array_equal(A[1], B[1])
        e = oracle_system(orc, x, cell, "soft_energy", np.float64, params=[RC])
        d = np.asarray(ref["d"], np.float64)
        assert abs(res[1][s] - e["scalar"]) <= 1e-5 * np.sum((RC - d) ** 2)


def test_batch_lcell_and_parts(orc, clm):
    pos, cells = make_batch(nsys=16, seed=7)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    for lc, sp, gd in [(2, 1, 1), (3, 2, 2), (1, 2, 1)]:
        bs.set_config(lcell=lc, cell_split=sp, grid_div=gd)
        check_batch(orc, clm, bs, pos, cells, np.float64, lcell=lc)


def test_batch_graph_replay_and_update(orc, clm):
    pos, cells = make_batch(nsys=20, seed=8)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC, graph=True)
    first = bs.run(clm.SoftEnergy(), clm.Count())
    again = bs.run(clm.SoftEnergy(), clm.Count())  # replayed graph
    np.testing.assert_array_equal(first[0], again[0])
    np.testing.assert_array_equal(first[1], again[1])
    st = bs.last_step()
    assert st["launches"] > 0 and st["step_ms"] > 0
    rng = np.random.default_rng(1)
    moved = [x + rng.normal(0, 0.3, x.shape) for x in pos]
    bs.update(positions=np.concatenate(moved))
    check_batch(orc, clm, bs, moved, cells, np.float64)
    check_batch(orc, clm, bs, moved, cells, np.float64)  # replay after the recording with NL


def test_batch_nan_marks_one_system(orc, clm):
    pos, cells = make_batch(nsys=10, seed=9)
    pos[3] = pos[3].copy()
    pos[3][5, 1] = np.nan
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    e = bs.run(clm.SoftEnergy())[0]
    st = bs.status()
    assert st[3] == 3 and np.isnan(e[3])
    for s in range(10):
        if s in (0, 3) or not cell_ok(cells[s]):
            continue
        assert st[s] == 0
        ref = oracle_system(orc, pos[s], cells[s], "soft_energy", np.float64, params=[RC])
        assert abs(e[s] - ref["scalar"]) <= 1e-12 * max(1.0, abs(ref["scalar"])) * 10


def test_batch_autotune(orc, clm):
    pos, cells = make_batch(nsys=30, seed=10)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    cfg = bs.autotune(clm.NeighborList(), clm.SoftEnergy(), reps=2)
    assert cfg["lcell"] in (1, 2, 3) and cfg["cell_split"] in (1, 2) and cfg["grid_div"] in (1, 2)
    assert cfg["step_ms"] > 0
    check_batch(orc, clm, bs, pos, cells, np.float64, lcell=cfg["lcell"])


def test_batch_matches_plain_path(clm):
    pos, cells = make_batch(nsys=12, seed=12)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    cnt, e = bs.run(clm.Count(), clm.SoftEnergy())
    for s, (x, cell) in enumerate(zip(pos, cells)):
        if not cell_ok(cell):
            continue
        sysm = clm.ParticleSystem(positions=x, unitcell=cell, cutoff=RC)
        assert clm.pairwise(clm.Count(), sysm) == cnt[s]
        ref = clm.pairwise(clm.SoftEnergy(), sysm)
        assert abs(ref - e[s]) <= 1e-12 * max(1.0, abs(ref))


def test_batch_errors(clm):
    pos, cells = make_batch(nsys=4, seed=13)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    with pytest.raises(clm.ArgumentError):
        bs.run(clm.MinimumDistance())
    with pytest.raises(clm.DimensionMismatch):
        bs.update(positions=np.concatenate(pos)[:-1])


def test_batch_2d(orc, clm):
    rng = np.random.default_rng(21)
    pos, cells = [], []
    for n in (50, 300, 900, 2000):
        L = (n / 0.3) ** 0.5
        pos.append(rng.random((n, 2)) * L)
        cells.append([L, L])
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC)
    nls, e = bs.run(clm.NeighborList(), clm.SoftEnergy())
    st = bs.status()
    for s, (x, L) in enumerate(zip(pos, cells)):
        if min(L) <= 2 * RC:
            assert st[s] == 2
            continue
        ref = orc.run("nl", x, dim=2, kind="ortho", unitcell=L, cutoff=RC)
        A = orc.canonical_pairs(*nls[s])
        B = orc.canonical_pairs(ref["i"], ref["j"], ref["d"])
        np.testing.assert_array_equal(A[0], B[0])
        np.testing.assert_array_equal(A[1], B[1])
        np.testing.assert_array_equal(A[2], B[2])
        er = orc.run("soft_energy", x, dim=2, kind="ortho", unitcell=L, cutoff=RC, params=[RC])["scalar"]
        assert abs(e[s] - er) <= 1e-12 * max(1.0, abs(er)) * 10


def test_batch_graph_follows_precision(orc, clm):
    pos, cells = make_batch(nsys=8, seed=14)
    bs = clm.BatchedSystems(positions=pos, unitcells=cells, cutoff=RC, graph=True)
    exact = [bs.run(clm.SoftEnergy())[0] for _ in range(2)][-1]  # recorded and replayed
    bs.set_precision("split")
    split = bs.run(clm.SoftEnergy())[0]
    bs.set_precision("exact")
    again = bs.run(clm.SoftEnergy())[0]
    np.testing.assert_array_equal(exact, again)
    ok = ~np.isnan(exact)
    assert np.any(split[ok] != exact[ok])  # the split form ran (FP32 pair values differ in the last bits)
    np.testing.assert_allclose(split[ok], exact[ok], rtol=1e-5)
