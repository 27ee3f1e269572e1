"""GPU parity: the CUDA path (through the C ABI) against the oracle on the same seeded inputs.

Bar (stated here):
  * neighbour lists: bit-exact as sorted (min(i,j), max(i,j)) sets, d bit-exact (exact form);
  * counts and histogram counts: exact;
  * energies: relative 1e-12 (Float64) / 1e-5 (Float32) of the FP64 oracle, relative to sum|u|;
  * forces: max-abs error <= 1e-12 (Float64) / 1e-5 (Float32) times max|F_oracle|.
Two per-result bars are looser, on purpose:
  * LJ forces with per-type tables (test_lennard_jones_types): 10x the force bar (1e-11 / 1e-4 times
    max|F_oracle|).  Each term carries (sigma/d)^12 from the hardware reciprocal estimate (a few ulp, times
    12 through the power) and the per-particle sums cancel large repulsive and attractive terms, so the
    error relative to the largest force is about ten times that of the untyped LJ forces;
  * split-form forces (test_split_form_keeps_sets_exact): 1e-4 times max|F_oracle|.  The split form
    computes each pair term in FP32 from cell-relative offsets whose distances carry an absolute error of
    about cell size x 2^-22; its energy keeps the 1e-5 bar.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 1e-5}


def gen(n, dim, span, seed, dtype=np.float64, shift=-1.0):
    rng = np.random.default_rng(seed)
    return (rng.random((n, dim)) * span + shift).astype(dtype)


def kind_of(uc):
    if uc is None:
        return "nonperiodic"
    return "ortho" if np.asarray(uc).ndim == 1 else "tri"


def assert_same_pairs(orc, got, ref, cross=False, exact_d=True, d_rtol=0.0, d_atol=0.0):
    gi, gj, gd = got
    if cross:
        a = np.lexsort((gj, gi))
        b = np.lexsort((ref["j"], ref["i"]))
        A = (gi[a], gj[a], gd[a])
        B = (ref["i"][b], ref["j"][b], ref["d"][b])
    else:
        A = orc.canonical_pairs(gi, gj, gd)
        B = orc.canonical_pairs(ref["i"], ref["j"], ref["d"])
    assert len(A[0]) == len(B[0]), (len(A[0]), len(B[0]))
    np.testing.assert_array_equal(A[0], B[0])
    np.testing.assert_array_equal(A[1], B[1])
    if exact_d:
        np.testing.assert_array_equal(np.asarray(A[2], np.float64), np.asarray(B[2], np.float64))
    else:
        np.testing.assert_allclose(np.asarray(A[2], np.float64), B[2], rtol=d_rtol, atol=d_atol)


CASES = [
    # dim, unitcell, cutoff, lcell, n, span
    (3, [10.0, 12.0, 11.0], 1.5, 1, 3000, 12.0),
    (3, [10.0, 12.0, 11.0], 1.5, 2, 3000, 12.0),
    (3, [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]], 1.5, 1, 3000, 12.0),
    (3, [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]], 1.5, 3, 2000, 12.0),
    (3, None, 1.5, 1, 3000, 12.0),
    (3, None, 1.5, 2, 2000, 12.0),
    (2, [10.0, 12.0], 1.2, 1, 2000, 12.0),
    (2, [[10.0, 3.0], [0.0, 11.0]], 1.2, 2, 2000, 12.0),
    (2, None, 1.2, 1, 2000, 12.0),
]


def ids(c):
    return f"d{c[0]}-{kind_of(c[1])}-l{c[3]}"


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("cross", [False, True])
@pytest.mark.parametrize("case", CASES, ids=ids)
def test_neighborlist_bit_exact(clm, orc, case, cross, dtype):
    dim, uc, cut, lcell, n, span = case
    x = gen(n, dim, span, 11 + lcell, dtype)
    y = gen(n // 2, dim, span, 23 + lcell, dtype) if cross else None
    sysd = clm.ParticleSystem(xpositions=x, ypositions=y, unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    got = clm.pairwise(clm.NeighborList(), sysd)
    ref = orc.run("nl", x, y, dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    assert_same_pairs(orc, got, ref, cross=cross)
    # the cell lists agree copy by copy (same cells, same in-cell order, same coordinates)
    if not cross:
        cl = sysd.fetch_celllist(0)
        oc = orc.celllist(x, dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
        np.testing.assert_array_equal(cl["cell"], oc["cell"])
        np.testing.assert_array_equal(cl["index"], oc["index"])
        np.testing.assert_array_equal(cl["real"], oc["real"])
        np.testing.assert_array_equal(cl["coords"].astype(np.float64), oc["coords"])
    sysd.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("cross", [False, True])
@pytest.mark.parametrize("case", CASES[:5] + CASES[6:8], ids=ids)
def test_energy_and_forces(clm, orc, case, cross, dtype):
    dim, uc, cut, lcell, n, span = case
    x = gen(n, dim, span, 5 + lcell, dtype)
    y = gen(n // 2, dim, span, 9 + lcell, dtype) if cross else None
    s = clm.ParticleSystem(xpositions=x, ypositions=y, unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    kw = dict(dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell, dtype=dtype)
    tol = TOL[dtype]
    ef = clm.pairwise(clm.SoftForces(), s)
    r = orc.run("soft_forces", x, y, **kw)
    assert abs(ef.energy - r["scalar"]) <= tol * abs(r["scalar"]) + 1e-300
    fx = np.asarray(ef.forces, np.float64)
    assert np.abs(fx - r["forces_x"]).max() <= tol * max(np.abs(r["forces_x"]).max(), 1e-300)
    if cross:
        fy = np.asarray(ef.forces_y, np.float64)
        assert np.abs(fy - r["forces_y"]).max() <= tol * max(np.abs(r["forces_y"]).max(), 1e-300)
    # scalar reductions
    for op, cls in [("sum_d2", clm.SumD2()), ("sum_d", clm.SumD()), ("soft_energy", clm.SoftEnergy())]:
        e = clm.pairwise(cls, s)
        rr = orc.run(op, x, y, **kw)
        assert abs(e - rr["scalar"]) <= tol * abs(rr["scalar"]) + 1e-300, op
    c = clm.pairwise(clm.Count(), s)
    assert c == orc.run("count", x, y, **kw)["count"]
    s.close()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_lennard_jones_types(clm, orc, dtype):
    rng = np.random.default_rng(3)
    x = gen(4000, 3, 14.0, 4, dtype, shift=0.0)
    types = (rng.random(4000) < 0.2).astype(np.int32)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    s = clm.ParticleSystem(xpositions=x, unitcell=[14.0, 14.0, 14.0], cutoff=2.5, dtype=dtype)
    ef = clm.pairwise(clm.LennardJonesForces(types_x=types, eps_table=eps, sig_table=sig), s)
    r = orc.run("lj_forces", x, unitcell=[14.0, 14.0, 14.0], cutoff=2.5, dtype=dtype, params=[1.0, 1.0, 4.0, 4.0],
                types_x=types, eps_table=eps, sig_table=sig)
    tol = TOL[dtype]
    # LJ terms cancel: compare against the scale of the terms, not the total
    scale = orc.run("lj_energy", x, unitcell=[14.0, 14.0, 14.0], cutoff=2.5, dtype=dtype, params=[1.0, 1.0, 4.0, 0.0],
                    types_x=types, eps_table=eps, sig_table=sig)["scalar"]
    assert abs(ef.energy - r["scalar"]) <= tol * (abs(r["scalar"]) + abs(scale))
    assert np.abs(np.asarray(ef.forces, np.float64) - r["forces_x"]).max() <= tol * np.abs(r["forces_x"]).max() * 10
    s.close()


def test_argon_kats_on_gpu(clm, orc, golden_dir):
    import os
    x = np.load(os.path.join(golden_dir, "argon_cubic.npy"))
    s = clm.ParticleSystem(xpositions=x, unitcell=[21.0, 21.0, 21.0], cutoff=8.0)
    assert clm.pairwise(clm.SumD2(), s) == pytest.approx(43774.54367600001, rel=1e-12)
    assert clm.pairwise(clm.MinimumDistance(), s)[2] == 2.1991993997816563
    ef = clm.pairwise(clm.InverseDistanceForces(), s)
    assert ef.energy == pytest.approx(207.37593043370862, rel=1e-12)
    np.testing.assert_allclose(ef.forces[0], [0.02649383330735732, 0.18454277989323772, -0.012253902366284958],
                               rtol=1e-10)
    s.close()
    x32 = x.astype(np.float32).astype(np.float64)
    i, j, d = clm.neighborlist(xpositions=x32, cutoff=8.0, unitcell=[21.0, 21.0, 21.0])
    assert len(i) == 1143
    a, b, dd = orc.canonical_pairs(i, j, d)
    assert dd[(a == 0) & (b == 6)][0] == 3.3638756414119397
    i, j, d = clm.neighborlist(xpositions=x32, cutoff=8.0)
    assert len(i) == 857
    i, j, d = clm.neighborlist(xpositions=x32[:50], ypositions=x32[50:], cutoff=8.0)
    assert len(i) == 439
    assert d[(i == 0) & (j == 29)][0] == 2.4572288423012236


@pytest.mark.parametrize("name,lcell", [("o1", 1), ("o3", 1), ("t1", 1), ("t2", 3), ("o6", 3)])
def test_namd_lj_on_gpu(clm, golden_dir, name, lcell):
    import os
    from tests.test_oracle_kat import NAMD_CASES, NAMD_EPS, NAMD_SIG
    f = np.load(os.path.join(golden_dir, "namd_frames.npz"))
    uc, expected = [(c[1], c[2]) for c in NAMD_CASES if c[0] == name][0]
    s = clm.ParticleSystem(xpositions=f[name].astype(np.float64), unitcell=np.asarray(uc, float), cutoff=10.0,
                           lcell=lcell)
    u = clm.pairwise(clm.LennardJones(NAMD_EPS, NAMD_SIG, 1.0, 2.0), s)
    assert u == pytest.approx(expected, rel=1e-12)
    s.close()


@pytest.mark.parametrize("lcell", [1, 2, 3])
@pytest.mark.parametrize("name", ["minimal", "cubic", "dodecahedron", "octahedron"])
def test_gromacs_lj_on_gpu(clm, orc, golden_dir, name, lcell):
    from tests.test_oracle_kat import GROMACS_C12, GROMACS_C6, GROMACS_CASES, gromacs_frame
    x, kind, uc = gromacs_frame(golden_dir, name)
    expected = dict(GROMACS_CASES)[name]
    s = clm.ParticleSystem(xpositions=x, unitcell=uc, cutoff=8.0, lcell=lcell)
    u = clm.pairwise(clm.LennardJones(1.0, 1.0, GROMACS_C12, GROMACS_C6), s)
    s.close()
    r = orc.run("lj_energy", x, kind=kind, unitcell=uc, cutoff=8.0, lcell=lcell,
                params=[1.0, 1.0, GROMACS_C12, GROMACS_C6])
    assert u == pytest.approx(r["scalar"], rel=1e-12)
    assert u == pytest.approx(expected, rel=1e-5)


@pytest.mark.parametrize("cross", [False, True])
def test_min_distance_and_histogram(clm, orc, cross):
    x = gen(3000, 3, 20.0, 77)
    y = gen(2000, 3, 20.0, 78) if cross else None
    uc = [20.0, 20.0, 20.0]
    s = clm.ParticleSystem(xpositions=x, ypositions=y, unitcell=uc, cutoff=2.0)
    i, j, d = clm.pairwise(clm.MinimumDistance(), s)
    r = orc.run("mindist", x, y, unitcell=uc, cutoff=2.0)
    assert d == r["min"][2]
    rng = np.random.default_rng(1)
    vx = rng.normal(size=x.shape)
    vy = rng.normal(size=y.shape) if cross else None
    bins = 10 ** np.linspace(np.log10(0.1), np.log10(2.0), 21)
    hc, hs = clm.pairwise(clm.RadialHistogram(bins, vx, vy), s)
    rr = orc.run("rhist", x, y, unitcell=uc, cutoff=2.0, bins=bins, vel_x=vx, vel_y=vy)
    np.testing.assert_array_equal(hc, rr["hist_count"])
    np.testing.assert_allclose(hs, rr["hist_sum"], rtol=1e-10, atol=1e-9 * np.abs(rr["hist_sum"]).max())
    s.close()


@pytest.mark.parametrize("dim", [3, 2])
@pytest.mark.parametrize("cross", [False, True])
def test_histogram_split_form(clm, orc, cross, dim):
    """FP32-split histogram: counts exact; per-bin sums within 1e-5 of the bin's sum of |v_i - v_j|
    (a bound on the sum of |terms|), the FP32 pair arithmetic being accumulated in FP64."""
    x = gen(3000, dim, 20.0, 87)
    y = gen(2500, dim, 20.0, 88) if cross else None
    uc = [20.0] * dim
    rng = np.random.default_rng(3)
    vx = rng.normal(0, 300.0, x.shape)
    vy = rng.normal(0, 300.0, y.shape) if cross else None
    bins = 10 ** np.linspace(np.log10(0.1), np.log10(2.0), 21)
    s = clm.ParticleSystem(xpositions=x, ypositions=y, unitcell=uc, cutoff=2.0, precision="split")
    hc, hs = clm.pairwise(clm.RadialHistogram(bins, vx, vy), s)
    rr = orc.run("rhist", x, y, dim=dim, unitcell=uc, cutoff=2.0, bins=bins, vel_x=vx, vel_y=vy)
    np.testing.assert_array_equal(hc, rr["hist_count"])
    nl = orc.run("nl", x, y, dim=dim, unitcell=uc, cutoff=2.0)
    vyy = vy if cross else vx
    dv = np.linalg.norm(vx[nl["i"]] - vyy[nl["j"]], axis=1)
    b = np.searchsorted(bins, nl["d"], side="left") - 1
    ok = (b >= 0) & (b < len(bins) - 1)
    scale = np.bincount(b[ok], weights=dv[ok], minlength=len(bins) - 1)
    assert np.all(np.abs(hs - rr["hist_sum"]) <= 1e-5 * scale + 1e-9)
    s.close()


@pytest.mark.parametrize("case", [CASES[0], CASES[2], CASES[4]], ids=ids)
def test_split_form_keeps_sets_exact(clm, orc, case):
    dim, uc, cut, lcell, n, span = case
    x = gen(n, dim, span, 31)
    s = clm.ParticleSystem(xpositions=x, unitcell=uc, cutoff=cut, lcell=lcell, precision="split")
    got = clm.pairwise(clm.NeighborList(), s)
    ref = orc.run("nl", x, dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell)
    # split form: d carries the FP32 offset error, absolute ~ cell size * 2^-22
    assert_same_pairs(orc, got, ref, exact_d=False, d_rtol=1e-6, d_atol=2e-6 * cut)
    assert clm.pairwise(clm.Count(), s) == len(ref["i"])
    ef = clm.pairwise(clm.SoftForces(), s)
    r = orc.run("soft_forces", x, dim=dim, kind=kind_of(uc), unitcell=uc, cutoff=cut, lcell=lcell)
    assert abs(ef.energy - r["scalar"]) <= 1e-5 * abs(r["scalar"])
    assert np.abs(ef.forces - r["forces_x"]).max() <= 1e-4 * np.abs(r["forces_x"]).max()
    s.close()


def test_pathological_coordinates_gpu(clm, orc):
    rng = np.random.default_rng(5)
    sides = np.array([250.0, 250.0, 250.0])
    x = sides * rng.random((2000, 3))
    x[0] = -sides / 2
    x[1] = -sides / 2 + [np.nextafter(0, 1), np.nextafter(0, 1), sides[2] * rng.random()]
    x[2] = -sides / 2 + [np.nextafter(0, -1), np.nextafter(0, -1), sides[2] * rng.random()]
    x[3] = sides / 2 + [np.nextafter(0, 1), np.nextafter(0, 1), sides[2] * rng.random()]
    x[4] = sides / 2 + [np.nextafter(0, -1), np.nextafter(0, -1), sides[2] * rng.random()]
    x[9] = sides
    x[10] = sides + [np.nextafter(0, 1), np.nextafter(0, 1), sides[2] * rng.random()]
    x[11] = sides + [np.nextafter(0, -1), np.nextafter(0, -1), sides[2] * rng.random()]
    x[12] = [np.nextafter(0, 1), np.nextafter(0, 1), sides[2] * rng.random()]
    x[13] = [np.nextafter(0, -1), np.nextafter(0, -1), sides[2] * rng.random()]
    x[14] = 0.0
    x[99] = [sides[0] / 2, -sides[1] / 2, 2 * sides[2]]
    for lcell in (1, 2):
        got = clm.neighborlist(xpositions=x, unitcell=sides, cutoff=10.0, lcell=lcell)
        ref = orc.run("nl", x, unitcell=sides, cutoff=10.0, lcell=lcell)
        assert_same_pairs(orc, got, ref)


def test_small_exact_cases_gpu(clm):
    side = 2.0 + np.nextafter(1.0, 2.0)
    i, j, d = clm.neighborlist(xpositions=[[0.0, 0.0], [0.0, 1.0]], cutoff=1.0, unitcell=[side, side])
    assert list(zip(np.minimum(i, j), np.maximum(i, j), d)) == [(0, 1, 1.0)]
    i, j, d = clm.neighborlist(xpositions=[[0.0, 0.0], [0.0, 1.0]], cutoff=np.nextafter(1.0, 0.0), unitcell=[2.0, 2.0])
    assert len(i) == 0
    i, j, d = clm.neighborlist(xpositions=[[0.0, 0.0]], cutoff=2.0)
    assert len(i) == 0
    i, j, d = clm.neighborlist(xpositions=[[0.0, 0.0, 1.0], [0.0, 0.0, 10.0], [0.0, 0.0, 7.0]], cutoff=2.0)
    assert len(i) == 0
    for xx in [np.nextafter(0.1, 1.0), np.nextafter(0.9, 0.0)]:
        assert len(clm.neighborlist(xpositions=[[0.0, 0.0], [xx, 0.0]], cutoff=0.1, unitcell=[1.0, 1.0])[0]) == 0
    for xx in [-0.1, 0.1, 0.9]:
        assert len(clm.neighborlist(xpositions=[[0.0, 0.0], [xx, 0.0]], cutoff=0.1, unitcell=[1.0, 1.0])[0]) == 1


def test_errors_map_to_reference_exceptions(clm):
    x = gen(100, 3, 10.0, 1)
    with pytest.raises(clm.ArgumentError):
        clm.ParticleSystem(xpositions=x, unitcell=[10.0, 10.0, 10.0], cutoff=5.0)  # cell too small
    with pytest.raises(clm.ArgumentError):
        clm.ParticleSystem(xpositions=x, unitcell=[10.0, 10.0, 10.0], cutoff=1.0, lcell=0)
    bad = x.copy()
    bad[7, 2] = np.nan
    with pytest.raises(clm.ArgumentError):
        clm.ParticleSystem(xpositions=bad, unitcell=[10.0, 10.0, 10.0], cutoff=1.0)
    with pytest.raises(clm.ArgumentError):
        clm.ParticleSystem(xpositions=bad, cutoff=1.0)
    with pytest.raises(clm.ArgumentError):  # get_dim, src/internals/auxiliary_functions.jl:104-110
        clm.ParticleSystem(xpositions=x[:, :2], unitcell=[10.0, 10.0, 10.0], cutoff=1.0)
    s = clm.ParticleSystem(xpositions=x, cutoff=1.0)
    with pytest.raises(clm.DimensionMismatch):  # UpdateCellList!, src/internals/CellLists.jl:740-751
        s.update(xpositions=x[:, :2])
    with pytest.raises(clm.ArgumentError):
        s.update(unitcell=[10.0, 10.0, 10.0])
    s.close()


def test_update_flow_and_empty_sets(clm, orc):
    """update!: positions, number of particles, cutoff and unit cell changes (test/internals/tests.jl:301-455)."""
    x = gen(3000, 3, 12.0, 3)
    s = clm.InPlaceNeighborList(xpositions=x, cutoff=1.2, unitcell=[12.0, 12.0, 12.0])
    for step in range(3):
        x2 = gen(2000 + 700 * step, 3, 12.0, 100 + step)
        cut = 1.0 + 0.2 * step
        uc = [12.0 + step, 12.0, 12.5]
        clm.update(s, xpositions=x2, cutoff=cut, unitcell=uc)
        got = clm.neighborlist_(s)
        ref = orc.run("nl", x2, unitcell=uc, cutoff=cut)
        assert_same_pairs(orc, got, ref)
    clm.update(s, xpositions=np.zeros((0, 3)))
    assert len(clm.neighborlist_(s)[0]) == 0
    s.sys.close()


def test_device_resident_positions(clm, orc):
    torch = pytest.importorskip("torch")
    x = gen(5000, 3, 15.0, 8)
    xt = torch.tensor(x, device="cuda")
    s = clm.ParticleSystem(xpositions=xt, unitcell=[15.0, 15.0, 15.0], cutoff=1.5)
    got = clm.pairwise(clm.NeighborList(), s)
    ref = orc.run("nl", x, unitcell=[15.0, 15.0, 15.0], cutoff=1.5)
    assert_same_pairs(orc, got, ref)
    s.close()


def test_determinism(clm):
    x = gen(20000, 3, 30.0, 9)
    s = clm.ParticleSystem(xpositions=x, unitcell=[30.0, 30.0, 30.0], cutoff=2.0)
    e1 = clm.pairwise(clm.SoftEnergy(), s)
    s.update(xpositions=x)
    e2 = clm.pairwise(clm.SoftEnergy(), s)
    assert e1 == e2  # fixed-order reductions: bitwise reproducible
    s.close()


@pytest.mark.parametrize("via_run", [False, True])
def test_copy_capacity_overflow_rebuilds(clm, orc, via_run):
    """Particles packed in a corner have 7 images each, far above the uniform-density capacity estimate:
    the build must detect the overflow on the device and repeat with the exact size."""
    rng = np.random.default_rng(4)
    x = 0.05 + 0.04 * rng.random((6000, 3))
    uc = [10.0, 10.0, 10.0]
    s = clm.ParticleSystem(xpositions=x[:10], unitcell=uc, cutoff=1.0)
    s.update(xpositions=x)  # dirty: the next pairwise builds without waiting for the device
    if not via_run:
        s.build()
    got = clm.pairwise(clm.NeighborList(), s)
    ref = orc.run("nl", x, unitcell=uc, cutoff=1.0)
    assert_same_pairs(orc, got, ref)
    assert s.celllist_info()["n_particles"] == 8 * len(x)
    s.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_clustered_cells_switch_to_the_radix_build(clm, orc, dtype):
    """A blob of 3000 particles inside one or two cells of a large box: the uniform-density estimate picks the
    counting build, which then finds cells of more than 1024 copies, and the set's later builds sort by
    radix (more launches per build than the counting build of a uniform set of the same size).  Every
    build's cell list (copy by copy) and neighbour list must equal the oracle's."""
    import ctypes as C
    L = clm._abi.load()

    def launches(sys_):
        v = C.c_int64()
        assert L.clm_stats(sys_._handle.h, C.byref(v)) == 0
        return v.value

    def step_launches(sys_, xx):
        sys_.update(xpositions=xx)  # the next map rebuilds
        n0 = launches(sys_)
        got = clm.pairwise(clm.NeighborList(), sys_)
        return got, launches(sys_) - n0

    rng = np.random.default_rng(21)
    uc = [20.0, 20.0, 20.0]
    kw = dict(unitcell=uc, cutoff=1.0, dtype=dtype)
    u = (20.0 * rng.random((3000, 3))).astype(dtype)  # the same number of particles, uniform: counting build
    su = clm.ParticleSystem(xpositions=u, unitcell=uc, cutoff=1.0, dtype=dtype)
    _, counting = step_launches(su, u)
    su.close()
    x = (10.2 + 0.5 * rng.random((3000, 3))).astype(dtype)
    s = clm.ParticleSystem(xpositions=x, unitcell=uc, cutoff=1.0, dtype=dtype)
    per_step = []
    for step in range(3):
        x = (x + dtype(0.01)).astype(dtype)
        got, nl = step_launches(s, x)
        per_step.append(nl)
        assert_same_pairs(orc, got, orc.run("nl", x, **kw))
        cl = s.fetch_celllist(0)
        oc = orc.celllist(x, **kw)
        np.testing.assert_array_equal(cl["cell"], oc["cell"])
        np.testing.assert_array_equal(cl["index"], oc["index"])
        np.testing.assert_array_equal(cl["coords"].astype(np.float64), oc["coords"])
    assert per_step[-1] > counting, (per_step, counting)
    s.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_many_scan_tiles(clm, orc, dtype):
    """~200k particles of the headline geometry: the build's scans run over ~100 tiles (copy offsets) and
    ~170 tiles x 512 digits (radix histograms), so the single-pass look-back is exercised across many
    tiles; the cell list (copy by copy), the neighbour list, the LJ energy and forces match the oracle."""
    x, M = clm.workloads.cfg2(ncell=37)
    x = x.astype(dtype)
    kw = dict(kind="tri", unitcell=M, cutoff=2.5, dtype=dtype)
    s = clm.ParticleSystem(xpositions=x, unitcell=M, cutoff=2.5, dtype=dtype)
    got = clm.pairwise(clm.NeighborList(), s)
    assert_same_pairs(orc, got, orc.run("nl", x, **kw))
    cl = s.fetch_celllist(0)
    oc = orc.celllist(x, **kw)
    np.testing.assert_array_equal(cl["cell"], oc["cell"])
    np.testing.assert_array_equal(cl["index"], oc["index"])
    np.testing.assert_array_equal(cl["coords"].astype(np.float64), oc["coords"])
    ef = clm.pairwise(clm.LennardJonesForces(1.0, 1.0, 4.0, 4.0), s)
    r = orc.run("lj_forces", x, params=[1.0, 1.0, 4.0, 4.0], **kw)
    tol = TOL[dtype]
    assert abs(ef.energy - r["scalar"]) <= tol * abs(r["scalar"])
    fx = np.asarray(ef.forces, np.float64)
    assert np.abs(fx - r["forces_x"]).max() <= tol * np.abs(r["forces_x"]).max()
    s.close()

