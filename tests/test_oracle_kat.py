"""CPU tests: the oracle against the reference's known-answer values and its naive O(N^2) check.

Expected values are quoted from the reference (file:line beside each).
"""
import os

import numpy as np
import pytest

ARGON_SIDES = [21.0, 21.0, 21.0]


@pytest.fixture(scope="module")
def argon(golden_dir):
    return np.load(os.path.join(golden_dir, "argon_cubic.npy"))


@pytest.fixture(scope="module")
def namd(golden_dir):
    return np.load(os.path.join(golden_dir, "namd_frames.npz"))


def test_argon_sum_d2(orc, argon):
    # src/API/ParticleSystem.jl:110-118
    r = orc.run("sum_d2", argon, unitcell=ARGON_SIDES, cutoff=8.0)
    assert r["scalar"] == pytest.approx(43774.54367600001, rel=1e-12)


def test_argon_two_sets_sum_d2(orc, argon):
    # src/API/ParticleSystem.jl:122-139
    r = orc.run("sum_d2", argon[:50], argon[50:], unitcell=ARGON_SIDES, cutoff=8.0)
    assert r["scalar"] == pytest.approx(21886.196785000004, rel=1e-12)


def test_argon_neighborlists(orc, argon):
    # src/API/neighborlist.jl:262-311.  These docstrings were produced with PDBTools returning Float32
    # coordinates (promoted to Float64 by the Float64 cutoff): with them every quoted distance is bit-exact.
    x32 = argon.astype(np.float32).astype(np.float64)
    nl = orc.run("nl", x32, kind="nonperiodic", cutoff=8.0)
    assert len(nl["i"]) == 857
    a, b, d = orc.canonical_pairs(nl["i"], nl["j"], nl["d"])
    for (i, j), dist in {(0, 19): 3.163779526466901, (0, 60): 4.08865164675529, (0, 66): 5.939772435456664,
                         (77, 87): 7.0061163797598445, (53, 87): 7.933654063435482}.items():
        assert d[(a == i) & (b == j)][0] == dist
    nl = orc.run("nl", x32, unitcell=ARGON_SIDES, cutoff=8.0)
    assert len(nl["i"]) == 1143
    a, b, d = orc.canonical_pairs(nl["i"], nl["j"], nl["d"])
    for (i, j), dist in {(0, 6): 3.3638756414119397, (0, 19): 3.163779526466901, (0, 46): 6.243868666689442,
                         (37, 67): 7.409287768713663, (67, 89): 7.8758006026725464}.items():
        assert d[(a == i) & (b == j)][0] == dist
    nl = orc.run("nl", x32[:50], x32[50:], kind="nonperiodic", cutoff=8.0)
    assert len(nl["i"]) == 439
    for (i, j), dist in {(0, 10): 4.08865164675529, (0, 16): 5.939772435456664, (0, 29): 2.4572288423012236,
                         (45, 47): 4.9269093987894745, (45, 0): 7.99947286297016}.items():
        assert nl["d"][(nl["i"] == i) & (nl["j"] == j)][0] == dist


def test_argon_min_distance(orc, argon):
    # src/API/parallel_custom.jl:174-192
    r = orc.run("mindist", argon, unitcell=ARGON_SIDES, cutoff=8.0)
    assert r["min"][2] == 2.1991993997816563  # bit-exact with Float64 coordinates


def test_argon_inverse_distance_and_gradient(orc, argon):
    # docs/src/ParticleSystem/single_set_compound.md:103-117
    r = orc.run("inv_d_forces", argon, unitcell=ARGON_SIDES, cutoff=8.0)
    assert r["scalar"] == pytest.approx(207.37593043370862, rel=1e-13)
    np.testing.assert_allclose(r["forces_x"][0], [0.02649383330735732, 0.18454277989323772, -0.012253902366284958],
                               rtol=1e-10)
    np.testing.assert_allclose(r["forces_x"][-1], [-0.031012009183076745, 0.03543655648545698, 0.03184912163097636],
                               rtol=1e-10)


def test_argon_nonperiodic_box(orc, argon):
    # test/API/ParticleSystem.jl:214-223 (sides of the non-periodic box, 2 decimals)
    b8 = orc.box_info(argon, kind="nonperiodic", cutoff=8.0)
    np.testing.assert_allclose(np.diag(b8["input_unit_cell"]), [35.63, 35.76, 35.79], atol=6e-3)
    b10 = orc.box_info(argon, kind="nonperiodic", cutoff=10.0)
    np.testing.assert_allclose(np.diag(b10["input_unit_cell"]), [39.83, 39.96, 39.99], atol=6e-3)


NAMD_CASES = [
    # test/applications/namd/ParticleSystem_vs_NAMD.jl:55-116
    ("o1", [50.0, 50.0, 50.0], 32230.01699504111),
    ("o2", [80.0, 70.0, 50.0], 1093.7225407797744),
    ("o3", [[50.0, 0.0, 50.0], [50.0, 50.0, 0.0], [0.0, 50.0, 50.0]], 1724.3195067566828),
    ("o4", np.array([[70.7107, 0.0, 0.0], [35.3553, 61.2372, 0.0], [35.3553, 20.4124, 57.735]]).T, 1754.0802503953591),
    ("o5", np.array([[70.7107, 0.0, 0.0], [35.3553, 61.2372, 0.0], [35.3553, 20.4124, 57.735]]).T, 1765.1389457850137),
    ("o6", [80.0, 80.0, 80.0], -158.04751357760088),
    ("t1", [[80.0, 0.0, 30.0], [30.0, 80.0, 0.0], [0.0, 40.0, 80.0]], -116.53213607052128),
    ("t2", [[50.0, 0.0, 0.0], [50.0, 50.0, 0.0], [0.0, 50.0, 50.0]], 32096.48839031735),
]
NAMD_EPS, NAMD_SIG = 0.0441795, 2 * 1.64009


@pytest.mark.parametrize("lcell", [1, 3])
@pytest.mark.parametrize("name,uc,expected", NAMD_CASES)
def test_namd_lj_energies(orc, namd, name, uc, expected, lcell):
    uc = np.asarray(uc, float)
    kind = "ortho" if uc.ndim == 1 else "tri"
    r = orc.run("lj_energy", namd[name].astype(np.float64), kind=kind, unitcell=uc, cutoff=10.0, lcell=lcell,
                params=[NAMD_EPS, NAMD_SIG, 1.0, 2.0])
    assert r["scalar"] == pytest.approx(expected, rel=1e-12)


# test/applications/gromacs/compare_with_gromacs.jl:7-11,47-60: plain cut-off LJ c12/d^12 - c6/d^6 (kJ/mol,
# Angstrom) at rc 8 against the "LJ (SR)" energies GROMACS printed (test/applications/gromacs/argon/*.log),
# which carry 6 significant digits; the reference's own tolerance is rtol 1e-5 for lcell 1, 2 and 3.
GROMACS_CASES = [("minimal", -3.58447e-01), ("cubic", 1.01353e+04), ("dodecahedron", 4.62904e+05),
                 ("octahedron", 1.82849e+04)]
GROMACS_C12, GROMACS_C6 = 9.69576e6, 0.00622127e6


def gromacs_frame(golden_dir, name):
    """Positions and cell of a GROMACS argon frame; (kind, unitcell) as the pair engine takes them."""
    f = np.load(os.path.join(golden_dir, "gromacs_argon.npz"))
    x, cell = f[name + "_x"], f[name + "_cell"]
    if np.count_nonzero(cell - np.diag(np.diag(cell))):
        return x, "tri", cell
    return x, "ortho", np.diag(cell).copy()


@pytest.mark.parametrize("lcell", [1, 2, 3])
@pytest.mark.parametrize("name,expected", GROMACS_CASES)
def test_gromacs_lj_energies(orc, golden_dir, name, expected, lcell):
    x, kind, uc = gromacs_frame(golden_dir, name)
    r = orc.run("lj_energy", x, kind=kind, unitcell=uc, cutoff=8.0, lcell=lcell,
                params=[1.0, 1.0, GROMACS_C12, GROMACS_C6])
    assert r["scalar"] == pytest.approx(expected, rel=1e-5)


def test_small_exact_cases(orc):
    # test/API/neighborlists.jl:183-193
    def nl(x, **kw):
        x = np.asarray(x, float)
        r = orc.run("nl", x, dim=x.shape[1], **kw)
        return list(zip(r["i"], r["j"], r["d"]))

    assert nl([[0.0, 0.0, 1.0], [0.0, 0.0, 10.0], [0.0, 0.0, 7.0]], kind="nonperiodic", cutoff=2.0) == []
    assert nl([[0.0, 1.0], [0.0, 10.0]], kind="nonperiodic", cutoff=2.0) == []
    side = 2.0 + np.nextafter(1.0, 2.0)
    assert nl([[0.0, 0.0]], unitcell=[side, side], cutoff=1.0) == []
    got = nl([[0.0, 0.0], [0.0, 1.0]], unitcell=[side, side], cutoff=1.0)
    assert [(min(a, b), max(a, b), d) for a, b, d in got] == [(0, 1, 1.0)]
    assert nl([[0.0, 0.0], [0.0, 1.0]], unitcell=[2.0, 2.0], cutoff=np.nextafter(1.0, 0.0)) == []
    got = nl([[0.0, 0.0], np.array([0.0, 1.0]) + np.nextafter(1.0, 2.0)], unitcell=[2.0, 2.0], cutoff=np.nextafter(1.0, 0.0))
    assert [(min(a, b), max(a, b), d) for a, b, d in got] == [(0, 1, 0.9999999999999998)]


def test_cutoff_ties_unit_square(orc):
    # test/API/neighborlists.jl:244-266
    for x in [np.nextafter(0.1, 1.0), np.nextafter(0.9, 0.0)]:
        r = orc.run("nl", np.array([[0.0, 0.0], [x, 0.0]]), dim=2, unitcell=[1.0, 1.0], cutoff=0.1)
        assert len(r["i"]) == 0
    for x in [-0.1, 0.1, 0.9]:
        r = orc.run("nl", np.array([[0.0, 0.0], [x, 0.0]]), dim=2, unitcell=[1.0, 1.0], cutoff=0.1)
        assert len(r["i"]) == 1


def test_computing_box(orc):
    # test/API/ParticleSystem.jl:228-234: unit cube, cutoff 0.1 -> computing box (-0.1, 1.1)
    b = orc.box_info(unitcell=[1.0, 1.0, 1.0], cutoff=0.1)
    np.testing.assert_allclose(b["computing_box"][0], [-0.1] * 3, atol=1e-15)
    np.testing.assert_allclose(b["computing_box"][1], [1.1] * 3, atol=1e-15)


def test_box_docstring_examples(orc):
    # jldoctests of src/internals/Box.jl:159-188 and 320-327
    assert list(orc.box_info(unitcell=[[100, 50, 0], [0, 120, 0], [0, 0, 130]], kind="tri", cutoff=10.0)["nc"]) == [20, 13, 16]
    assert list(orc.box_info(unitcell=[100, 120, 150], cutoff=10.0)["nc"]) == [13, 15, 18]
    assert list(orc.box_info(unitcell=[120, 150, 100], cutoff=10.0)["nc"]) == [15, 18, 13]


def test_align_cell_and_cell_limits(orc):
    # test/internals/CellOperations.jl:109-190: align_cell of 2D cells and cell_limits of aligned cells.
    # box_info gives the aligned cell, the rotation and the computing box, which is cell_limits widened by
    # lcell cells on each side.
    l = np.sqrt(2) / 2
    for m, mt, R in [([[l, 0], [l, 1]], [[1, l], [0, l]], [[l, l], [-l, l]]),
                     ([[-l, 0], [l, 1]], [[1, l], [0, -l]], [[-l, l], [-l, -l]])]:
        b = orc.box_info(dim=2, kind="tri", unitcell=m, cutoff=0.05)
        np.testing.assert_allclose(b["aligned_unit_cell"], mt, atol=1e-12)
        np.testing.assert_allclose(b["rotation"], R, atol=1e-12)
    for m, lo, hi in [([[10, 5], [5, 10]], [0.0, 0.0], [20.12461179749811, 6.708203932499369]),
                      ([[10, 5], [0, 10]], [0.0, -8.94427190999916], [15.652475842498529, 0.0]),
                      ([[1, 0, 0], [0, 2, 0], [0, 0, 1]], [0.0, -1.0, 0.0], [2.0, 0.0, 1.0]),
                      ([[1, 0, 0], [0, 2, 0], [0, 0, 3]], [0.0, 0.0, -1.0], [3.0, 2.0, 0.0])]:
        b = orc.box_info(dim=len(lo), kind="tri", unitcell=m, cutoff=0.1)
        h = b["cell_size"]
        np.testing.assert_allclose(b["computing_box"][0] + h, lo, atol=1e-10)
        np.testing.assert_allclose(b["computing_box"][1] - h, hi, atol=1e-10)
    # a rotated diag(3, 2, 1): the longest vector goes back onto x, the other two into the y-z plane
    rng = np.random.default_rng(5)
    for _ in range(5):
        q, r = np.linalg.qr(rng.normal(size=(3, 3)))
        R = q * np.sign(np.diag(r))
        if np.linalg.det(R) < 0:  # a proper rotation
            R[:, 0] = -R[:, 0]
        b = orc.box_info(dim=3, kind="tri", unitcell=R @ np.diag([3.0, 2.0, 1.0]), cutoff=0.1)
        ma = b["aligned_unit_cell"]
        np.testing.assert_allclose(ma[:, 0], [3.0, 0.0, 0.0], atol=1e-12)
        np.testing.assert_allclose(np.cross([1.0, 0.0, 0.0], np.cross(ma[:, 1], ma[:, 2])), 0.0, atol=1e-10)


def test_cell_too_small_and_lcell(orc):
    # src/internals/Box.jl:192, 243
    with pytest.raises(orc.OracleError) as e:
        orc.box_info(unitcell=[10.0, 10.0, 10.0], cutoff=5.0)
    assert e.value.code == 2
    with pytest.raises(orc.OracleError) as e:
        orc.box_info(unitcell=[10.0, 10.0, 10.0], cutoff=1.0, lcell=0)
    assert e.value.code == 10


def test_nan_coordinates(orc):
    # src/internals/CellOperations.jl:6-21
    x = np.random.default_rng(0).random((10, 3))
    x[3, 1] = np.nan
    with pytest.raises(orc.OracleError) as e:
        orc.run("count", x, unitcell=[1.0, 1.0, 1.0], cutoff=0.1)
    assert e.value.code == 3


CASES = [
    # (dim, kind, unitcell, cutoff, lcell, n)
    (3, "ortho", [10.0, 12.0, 11.0], 1.5, 1, 800),
    (3, "ortho", [10.0, 12.0, 11.0], 1.5, 2, 800),
    (3, "tri", [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]], 1.5, 1, 800),
    (3, "tri", [[10.0, 2.0, 1.0], [0.0, 11.0, 1.5], [0.0, 0.0, 12.0]], 1.5, 3, 600),
    (3, "nonperiodic", None, 1.5, 1, 800),
    (2, "ortho", [10.0, 12.0], 1.2, 1, 600),
    (2, "tri", [[10.0, 3.0], [0.0, 11.0]], 1.2, 2, 600),
    (2, "nonperiodic", None, 1.2, 1, 600),
]


@pytest.mark.parametrize("cross", [False, True])
@pytest.mark.parametrize("dim,kind,uc,cut,lcell,n", CASES)
def test_celllist_matches_naive(orc, dim, kind, uc, cut, lcell, n, cross):
    """The cell-list restatement finds the same pairs as the naive minimum-image loop
    (the reference's own correctness strategy, test/internals/tests.jl:181-299)."""
    rng = np.random.default_rng(dim * 100 + lcell + (7 if cross else 0))
    span = 12.0
    x = rng.random((n, dim)) * span - 1.0
    y = rng.random((n // 2, dim)) * span - 1.0 if cross else None
    kw = dict(dim=dim, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell)
    cl = orc.run("nl", x, y, **kw)
    nv = orc.run("nl", x, y, naive=True, **kw)
    if cross:
        a = np.lexsort((cl["j"], cl["i"]))
        b = np.lexsort((nv["j"], nv["i"]))
        np.testing.assert_array_equal(cl["i"][a], nv["i"][b])
        np.testing.assert_array_equal(cl["j"][a], nv["j"][b])
        np.testing.assert_allclose(cl["d"][a], nv["d"][b], rtol=1e-12)
    else:
        A = orc.canonical_pairs(cl["i"], cl["j"], cl["d"])
        B = orc.canonical_pairs(nv["i"], nv["j"], nv["d"])
        np.testing.assert_array_equal(A[0], B[0])
        np.testing.assert_array_equal(A[1], B[1])
        np.testing.assert_allclose(A[2], B[2], rtol=1e-12)
    e1 = orc.run("soft_forces", x, y, **kw)
    e2 = orc.run("soft_forces", x, y, naive=True, **kw)
    assert e1["scalar"] == pytest.approx(e2["scalar"], rel=1e-12)
    np.testing.assert_allclose(e1["forces_x"], e2["forces_x"], atol=1e-11 * max(1.0, np.abs(e2["forces_x"]).max()))


def _pathological(rng, n, sides):
    """test/modules/Testing.jl:36-60: points on faces, +-nextfloat(0), outside the box."""
    x = sides * rng.random((n, 3))
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
    return x


def test_pathological_coordinates(orc):
    """test/modules/Testing.jl:36-60: points on faces, +-nextfloat(0), outside the box."""
    rng = np.random.default_rng(5)
    sides = np.array([250.0, 250.0, 250.0])
    x = _pathological(rng, 200, sides)
    for lcell in (1, 2):
        cl = orc.run("count", x, unitcell=sides, cutoff=10.0, lcell=lcell)
        nv = orc.run("count", x, unitcell=sides, cutoff=10.0, naive=True)
        assert cl["count"] == nv["count"]


def _gravity_brute_force(x, side, cutoff, m, c=9.8):
    """test/examples/gravitational_potential.jl:30-33 and gravitational_force.jl:37-46 written out over
    all pairs with the minimum image in a cubic box."""
    n = len(x)
    u = 0.0
    f = np.zeros_like(x)
    for i in range(n - 1):
        dx = x[i] - x[i + 1:]
        dx -= side * np.rint(dx / side)
        d2 = np.sum(dx * dx, axis=1)
        sel = np.nonzero(d2 <= cutoff * cutoff)[0]
        for k in sel:
            j = i + 1 + k
            d = np.sqrt(d2[k])
            u -= c * m[i] * m[j] / d
            df = (c * m[i] * m[j] / d2[k] / d) * dx[k]
            f[i] -= df
            f[j] += df
    return u, f


@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_weighted_inverse_distance(orc, kind):
    # the gravitational examples' closures, with masses m = 5 x_1 as in the reference's examples
    rng = np.random.default_rng(21)
    side = 60.0
    x = rng.random((1500, 3)) * side
    m = 5 * x[:, 0]
    uc = [side] * 3 if kind == "ortho" else np.diag([side] * 3)
    r = orc.run("weighted_inv_d", x, kind=kind, unitcell=uc, cutoff=10.0, params=[9.8], weights_x=m)
    rn = orc.run("weighted_inv_d", x, kind=kind, unitcell=uc, cutoff=10.0, params=[9.8], weights_x=m, naive=True)
    assert r["scalar"] == pytest.approx(rn["scalar"], rel=1e-12)
    np.testing.assert_allclose(r["forces_x"], rn["forces_x"], rtol=0, atol=1e-12 * np.abs(rn["forces_x"]).max())
    u, f = _gravity_brute_force(x, side, 10.0, m)
    assert r["scalar"] == pytest.approx(u, rel=1e-12)
    np.testing.assert_allclose(r["forces_x"], f, rtol=0, atol=1e-12 * np.abs(f).max())
    # two sets: weights of y apply to the partner
    y = rng.random((700, 3)) * side
    my = 5 * y[:, 0]
    rc = orc.run("weighted_inv_d", x, y, kind=kind, unitcell=uc, cutoff=10.0, params=[9.8], weights_x=m,
                 weights_y=my)
    rcn = orc.run("weighted_inv_d", x, y, kind=kind, unitcell=uc, cutoff=10.0, params=[9.8], weights_x=m,
                  weights_y=my, naive=True)
    assert rc["scalar"] == pytest.approx(rcn["scalar"], rel=1e-12)
    np.testing.assert_allclose(rc["forces_y"], rcn["forces_y"], rtol=0, atol=1e-12 * np.abs(rcn["forces_y"]).max())


@pytest.mark.parametrize("dim", [2, 3])
def test_neighborlists_vs_kdtree(orc, dim):
    # test/API/neighborlists.jl:1-45: non-periodic self and cross lists against a tree-based search
    # (NearestNeighbors.jl there, scipy's cKDTree here), for two cutoffs
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(40 + dim)
    for n, m, r in [(500, 1000, 0.1), (450, 831, 0.05)]:
        x = rng.random((n, dim))
        y = rng.random((m, dim))
        got = orc.run("nl", x, dim=dim, kind="nonperiodic", cutoff=r)
        a, b = np.minimum(got["i"], got["j"]), np.maximum(got["i"], got["j"])
        assert len(set(zip(a.tolist(), b.tolist()))) == len(a)  # each pair once
        ref = spatial.cKDTree(x).query_pairs(r, output_type="ndarray")
        assert set(zip(a.tolist(), b.tolist())) == set(map(tuple, ref.tolist()))
        np.testing.assert_allclose(got["d"], np.linalg.norm(x[got["i"]] - x[got["j"]], axis=1), rtol=1e-12)
        got = orc.run("nl", x, y, dim=dim, kind="nonperiodic", cutoff=r)
        pairs = set(zip(got["i"].tolist(), got["j"].tolist()))
        assert len(pairs) == len(got["i"])
        sm = spatial.cKDTree(x).sparse_distance_matrix(spatial.cKDTree(y), r, output_type="ndarray")
        assert pairs == set(zip(sm["i"].tolist(), sm["j"].tolist()))


def test_images_counted_once(orc):
    # test/internals/tests.jl:490-593: pairs through the periodic boundary, triclinic wrapping and a dense
    # cluster at the boundaries, each pair counted once (cell lists against the naive loop)
    x = np.array([[0.5, 5.0, 5.0], [9.6, 5.0, 5.0]])
    assert orc.run("count", x, unitcell=[10.0] * 3, cutoff=2.0)["count"] == 1
    uc = np.array([[10.0, 3.0, 0.0], [0.0, 10.0, 2.0], [0.0, 0.0, 10.0]])
    x = np.array([[0.5, 0.5, 0.5], [2.0, 1.0, 1.0], [9.5, 9.5, 9.5], [8.5, 9.0, 9.0]])
    kw = dict(kind="tri", unitcell=uc, cutoff=2.5)
    assert orc.run("count", x, **kw)["count"] == orc.run("count", x, naive=True, **kw)["count"]
    g = np.array([[0.3 * i, 0.3 * j, 0.3 * k] for i in range(1, 6) for j in range(1, 6) for k in range(1, 6)])
    x = np.concatenate([g, 15.0 - g])
    kw = dict(unitcell=[15.0] * 3, cutoff=2.5)
    n = orc.run("count", x, **kw)["count"]
    assert n == orc.run("count", x, naive=True, **kw)["count"]
    nl = orc.run("nl", x, **kw)
    a, b = np.minimum(nl["i"], nl["j"]), np.maximum(nl["i"], nl["j"])
    assert len(set(zip(a.tolist(), b.tolist()))) == len(a) == n


def test_margins_with_large_lcell(orc):
    # test/internals/tests.jl:595-684: particles at cell corners with lcell up to 5, triclinic cells with
    # lcell up to 3, and pairs just inside the cutoff across cell boundaries
    rng = np.random.default_rng(55)
    for lcell in [1, 2, 3, 5]:
        sides = np.array([20.0] * 3)
        x = list(rng.random((200, 3)) * sides)
        cs = sides / (2 * lcell + 1)
        for i in range(1, lcell + 2):
            for j in range(1, lcell + 2):
                for k in range(1, lcell + 2):
                    c = np.array([cs[0] * i + 0.1, cs[1] * j + 0.1, cs[2] * k + 0.1])
                    if np.all(c < sides):
                        x.append(c)
        x = np.array(x)
        kw = dict(unitcell=list(sides), cutoff=2.5, lcell=lcell)
        assert orc.run("sum_d", x, **kw)["scalar"] == pytest.approx(orc.run("sum_d", x, naive=True, **kw)["scalar"],
                                                                    rel=1e-10)
    uc = np.array([[15.0, 5.0, 0.0], [0.0, 15.0, 3.0], [0.0, 0.0, 15.0]])
    for lcell in [1, 2, 3]:
        x = rng.random((150, 3)) @ uc.T
        kw = dict(kind="tri", unitcell=uc, cutoff=2.0, lcell=lcell)
        assert orc.run("sum_d", x, **kw)["scalar"] == pytest.approx(orc.run("sum_d", x, naive=True, **kw)["scalar"],
                                                                    rel=1e-10)
    c = 3.0 - 0.001
    x = np.array([[5.0, 5.0, 5.0], [5.0 + c, 5.0, 5.0], [10.0, 10.0, 10.0], [10.0, 10.0 + c, 10.0],
                  [15.0, 15.0, 15.0], [15.0, 15.0, 15.0 + c]])
    kw = dict(unitcell=[30.0] * 3, cutoff=3.0, lcell=3)
    n = orc.run("count", x, **kw)["count"]
    assert n == orc.run("count", x, naive=True, **kw)["count"] and n >= 3


def test_disjoint_sets_gravitational_potential(orc):
    # test/internals/tests.jl:1-33: the gravitational potential between two pathological sets (masses
    # indexed by each set's own index), lcell 1 and 3, against the naive loop
    rng = np.random.default_rng(6)
    sides = np.array([250.0, 250.0, 250.0])
    x = _pathological(rng, 2000, sides)
    y = _pathological(rng, 2000, sides) + 0.25  # no point of y on a point of x (1/d finite)
    mass = rng.random(2000)
    kw = dict(unitcell=sides, cutoff=10.0, params=[9.8], weights_x=mass, weights_y=mass)
    naive = orc.run("weighted_inv_d", x, y, naive=True, **kw)["scalar"]
    for lcell in (1, 3):
        assert orc.run("weighted_inv_d", x, y, lcell=lcell, **kw)["scalar"] == pytest.approx(naive, rel=1e-12)


def test_pathological_2d_cells(orc):
    # test/modules/Testing.jl:563-599 (test_pathological2D, test/internals/tests.jl:700-702): two random
    # points in 11 awkward 2D cells (sheared, rotated, negative determinant) for lcell 1..5, cell lists
    # against the naive loop
    l = np.sqrt(2) / 2
    mats = [[[1, 0], [0, 1]], [[l, 0], [l, 1]], [[1.1, 0], [0, 1]], [[1.2, 0], [0, 1]], [[1, 0], [0, 1.1]],
            [[1, 0], [0, 1.2]], [[1, 0.2], [0, 1.2]], [[1, 0.2], [0.2, 1.2]], [[1.2, 0.2], [0.2, 1.2]],
            [[-1.2, 0.2], [0.2, 1.2]], [[-1.2, 0.2], [0.2, -1.2]]]
    rng = np.random.default_rng(7)
    for _ in range(200):
        for M in mats:
            for lcell in range(1, 6):
                x = rng.random((2, 2))
                kw = dict(dim=2, kind="tri", unitcell=M, cutoff=0.2, lcell=lcell)
                assert orc.run("count", x, **kw)["count"] == orc.run("count", x, naive=True, **kw)["count"], (M, lcell, x)


@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_random_cells_sweep(orc, kind):
    # test/modules/Testing.jl:162-257 (test_random_cells, test/internals/tests.jl:686-698): random cells with
    # entries in [-10, 10] (orthorhombic: the diagonal), cutoff in [1, 2], lcell 1..3, kept when they pass the
    # unit-cell check; 10-20 points far outside the cell (wrapped in); cell lists against the naive loop
    rng = np.random.default_rng(3 if kind == "ortho" else 4)
    for dim in (2, 3):
        for lcell in (1, 2, 3):
            done = trials = 0
            while done < 40 and trials < 3000:
                trials += 1
                M = np.diag(-10 + 20 * rng.random(dim)) if kind == "ortho" else -10 + 20 * rng.random((dim, dim))
                uc = np.diag(M) if kind == "ortho" else M
                cut = 1 + rng.random()
                try:
                    b = orc.box_info(dim=dim, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell)
                except orc.OracleError as e:
                    assert e.code == 2  # only the unit-cell check may refuse a cell
                    continue
                if np.prod(b["nc"]) > 100000:
                    continue
                x = 10 * rng.random((int(rng.integers(10, 21)), dim)) - 50
                kw = dict(dim=dim, kind=kind, unitcell=uc, cutoff=cut, lcell=lcell)
                assert orc.run("count", x, **kw)["count"] == orc.run("count", x, naive=True, **kw)["count"]
                assert orc.run("sum_d2", x, **kw)["scalar"] == pytest.approx(
                    orc.run("sum_d2", x, naive=True, **kw)["scalar"], rel=1e-10, abs=1e-10)
                done += 1
            assert done == 40
