"""GPU parity at the full sizes of the benchmark workloads, kept after every other GPU suite.

The other GPU tests compare with the oracle on inputs it finishes in milliseconds.  These run the workloads
the bench measures, at their full sizes, and check them against the oracle where it finishes in seconds on
the host's cores:
  * the headline: 1,048,576 Float32 particles (jittered fcc, triclinic cell), LJ energy and forces, the pair
    count and the cell list copy by copy;
  * 100,000 uniform Float64 points, cutoff 8: the neighbour list bit-exact (10.7M pairs), soft energy and
    forces;
  * the 200,000-particle two-type LJ mixture: energy, forces and the adjoint (virial, dU/dM, dU/deps,
    dU/dsigma);
  * the 4096 batched systems (14.2M particles): every system's status, and counts and energies of a
    sample of systems;
  * the two-set radial histogram, 3D and 2D, on a subsample of x against all 2M points of y.
and through size-independent properties at full size: Newton's third law on the forces (sum of F ~ 0),
equal counts across operators and precision forms, histogram counts equal between the exact and FP32-split
forms, the dropped pairs (r <= first edge) accounted for.  Last, a split-form histogram with edges finer than
the split form's FP32 distance error, which the library runs in the exact form: its counts equal the
oracle's for pairs planted within 1e-9 of the edges.

Bars as in the other suites: counts and sets exact; Float64 values within 1e-12 and Float32 (or split)
values within 1e-5 of the stated scale.  Each check compares plain numpy results (`check_*`), so the same
functions compare the oracle with itself on the CPU.
"""
import os

import numpy as np
import pytest

from tests.test_adjoint import C12, C6, CUT, cls_index, pair_terms
from tests.test_gpu_parity import assert_same_pairs

pytestmark = pytest.mark.gpu

NT = max(1, os.cpu_count() or 1)  # oracle threads: all host cores
LJ = [1.0, 1.0, 4.0, 4.0]


def newton_residual(f):
    """|sum of the forces| relative to the sum of their magnitudes (Newton's third law: ~0)."""
    f = np.asarray(f, np.float64)
    return np.abs(f.sum(0)).max() / max(np.abs(f).sum(), 1e-300)


# ------------------------------------------------------------------ headline: 1M Float32 LJ, triclinic
def check_headline(g, r, tol=1e-5):
    assert g["count"] == r["count"]
    assert abs(g["energy"] - r["energy"]) <= tol * abs(r["energy"])
    fr = np.asarray(r["forces"], np.float64)
    assert np.abs(np.asarray(g["forces"], np.float64) - fr).max() <= tol * np.abs(fr).max()
    assert newton_residual(g["forces"]) <= 1e-6
    for k in ("cell", "index", "coords"):
        np.testing.assert_array_equal(np.asarray(g["celllist"][k], np.float64),
                                      np.asarray(r["celllist"][k], np.float64))


def headline_oracle(orc, x, M):
    kw = dict(kind="tri", unitcell=M, cutoff=2.5, dtype=np.float32)
    f = orc.run("lj_forces", x, params=LJ, nthreads=NT, **kw)
    return {"count": orc.run("count", x, nthreads=NT, **kw)["count"], "energy": f["scalar"],
            "forces": f["forces_x"], "celllist": orc.celllist(x, **kw)}


def test_headline_full_size(clm, orc):
    x, M = clm.workloads.cfg2()  # 1,048,576 Float32 particles
    s = clm.ParticleSystem(xpositions=x, unitcell=M, cutoff=2.5, dtype=np.float32)
    ef = clm.pairwise(clm.LennardJonesForces(*LJ), s)
    g = {"count": clm.pairwise(clm.Count(), s), "energy": ef.energy, "forces": ef.forces,
         "celllist": s.fetch_celllist(0)}
    s.close()
    r = headline_oracle(orc, x, M)
    assert r["count"] == 25_803_334
    check_headline(g, r)


# ------------------------------------------------------------------ 100k Float64 uniform, cutoff 8
def check_nl_f64(orc, g, r):
    assert_same_pairs(orc, g["nl"], r["nl"])  # bit-exact sets and distances
    assert g["count"] == len(r["nl"]["i"])
    assert abs(g["energy"] - r["energy"]) <= 1e-12 * r["energy"]  # every term (8 - d)^2 >= 0
    fr = np.asarray(r["forces"], np.float64)
    assert np.abs(np.asarray(g["forces"]) - fr).max() <= 1e-12 * np.abs(fr).max()
    assert newton_residual(g["forces"]) <= 1e-12


def nl_f64_oracle(orc, x, sides, nthreads=NT):
    kw = dict(kind="ortho", unitcell=sides, cutoff=8.0)
    f = orc.run("soft_forces", x, nthreads=nthreads, **kw)
    return {"nl": orc.run("nl", x, nthreads=nthreads, **kw), "energy": f["scalar"], "forces": f["forces_x"]}


def test_neighbor_list_100k_full_size(clm, orc):
    x, sides = clm.workloads.cfg1()
    s = clm.ParticleSystem(xpositions=x, unitcell=sides, cutoff=8.0)
    nl = clm.pairwise(clm.NeighborList(), s)
    ef = clm.pairwise(clm.SoftForces(), s)
    g = {"nl": nl, "count": clm.pairwise(clm.Count(), s), "energy": ef.energy, "forces": ef.forces}
    s.close()
    check_nl_f64(orc, g, nl_f64_oracle(orc, x, sides))


# ------------------------------------------------------------------ 200k Float32 LJ mixture and its adjoint
def check_adjoint(g, r, p, tol=1e-5):
    assert abs(g["energy"] - r["scalar"]) <= tol * np.abs(p["u"]).sum()
    fr = np.asarray(r["forces_x"], np.float64)
    assert np.abs(np.asarray(g["forces"], np.float64) - fr).max() <= tol * np.abs(fr).max()
    assert newton_residual(g["forces"]) <= 1e-6
    wscale = np.abs(p["g"] * (p["dx"] ** 2).sum(1)).sum()
    assert np.abs(np.asarray(g["virial"]) - r["virial"]).max() <= tol * wscale
    for a in range(2):
        for b in range(2):
            k = cls_index(a, b)
            m = p["cls"] == k
            assert abs(g["deps"][a, b] - r["deps"][k]) <= tol * np.abs(p["u_over_eps"][m]).sum()
            assert abs(g["dsig"][a, b] - r["dsig"][k]) <= tol * np.abs(p["du_dsig"][m]).sum()


def adjoint_oracle(orc, x, L, t, eps, sig, nthreads=NT):
    return orc.run("lj_adjoint", x, dim=3, kind="ortho", unitcell=[L] * 3, cutoff=CUT, lcell=1, dtype=np.float32,
                   params=[1.0, 1.0, C12, C6], types_x=t, eps_table=eps, sig_table=sig, nthreads=nthreads)


def test_mixture_adjoint_full_size(clm, orc):
    x, L, t, eps, sig = clm.workloads.cfg4()  # 200,000 Float32 particles, 80:20 types
    op = clm.LennardJonesAdjoint(c12=C12, c6=C6, types_x=t, eps_table=eps, sig_table=sig)
    s = clm.ParticleSystem(positions=x, unitcell=[L] * 3, cutoff=CUT, dtype=np.float32)
    a = clm.pairwise(op, s)
    s.close()
    g = {"energy": a.energy, "forces": a.forces, "virial": a.virial, "deps": a.dU_deps, "dsig": a.dU_dsigma}
    r = adjoint_oracle(orc, x, L, t, eps, sig)
    check_adjoint(g, r, pair_terms(orc, x, np.diag([L] * 3), t, eps, sig, "ortho", dtype=np.float32))


# ------------------------------------------------------------------ 4096 batched Float64 systems
RC3 = 6.0


def batch_sample(sides, k=48):
    """A deterministic sample of the systems the reference accepts (side > 2 cutoff): evenly spaced by
    index, plus the largest."""
    valid = np.flatnonzero(sides > 2 * RC3)
    pick = valid[np.linspace(0, len(valid) - 1, k).astype(np.int64)]
    return np.unique(np.concatenate([pick, [valid[np.argmax(sides[valid])]]]))


def check_batch_full(g, r, sides):
    valid = sides > 2 * RC3  # the reference's unit-cell check for a cube (Box.jl:243)
    assert np.all(g["status"][~valid] == 2) and np.all(g["status"][valid] == 0)
    assert np.all(np.isnan(g["energy"][~valid])) and np.all(np.isfinite(g["energy"][valid]))
    for s, (cnt, e) in r.items():
        assert g["count"][s] == cnt, s
        assert abs(g["energy"][s] - e) <= 1e-12 * e, s  # soft energy: every term >= 0


def batch_oracle(orc, x, off, sides, systems):
    out = {}
    for s in systems:
        xs = x[off[s]:off[s + 1]]
        kw = dict(kind="ortho", unitcell=[sides[s]] * 3, cutoff=RC3, nthreads=NT)
        out[int(s)] = (orc.run("count", xs, **kw)["count"], orc.run("soft_energy", xs, params=[RC3], **kw)["scalar"])
    return out


def test_batched_systems_full_size(clm, orc):
    x, off, sides = clm.workloads.cfg3()  # 4096 systems, 14.2M particles
    bs = clm.BatchedSystems(positions=x, offsets=off, unitcells=np.repeat(sides[:, None], 3, axis=1), cutoff=RC3)
    cnt, en = bs.run(clm.Count(), clm.SoftEnergy())
    g = {"count": cnt, "energy": en, "status": bs.status()}
    bs.close()
    check_batch_full(g, batch_oracle(orc, x, off, sides, batch_sample(sides)), sides)


# ------------------------------------------------------------------ two sets of 2M points, radial histogram
def hist_bound(counts, vx, vy):
    """Per-bin bound on the sum of |dot(v_i - v_j, x - y)/r| <= |v_i - v_j|: count x max |v_i - v_j|."""
    vmax = np.linalg.norm(vx, axis=1).max() + np.linalg.norm(vy, axis=1).max()
    return counts * vmax


def check_hist_subsample(g, r, vx, vy):
    np.testing.assert_array_equal(g["count"], r["hist_count"])
    assert np.all(np.abs(g["sum"] - r["hist_sum"]) <= 1e-10 * hist_bound(r["hist_count"], vx, vy) + 1e-9)


def check_hist_forms(g, vx, vy):
    # the split form re-decides bins near their edges exactly: same counts; sums within 1e-5 of the bound
    np.testing.assert_array_equal(g["exact"][0], g["split"][0])
    assert np.all(np.abs(g["exact"][1] - g["split"][1]) <= 1e-5 * hist_bound(g["exact"][0], vx, vy) + 1e-9)
    # pairs within the cutoff: the same in both forms; those not binned are the pairs with r <= the first
    # edge, counted independently by a periodic k-d tree
    assert g["count_exact"] == g["count_split"]
    assert g["count_exact"] - int(g["exact"][0].sum()) == g["below_first_edge"]


@pytest.mark.parametrize("dim", [3, 2])
def test_histogram_two_sets_full_size(clm, orc, dim):
    # 2 x 2,000,000 Float64 points, side 250, cutoff 25 (3D: 1.7e10 pairs in bins; 2D: 1.3e11)
    x, y, vx, vy, sides = clm.workloads.cfg5(dim=dim)
    bins = clm.workloads.cfg5_bins()
    g = {}
    s = clm.ParticleSystem(xpositions=x, ypositions=y, unitcell=sides, cutoff=25.0)
    g["exact"] = clm.pairwise(clm.RadialHistogram(bins, vx, vy), s)
    g["count_exact"] = clm.pairwise(clm.Count(), s)
    s.set_precision("split")
    g["split"] = clm.pairwise(clm.RadialHistogram(bins, vx, vy), s)
    g["count_split"] = clm.pairwise(clm.Count(), s)
    s.close()
    # pairs with r <= 0.1 (3D: 1108 here, 4e12 (4/3 pi 0.1^3) / 250^3 ~ 1072 expected for uniform points;
    # 2D: ~ 4e12 pi 0.1^2 / 250^2 ~ 2.0e6)
    kd = pytest.importorskip("scipy.spatial")
    g["below_first_edge"] = int(kd.cKDTree(x, boxsize=sides[0]).count_neighbors(kd.cKDTree(y, boxsize=sides[0]),
                                                                                bins[0]))
    check_hist_forms(g, vx, vy)
    # a subsample of x against every point of y, against the oracle
    xs, vxs = x[:2000], vx[:2000]
    s = clm.ParticleSystem(xpositions=xs, ypositions=y, unitcell=sides, cutoff=25.0)
    hc, hs = clm.pairwise(clm.RadialHistogram(bins, vxs, vy), s)
    s.close()
    r = orc.run("rhist", xs, y, dim=dim, unitcell=sides, cutoff=25.0, bins=bins, vel_x=vxs, vel_y=vy, nthreads=NT)
    check_hist_subsample({"count": hc, "sum": hs}, r, vxs, vy)


# ------------------------------------------------------------------ split-form histogram with fine edges
def fine_edge_points(rng, edges, per_edge=40, side=20.0):
    """Pairs of points planted at distances within 1e-9 (relative) of the given edges, on both sides, in
    random directions, plus a uniform background."""
    pts = [rng.random((2000, 3)) * side]
    for e in edges:
        for sgn in (-1.0, 1.0):
            p = rng.random((per_edge, 3)) * side
            u = rng.normal(size=(per_edge, 3))
            u /= np.linalg.norm(u, axis=1)[:, None]
            pts += [p, p + u * e * (1.0 + sgn * 1e-9)]
    return np.concatenate(pts)


def check_hist_exact_counts(hc, r, dropped_gpu, dropped_ref):
    np.testing.assert_array_equal(hc, r["hist_count"])
    assert dropped_gpu == dropped_ref


def test_split_histogram_fine_edges(clm, orc):
    # edges finer than the split form's FP32 distance error (1e-4, 1e-3 with cell side 2): the library runs
    # such histograms in the exact form, so the counts equal the oracle's even for pairs within 1e-9 of an
    # edge, and the pairs at or below the first edge are dropped as in the reference
    rng = np.random.default_rng(17)
    edges = [1e-4, 1e-3, 1e-2]
    x = fine_edge_points(rng, edges)
    v = rng.normal(0.0, 1.0, x.shape)
    bins = np.array(edges + [0.1, 0.5, 1.0, 2.0])
    s = clm.ParticleSystem(xpositions=x, unitcell=[20.0] * 3, cutoff=2.0, precision="split")
    hc, hs = clm.pairwise(clm.RadialHistogram(bins, v), s)
    n_gpu = clm.pairwise(clm.Count(), s)
    s.close()
    r = orc.run("rhist", x, unitcell=[20.0] * 3, cutoff=2.0, bins=bins, vel_x=v, nthreads=NT)
    n_ref = orc.run("count", x, unitcell=[20.0] * 3, cutoff=2.0, nthreads=NT)["count"]
    check_hist_exact_counts(hc, r, n_gpu - int(hc.sum()), n_ref - int(r["hist_count"].sum()))
