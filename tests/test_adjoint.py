"""The adjoint form: LJ energy, forces and dU/d(cell, eps, sigma) of a two-type LJ mixture.

The reference obtains these gradients by running its map with ForwardDiff dual numbers
(test/examples/generic_types.jl:10-20,102); here they are built-in outputs of one pass.

CPU: the oracle's adjoint against central finite differences of its own energy (rel 1e-6) and against
a numpy restatement from its neighbour list (rel 1e-12).
GPU: the CUDA path against the oracle.  Bar: Float64 rel 1e-12, Float32 rel 1e-5, each relative to
the sum of absolute pair contributions of that quantity (computed from the oracle's neighbour list); and the
GPU adjoint against central finite differences of the GPU's own energy (rel 1e-6).
"""
import numpy as np
import pytest

CUT = 2.5
C12 = C6 = 4.0


def mixture(clm, n=2000, seed=4):
    x, L, t, eps, sig = clm.workloads.cfg4(n=n, seed=seed)
    return x.astype(np.float64), L, t, eps, sig


def tri_cell(L):
    return np.array([[L, 0.2 * L, 0.1 * L], [0.0, L, 0.15 * L], [0.0, 0.0, L]])


def orc_adj(orc, x, M, t, eps, sig, dtype=np.float64, kind=None):
    kind = kind or ("ortho" if np.allclose(M, np.diag(np.diag(M))) else "tri")
    uc = np.diag(M) if kind == "ortho" else M
    return orc.run("lj_adjoint", x, dim=3, kind=kind, unitcell=uc, cutoff=CUT, lcell=1, dtype=dtype,
                   params=[1.0, 1.0, C12, C6], types_x=t, eps_table=eps, sig_table=sig)


def energy(orc, x, M, t, eps, sig, kind=None):
    return orc_adj(orc, x, M, t, eps, sig, kind=kind)["scalar"]


def cls_index(a, b, nt=2):
    a, b = min(a, b), max(a, b)
    return a * nt - a * (a - 1) // 2 + (b - a)


@pytest.mark.parametrize("cell", ["cubic", "triclinic"])
def test_oracle_adjoint_finite_differences(orc, clm, cell):
    x, L, t, eps, sig = mixture(clm, n=1500 if cell == "cubic" else 1200)
    M = np.diag([L] * 3) if cell == "cubic" else tri_cell(L)
    kind = "ortho" if cell == "cubic" else "tri"
    if cell == "triclinic":
        x = x @ np.linalg.inv(np.diag([L] * 3)).T @ M.T  # same fractional coordinates in the triclinic cell
    r = orc_adj(orc, x, M, t, eps, sig, kind=kind)
    h = 1e-6
    for a in range(2):
        for b in range(a, 2):
            k = cls_index(a, b)
            for table, key in ((eps, "deps"), (sig, "dsig")):
                tp, tm = table.copy(), table.copy()
                tp[a, b] += h
                tp[b, a] = tp[a, b]
                tm[a, b] -= h
                tm[b, a] = tm[a, b]
                args_p = (tp, sig) if key == "deps" else (eps, tp)
                args_m = (tm, sig) if key == "deps" else (eps, tm)
                fd = (energy(orc, x, M, t, *args_p, kind=kind) - energy(orc, x, M, t, *args_m, kind=kind)) / (2 * h)
                assert abs(r[key][k] - fd) <= 1e-6 * max(1.0, abs(fd)), (key, a, b, r[key][k], fd)
    # cell: positions follow the cell (scaled coordinates fixed), dU/dM = W M^-T
    W = r["virial"]
    dM = W @ np.linalg.inv(M).T
    Minv = np.linalg.inv(M)
    entries = [(0, 0), (1, 1), (2, 2)] if cell == "cubic" else [(0, 0), (0, 1), (1, 2), (2, 2), (0, 2)]
    for a, b in entries:
        E = np.zeros((3, 3))
        E[a, b] = h
        up = energy(orc, x @ ((M + E) @ Minv).T, M + E, t, eps, sig, kind=kind)
        um = energy(orc, x @ ((M - E) @ Minv).T, M - E, t, eps, sig, kind=kind)
        fd = (up - um) / (2 * h)
        assert abs(dM[a, b] - fd) <= 1e-6 * max(1.0, abs(fd)), (a, b, dM[a, b], fd)
    if cell == "cubic":
        up = energy(orc, x * (L + h) / L, np.diag([L + h] * 3), t, eps, sig, kind=kind)
        um = energy(orc, x * (L - h) / L, np.diag([L - h] * 3), t, eps, sig, kind=kind)
        fd = (up - um) / (2 * h)
        assert abs(np.trace(W) / L - fd) <= 1e-6 * abs(fd)
    # positions: forces = -dU/dx
    for i in (0, 7, len(x) - 3):
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[i, c] += h
            xm[i, c] -= h
            fd = (energy(orc, xp, M, t, eps, sig, kind=kind) - energy(orc, xm, M, t, eps, sig, kind=kind)) / (2 * h)
            assert abs(-r["forces_x"][i, c] - fd) <= 1e-5 * max(1.0, abs(fd)), (i, c, r["forces_x"][i, c], fd)


def pair_terms(orc, x, M, t, eps, sig, kind, dtype=np.float64):
    """numpy restatement of the adjoint from the oracle's neighbour list (minimum-image vectors)."""
    uc = np.diag(M) if kind == "ortho" else M
    nl = orc.run("nl", x, dim=3, kind=kind, unitcell=uc, cutoff=CUT, lcell=1, dtype=dtype)
    i, j = nl["i"], nl["j"]
    xd = np.asarray(x, np.float64)
    dx = xd[j] - xd[i]
    s = dx @ np.linalg.inv(M).T
    dx = (s - np.round(s)) @ M.T
    d2 = (dx * dx).sum(1)
    ti, tj = t[i], t[j]
    e, sg = eps[ti, tj], sig[ti, tj]
    sr6 = (sg * sg / d2) ** 3
    sr12 = sr6 * sr6
    g = e * (-12 * C12 * sr12 + 6 * C6 * sr6) / d2
    cls = np.where(ti <= tj, ti * 2 - ti * (ti - 1) // 2 + (tj - ti), tj * 2 - tj * (tj - 1) // 2 + (ti - tj))
    return dict(g=g, dx=dx, u_over_eps=C12 * sr12 - C6 * sr6, du_dsig=e * (12 * C12 * sr12 - 6 * C6 * sr6) / sg,
                cls=cls, u=e * (C12 * sr12 - C6 * sr6))


@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_oracle_adjoint_vs_numpy(orc, clm, kind):
    x, L, t, eps, sig = mixture(clm, n=3000)
    M = np.diag([L] * 3) if kind == "ortho" else tri_cell(L)
    if kind == "tri":
        x = x / L @ M.T
    r = orc_adj(orc, x, M, t, eps, sig, kind=kind)
    p = pair_terms(orc, x, M, t, eps, sig, kind)
    W = np.einsum("p,pa,pb->ab", p["g"], p["dx"], p["dx"])
    np.testing.assert_allclose(r["virial"], W, rtol=1e-11, atol=1e-11 * np.abs(p["g"] * (p["dx"] ** 2).sum(1)).sum())
    np.testing.assert_allclose(r["scalar"], p["u"].sum(), rtol=1e-11)
    for k in range(3):
        m = p["cls"] == k
        np.testing.assert_allclose(r["deps"][k], p["u_over_eps"][m].sum(), rtol=1e-11)
        np.testing.assert_allclose(r["dsig"][k], p["du_dsig"][m].sum(), rtol=1e-11)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("kind", ["ortho", "tri"])
@pytest.mark.parametrize("typed", [True, False])
@pytest.mark.parametrize("precision", ["exact", "split"])
def test_gpu_adjoint_vs_oracle(orc, clm, dtype, kind, typed, precision):
    if precision == "split" and dtype == np.float32:
        pytest.skip("for Float32 inputs the split form is the exact form")
    x, L, t, eps, sig = mixture(clm, n=20000)
    M = np.diag([L] * 3) if kind == "ortho" else tri_cell(L)
    if kind == "tri":
        x = x / L @ M.T
    x = x.astype(dtype)
    uc = np.diag(M) if kind == "ortho" else M
    if typed:
        op = clm.LennardJonesAdjoint(c12=C12, c6=C6, types_x=t, eps_table=eps, sig_table=sig)
        teps, tsig, tt = eps, sig, t
    else:
        op = clm.LennardJonesAdjoint(eps=1.3, sigma=0.95, c12=C12, c6=C6)
        teps, tsig, tt = np.full((1, 1), 1.3), np.full((1, 1), 0.95), np.zeros(len(x), np.int32)
    sysm = clm.ParticleSystem(positions=x, unitcell=uc, cutoff=CUT, dtype=dtype)
    if precision == "split":
        sysm.set_precision("split")
    got = clm.pairwise(op, sysm)
    ref = orc.run("lj_adjoint", x, dim=3, kind=kind, unitcell=uc, cutoff=CUT, lcell=1, dtype=dtype,
                  params=[1.0, 1.0, C12, C6], types_x=tt, eps_table=teps, sig_table=tsig)
    p = pair_terms(orc, x, M, tt, teps, tsig, kind, dtype=dtype)
    tol = 1e-12 if (dtype == np.float64 and precision == "exact") else 1e-5
    assert abs(got.energy - ref["scalar"]) <= tol * np.abs(p["u"]).sum()
    fscale = np.abs(ref["forces_x"]).max()
    assert np.abs(np.asarray(got.forces, np.float64) - ref["forces_x"]).max() <= tol * fscale
    wscale = np.abs(p["g"] * (p["dx"] ** 2).sum(1)).sum()
    assert np.abs(got.virial - ref["virial"]).max() <= tol * wscale
    dcell = ref["virial"] @ np.linalg.inv(M).T
    assert np.abs(got.dU_dcell - dcell).max() <= tol * wscale * np.abs(np.linalg.inv(M)).sum()
    if typed:
        for a in range(2):
            for b in range(2):
                k = cls_index(a, b)
                m = p["cls"] == k
                assert abs(got.dU_deps[a, b] - ref["deps"][k]) <= tol * np.abs(p["u_over_eps"][m]).sum()
                assert abs(got.dU_dsigma[a, b] - ref["dsig"][k]) <= tol * np.abs(p["du_dsig"][m]).sum()
    else:
        assert abs(got.dU_deps - ref["deps"][0]) <= tol * np.abs(p["u_over_eps"]).sum()
        assert abs(got.dU_dsigma - ref["dsig"][0]) <= tol * np.abs(p["du_dsig"]).sum()
    np.testing.assert_allclose(got.grad_positions, -np.asarray(got.forces))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gpu_adjoint_2d(orc, clm, dtype):
    """2D: a jittered square lattice with two types in a periodic square; same bars as in 3D."""
    rng = np.random.default_rng(9)
    m = 60
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), indexing="ij"), -1).reshape(-1, 2) * 1.1
    x = (g + rng.normal(0, 0.05, g.shape)).astype(dtype)
    L = m * 1.1
    t = (rng.random(len(x)) < 0.3).astype(np.int32)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    op = clm.LennardJonesAdjoint(c12=C12, c6=C6, types_x=t, eps_table=eps, sig_table=sig)
    sysm = clm.ParticleSystem(positions=x, unitcell=[L, L], cutoff=CUT, dtype=dtype)
    got = clm.pairwise(op, sysm)
    ref = orc.run("lj_adjoint", x, dim=2, kind="ortho", unitcell=[L, L], cutoff=CUT, dtype=dtype,
                  params=[1.0, 1.0, C12, C6], types_x=t, eps_table=eps, sig_table=sig)
    nl = orc.run("nl", x, dim=2, kind="ortho", unitcell=[L, L], cutoff=CUT, dtype=dtype)
    i, j = nl["i"], nl["j"]
    d2 = np.asarray(nl["d"], np.float64) ** 2
    e, sg = eps[t[i], t[j]], sig[t[i], t[j]]
    sr6 = (sg * sg / d2) ** 3
    u = e * (C12 * sr6 * sr6 - C6 * sr6)
    gw = np.abs(e * (-12 * C12 * sr6 * sr6 + 6 * C6 * sr6))  # |g| d^2, bounds each virial contribution
    tol = 1e-12 if dtype == np.float64 else 1e-5
    assert got.virial.shape == (2, 2)
    assert abs(got.energy - ref["scalar"]) <= tol * np.abs(u).sum()
    assert np.abs(got.virial - ref["virial"]).max() <= tol * gw.sum()
    assert np.abs(np.asarray(got.forces, np.float64) - ref["forces_x"]).max() <= tol * np.abs(ref["forces_x"]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ortho", "tri"])
def test_autograd_lj_energy(orc, clm, kind):
    """torch autograd through the adjoint: gradients equal the oracle's adjoint (the counterpart of the
    ChainRulesCore rrule written out for the Julia extension)."""
    torch = pytest.importorskip("torch")
    import importlib
    ag = importlib.import_module(clm.__name__ + ".autograd")
    x, L, t, eps, sig = mixture(clm, n=4000)
    M = np.diag([L] * 3) if kind == "ortho" else tri_cell(L)
    if kind == "tri":
        x = x / L @ M.T
    xt = torch.tensor(x, requires_grad=True)
    cell = torch.tensor(np.diag(M) if kind == "ortho" else M, requires_grad=True)
    et = torch.tensor(eps, requires_grad=True)
    st = torch.tensor(sig, requires_grad=True)
    U = ag.lj_energy(xt, cell, et, st, torch.tensor(t), CUT, C12, C6)
    U.backward()
    ref = orc_adj(orc, x, M, t, eps, sig, kind=kind)
    p = pair_terms(orc, x, M, t, eps, sig, kind)
    tol = 1e-12
    assert abs(U.item() - ref["scalar"]) <= tol * np.abs(p["u"]).sum()
    assert np.abs(xt.grad.numpy() + ref["forces_x"]).max() <= tol * np.abs(ref["forces_x"]).max()
    dM = ref["virial"] @ np.linalg.inv(M).T
    gcell = cell.grad.numpy()
    want = np.diag(dM) if kind == "ortho" else dM
    wscale = np.abs(p["g"] * (p["dx"] ** 2).sum(1)).sum() * np.abs(np.linalg.inv(M)).sum()
    assert np.abs(gcell - want).max() <= tol * wscale
    for a in range(2):
        for b in range(2):
            k = cls_index(a, b)
            f = 1.0 if a == b else 0.5
            m = p["cls"] == k
            assert abs(et.grad[a, b].item() - f * ref["deps"][k]) <= tol * np.abs(p["u_over_eps"][m]).sum()
            assert abs(st.grad[a, b].item() - f * ref["dsig"][k]) <= tol * np.abs(p["du_dsig"][m]).sum()


@pytest.mark.gpu
@pytest.mark.parametrize("cell", ["cubic", "triclinic"])
def test_gpu_adjoint_finite_differences(clm, cell):
    """The GPU adjoint against FP64 central differences of the GPU's own LJ energy (the library
    differentiated, not the oracle): dU/dx = -F at a few particles, dU/dM (cubic: dU/dL = tr W / L), and
    dU/deps, dU/dsigma per type pair; 2,000-particle Float64 mixture, relative bar 1e-6 (1e-5 for the
    position derivatives, whose differences cancel more), as in the oracle's own finite-difference test.
    The reference checks its ForwardDiff gradients the same way (test/examples/generic_types.jl:10-20,102)."""
    x, L, t, eps, sig = mixture(clm, n=2000, seed=7)
    M = np.diag([L] * 3) if cell == "cubic" else tri_cell(L)
    if cell == "triclinic":
        x = x / L @ M.T
    uc = np.diag(M) if cell == "cubic" else M

    def energy(xx, MM, e_tab, s_tab):
        s = clm.ParticleSystem(positions=xx, unitcell=np.diag(MM) if cell == "cubic" else MM, cutoff=CUT,
                               dtype=np.float64)
        u = clm.pairwise(clm.LennardJones(c12=C12, c6=C6, types_x=t, eps_table=e_tab, sig_table=s_tab), s)
        s.close()
        return u

    s = clm.ParticleSystem(positions=x, unitcell=uc, cutoff=CUT, dtype=np.float64)
    a = clm.pairwise(clm.LennardJonesAdjoint(c12=C12, c6=C6, types_x=t, eps_table=eps, sig_table=sig), s)
    s.close()
    assert abs(a.energy - energy(x, M, eps, sig)) <= 1e-12 * abs(a.energy)
    h = 1e-6
    for p in range(2):
        for q in range(p, 2):
            for table, got in ((eps, a.dU_deps), (sig, a.dU_dsigma)):
                tp, tm = table.copy(), table.copy()
                tp[p, q] += h
                tp[q, p] = tp[p, q]
                tm[p, q] -= h
                tm[q, p] = tm[p, q]
                if table is eps:
                    fd = (energy(x, M, tp, sig) - energy(x, M, tm, sig)) / (2 * h)
                else:
                    fd = (energy(x, M, eps, tp) - energy(x, M, eps, tm)) / (2 * h)
                assert abs(got[p, q] - fd) <= 1e-6 * max(1.0, abs(fd)), (p, q, got[p, q], fd)
    # the cell, positions following it (scaled coordinates fixed)
    Minv = np.linalg.inv(M)
    entries = [(0, 0), (1, 1), (2, 2)] if cell == "cubic" else [(0, 0), (0, 1), (1, 2), (2, 2), (0, 2)]
    for r, c in entries:
        E = np.zeros((3, 3))
        E[r, c] = h
        fd = (energy(x @ ((M + E) @ Minv).T, M + E, eps, sig) - energy(x @ ((M - E) @ Minv).T, M - E, eps, sig)) / (2 * h)
        assert abs(a.dU_dcell[r, c] - fd) <= 1e-6 * max(1.0, abs(fd)), (r, c, a.dU_dcell[r, c], fd)
    if cell == "cubic":
        fd = (energy(x * (L + h) / L, np.diag([L + h] * 3), eps, sig)
              - energy(x * (L - h) / L, np.diag([L - h] * 3), eps, sig)) / (2 * h)
        assert abs(np.trace(a.virial) / L - fd) <= 1e-6 * abs(fd)
    for i in (0, 11, len(x) - 5):
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[i, c] += h
            xm[i, c] -= h
            fd = (energy(xp, M, eps, sig) - energy(xm, M, eps, sig)) / (2 * h)
            assert abs(-a.forces[i, c] - fd) <= 1e-5 * max(1.0, abs(fd)), (i, c, a.forces[i, c], fd)
