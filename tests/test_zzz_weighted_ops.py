"""GPU parity of the weighted inverse-distance operator (CLM_OP_WEIGHTED_INV_D): the gravitational
potential and force examples of the reference with per-particle masses, against the oracle.  Kept in its
own file, after the other GPU suites."""
import numpy as np
import pytest

from tests.test_gpu_parity import TOL


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("cross", [False, True])
@pytest.mark.parametrize("tri", [False, True])
def test_weighted_inverse_distance_on_gpu(clm, orc, dtype, cross, tri):
    """The gravitational examples' closures (test/examples/gravitational_potential.jl:30-33,
    gravitational_force.jl:37-46) with per-particle masses, against the oracle."""
    rng = np.random.default_rng(31 + cross + 2 * tri)
    side = 40.0
    x = (rng.random((4000, 3)) * side).astype(dtype)
    y = (rng.random((2500, 3)) * side).astype(dtype) if cross else None
    m = 5 * x[:, 0].astype(np.float64)
    my = 5 * y[:, 0].astype(np.float64) if cross else None
    uc = [[side, 4.0, 2.0], [0.0, side, 3.0], [0.0, 0.0, side]] if tri else [side] * 3
    s = clm.ParticleSystem(xpositions=x, ypositions=y, unitcell=uc, cutoff=6.0, dtype=dtype)
    ef = clm.pairwise(clm.WeightedInverseDistance(m, 9.8, my), s)
    r = orc.run("weighted_inv_d", x, y, kind="tri" if tri else "ortho", unitcell=uc, cutoff=6.0, dtype=dtype,
                params=[9.8], weights_x=m, weights_y=my)
    tol = TOL[dtype]
    assert abs(ef.energy - r["scalar"]) <= tol * abs(r["scalar"])
    fx = np.asarray(ef.forces, np.float64)
    assert np.abs(fx - r["forces_x"]).max() <= tol * np.abs(r["forces_x"]).max()
    if cross:
        fy = np.asarray(ef.forces_y, np.float64)
        assert np.abs(fy - r["forces_y"]).max() <= tol * np.abs(r["forces_y"]).max()
    s.close()
