"""Steady-state steps allocate nothing on the device: the GPU counterpart of the reference's allocation
tests for update!/neighborlist! on an InPlaceNeighborList (test/API/neighborlists.jl:114-177), single and
two sets, periodic and non-periodic.  Buffers grow only: the first list at a larger cutoff may grow the
neighbour-list capacity, later ones do not.  Replayed batched steps allocate nothing either."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("two_sets", [False, True])
def test_in_place_neighbor_list_steps_allocate_nothing(clm, periodic, two_sets):
    rng = np.random.default_rng(7)

    def pos():
        return rng.random((1000, 3)), (rng.random((1000, 3)) if two_sets else None)

    x, y = pos()
    uc = [1.0, 1.0, 1.0] if periodic else None
    s = clm.InPlaceNeighborList(xpositions=x, ypositions=y, cutoff=0.1, unitcell=uc)
    clm.neighborlist_(s)
    c0 = clm.device_allocations()[0]
    for _ in range(3):
        x, y = pos()
        clm.update(s, xpositions=x, ypositions=y)
        assert clm.device_allocations()[0] == c0
        i, j, d = clm.neighborlist_(s)
        assert len(i) > 0
        assert clm.device_allocations()[0] == c0
    clm.update(s, xpositions=x, ypositions=y, cutoff=0.2)
    assert clm.device_allocations()[0] == c0
    clm.neighborlist_(s)  # the list is ~8x longer: its capacity may grow once
    c1 = clm.device_allocations()[0]
    for _ in range(2):
        x, y = pos()
        clm.update(s, xpositions=x, ypositions=y)
        clm.neighborlist_(s)
    assert clm.device_allocations()[0] == c1
    s.sys.close()


def test_batched_graph_replays_allocate_nothing(clm):
    rng = np.random.default_rng(8)
    sides = [14.0, 18.0, 22.0]
    pos = [rng.random((int(0.1 * L ** 3), 3)) * L for L in sides]
    bs = clm.BatchedSystems(positions=pos, unitcells=[[L] * 3 for L in sides], cutoff=6.0, graph=True)
    bs.run(clm.NeighborList(), clm.SoftEnergy())  # direct run, then the step is recorded
    bs.run(clm.NeighborList(), clm.SoftEnergy())  # first replay
    c0 = clm.device_allocations()[0]
    for _ in range(3):
        bs.update(positions=np.concatenate([p + rng.normal(0, 0.01, p.shape) for p in pos]))
        bs.run(clm.NeighborList(), clm.SoftEnergy())
    assert clm.device_allocations()[0] == c0
    bs.close()
