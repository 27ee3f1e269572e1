"""clm_run_noalloc: pair-map reductions for callers that cannot allocate device memory where they
evaluate (under an application-owned device pool, or in a real-time loop that must not enter the CUDA
allocator).

The entry point is checked through the C ABI against clm_run on the same built handle, on two calls in
a row (the calls share a static scratch array, which keeps the previous call's contents), and the
device's free memory must not move across repeated calls.  Runs last so that a failure here leaves every
other test already run; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-12, np.float32: 1e-5}
OPS = [("soft_energy", ()), ("count", ()), ("sum_d2", ()), ("lj_energy", (1.0, 1.0, 4.0, 4.0)), ("mindist", ())]


def _built_system(clm, dtype, triclinic):
    rng = np.random.default_rng(12)
    x = (rng.random((20000, 3)) * 30.0).astype(dtype)
    uc = np.array([[30.0, 3.0, 1.0], [0.0, 30.0, 2.0], [0.0, 0.0, 30.0]]) if triclinic else [30.0, 30.0, 30.0]
    s = clm.ParticleSystem(xpositions=x, unitcell=uc, cutoff=2.0, dtype=dtype)
    s.build()
    return s


def _params(A, values):
    p = A.OpParams()
    for k, v in enumerate(values):
        p.p[k] = v
    return p


@pytest.mark.parametrize("triclinic", [False, True])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_noalloc_matches_clm_run_on_two_calls(clm, dtype, triclinic):
    A = clm._abi
    L = A.load()
    s = _built_system(clm, dtype, triclinic)
    h = s._handle.h
    for op, values in OPS:
        p = _params(A, values)
        ref = A.Outputs()
        assert L.clm_run(h, A.OP[op], C.byref(p), C.byref(ref)) == 0
        for _ in range(2):
            o = A.Outputs()
            assert L.clm_run_noalloc(h, A.OP[op], C.byref(p), C.byref(o)) == 0, op
            if op == "count":
                assert o.count == ref.count
            elif op == "mindist":
                assert o.min_d == ref.min_d and (o.min_i, o.min_j) == (ref.min_i, ref.min_j)
            else:
                assert abs(o.scalar - ref.scalar) <= TOL[dtype] * abs(ref.scalar), (op, o.scalar, ref.scalar)
    s.close()


def test_noalloc_leaves_device_memory_untouched(clm):
    torch = pytest.importorskip("torch")
    A = clm._abi
    L = A.load()
    s = _built_system(clm, np.float64, False)
    h = s._handle.h
    p = _params(A, ())
    o = A.Outputs()
    assert L.clm_run_noalloc(h, A.OP["soft_energy"], C.byref(p), C.byref(o)) == 0  # first call: set-up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(20):
        assert L.clm_run_noalloc(h, A.OP["soft_energy"], C.byref(p), C.byref(o)) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    s.close()


def test_noalloc_refuses_what_would_allocate(clm):
    A = clm._abi
    L = A.load()
    s = _built_system(clm, np.float64, False)
    h = s._handle.h
    o = A.Outputs()
    # forces and neighbour lists need buffers sized by the system: refused, not allocated
    assert L.clm_run_noalloc(h, A.OP["soft_forces"], C.byref(_params(A, ())), C.byref(o)) == 1
    assert L.clm_run_noalloc(h, A.OP["nl"], C.byref(_params(A, ())), C.byref(o)) == 1
    # dirty positions would need a rebuild, which allocates: refused with CLM_ERR_STATE
    s.update(xpositions=np.asarray(s.xpositions) + 0.1)
    assert L.clm_run_noalloc(h, A.OP["soft_energy"], C.byref(_params(A, ())), C.byref(o)) == 7
    s.build()
    assert L.clm_run_noalloc(h, A.OP["soft_energy"], C.byref(_params(A, ())), C.byref(o)) == 0
    # per-type LJ tables are staged in handle buffers: refused with CLM_ERR_ARG
    p = _params(A, (1.0, 1.0, 4.0, 4.0))
    t = np.zeros(s.n_x, np.int32)
    tab = np.ones(1)
    p.ntypes, p.types_x, p.eps_table, p.sig_table = 1, t.ctypes.data, tab.ctypes.data, tab.ctypes.data
    assert L.clm_run_noalloc(h, A.OP["lj_energy"], C.byref(p), C.byref(o)) == 1
    s.close()


def test_noalloc_refuses_a_build_nobody_checked(clm):
    # clm_run enqueues the rebuild of updated positions and checks its totals and error bits with the map's
    # results; when it returns early (an unknown operator), the rebuilt set was never checked, so the
    # allocation-free entry point refuses it (CLM_ERR_STATE) until clm_build has checked a build again
    A = clm._abi
    L = A.load()
    s = _built_system(clm, np.float64, False)
    h = s._handle.h
    o = A.Outputs()
    x2 = np.asarray(s.xpositions) + 0.05
    s.update(xpositions=x2)
    assert L.clm_run(h, 999, C.byref(_params(A, ())), C.byref(o)) == 1
    assert L.clm_run_noalloc(h, A.OP["soft_energy"], C.byref(_params(A, ())), C.byref(o)) == 7
    s.build()
    assert L.clm_run_noalloc(h, A.OP["soft_energy"], C.byref(_params(A, ())), C.byref(o)) == 0
    ref = A.Outputs()
    assert L.clm_run(h, A.OP["soft_energy"], C.byref(_params(A, ())), C.byref(ref)) == 0
    assert abs(o.scalar - ref.scalar) <= 1e-12 * abs(ref.scalar)
    s.close()
