"""Host-side mirror of CellListMap.jl's user API over the GPU library.

Names follow the reference (src/API/*.jl); Julia's mutating `!` functions map
to Python callables without the bang (``pairwise``/``pairwise_`` for
``pairwise!``, ``neighborlist_`` for ``neighborlist!``, ``update`` for
``update!``).  The pair function is one of the built-in operators of
``ops`` instead of a Julia closure: those are the operators the GPU library
implements.  Indices are 0-based (as in the reference's Python interface,
test/examples/CellListMap.py:19-58); pass ``index_base=1`` for Julia indices.

Errors map to the reference's exception types: ``ArgumentError`` (NaN
coordinates, unit cell too small, lcell < 1, non-periodic unit-cell update)
and ``DimensionMismatch``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Any, Optional

import numpy as np

from . import _abi


class ArgumentError(ValueError):
    """Mirror of Julia's ArgumentError."""


class DimensionMismatch(ValueError):
    """Mirror of Julia's DimensionMismatch."""


class CUDAError(RuntimeError):
    """A CUDA runtime call inside the library failed."""


def _raise(handle, status: int):
    msg = ""
    if handle:
        buf = C.create_string_buffer(512)
        _abi.load().clm_last_error(handle, buf, 512)
        msg = buf.value.decode(errors="replace")
    name = _abi.STATUS.get(status, str(status))
    if status in (1, 2, 3, 10, 11):
        raise ArgumentError(f"{name}: {msg}")
    if status == 4:
        raise DimensionMismatch(f"{name}: {msg}")
    if status in (5, 9):
        raise CUDAError(f"{name}: {msg}")
    raise RuntimeError(f"{name}: {msg}")


# ---------------------------------------------------------------------------- operators
class Operator:
    """A built-in pair operator (the GPU counterpart of a `f(pair, output)` closure)."""
    op = ""

    def params(self, system) -> tuple[_abi.OpParams, list]:
        return _abi.OpParams(), []

    def outputs(self, system) -> tuple[_abi.Outputs, dict]:
        return _abi.Outputs(), {}

    def result(self, system, out: _abi.Outputs, bufs: dict):
        return out.scalar


class Count(Operator):
    """Number of pairs within the cutoff (`(pair, n) -> n + 1`)."""
    op = "count"

    def result(self, system, out, bufs):
        return int(out.count)


class SumD2(Operator):
    """`output += pair.d2` (src/API/ParticleSystem.jl:110-118)."""
    op = "sum_d2"


class SumD(Operator):
    """`output += pair.d` (test/modules/Testing.jl:22)."""
    op = "sum_d"


class SumInvD(Operator):
    """`output += 1/pair.d`."""
    op = "sum_inv_d"


class SoftEnergy(Operator):
    """u = sum (c - d)^2 over pairs (c defaults to the cutoff; test/examples/packmol.jl:49-55)."""
    op = "soft_energy"

    def __init__(self, c: Optional[float] = None):
        self.c = c

    def params(self, system):
        p = _abi.OpParams()
        p.p[0] = float(self.c) if self.c is not None else 0.0
        return p, []


@dataclass
class EnergyAndForces:
    energy: float
    forces: Any
    forces_y: Any = None


class _ForcesOp(Operator):
    def outputs(self, system):
        o = _abi.Outputs()
        dt = system.dtype
        fx = np.zeros((system.n_x, system.dim), dtype=dt)
        o.forces_x = fx.ctypes.data
        bufs = {"fx": fx}
        if system.nsets == 2:
            fy = np.zeros((system.n_y, system.dim), dtype=dt)
            o.forces_y = fy.ctypes.data
            bufs["fy"] = fy
        return o, bufs

    def result(self, system, out, bufs):
        return EnergyAndForces(out.scalar, bufs["fx"], bufs.get("fy"))


class SoftForces(_ForcesOp, SoftEnergy):
    """Energy and forces of sum (c - d)^2; forces are -grad U (f[i] -= df; f[j] += df,
    test/examples/gravitational_force.jl:37-44)."""
    op = "soft_forces"


class LennardJones(Operator):
    """u = eps*(c12 (sigma/d)^12 - c6 (sigma/d)^6); (c12, c6) = (4, 4) is the usual LJ,
    (1, 2) the NAMD form (test/applications/namd/ParticleSystem_vs_NAMD.jl:15-18).
    Optional per-type tables: `types_x` (and `types_y`), `eps_table`, `sig_table` (ntypes x ntypes)."""
    op = "lj_energy"

    def __init__(self, eps=1.0, sigma=1.0, c12=4.0, c6=4.0, types_x=None, types_y=None, eps_table=None,
                 sig_table=None):
        self.eps, self.sigma, self.c12, self.c6 = eps, sigma, c12, c6
        self.types_x, self.types_y, self.eps_table, self.sig_table = types_x, types_y, eps_table, sig_table

    def params(self, system):
        p = _abi.OpParams()
        p.p[0], p.p[1], p.p[2], p.p[3] = float(self.eps), float(self.sigma), float(self.c12), float(self.c6)
        keep = []
        if self.types_x is not None:
            tx = np.ascontiguousarray(self.types_x, dtype=np.int32)
            et = np.ascontiguousarray(self.eps_table, dtype=np.float64)
            st = np.ascontiguousarray(self.sig_table, dtype=np.float64)
            if tx.shape[0] != system.n_x or et.ndim != 2 or et.shape != st.shape or et.shape[0] != et.shape[1]:
                raise DimensionMismatch("types/eps/sigma tables do not match the system")
            if tx.size and (tx.min() < 0 or tx.max() >= et.shape[0]):
                raise ArgumentError("particle type out of range of the tables")
            p.ntypes = et.shape[0]
            p.types_x, p.eps_table, p.sig_table = tx.ctypes.data, et.ctypes.data, st.ctypes.data
            keep += [tx, et, st]
            if system.nsets == 2:
                ty = np.ascontiguousarray(self.types_y, dtype=np.int32)
                if ty.shape[0] != system.n_y:
                    raise DimensionMismatch("types_y does not match the second set")
                p.types_y = ty.ctypes.data
                keep.append(ty)
        return p, keep


class LennardJonesForces(_ForcesOp, LennardJones):
    """Energy and forces (-grad U) of LennardJones."""
    op = "lj_forces"


@dataclass
class LJAdjoint:
    """Energy of a Lennard-Jones system and its adjoint (gradients of U)."""
    energy: float
    forces: Any              # -dU/dx (n x dim)
    virial: Any              # W = sum g dx dx^T, g = u'(r)/r (dim x dim)
    dU_dcell: Any            # dU/dM = W M^-T for the cell matrix M, scaled coordinates fixed (periodic cells)
    dU_deps: Any             # per type pair (ntypes x ntypes, symmetric) or scalar
    dU_dsigma: Any

    @property
    def grad_positions(self):
        return -np.asarray(self.forces)

    def dU_dL(self, L):
        """Derivative w.r.t. the side of a cubic box (all sides scaled together)."""
        return float(np.trace(self.virial)) / float(L)


class LennardJonesAdjoint(LennardJones):
    """Energy, forces and the adjoint of U w.r.t. the cell matrix and the per-type eps/sigma (at most 2
    types).  No reference counterpart: the reference differentiates closures with ForwardDiff
    (test/examples/generic_types.jl:10-20,102)."""
    op = "lj_adjoint"

    def outputs(self, system):
        o = _abi.Outputs()
        fx = np.zeros((system.n_x, system.dim), dtype=system.dtype)
        adj = np.zeros(32, np.float64)
        o.forces_x = fx.ctypes.data
        o.adjoint = adj.ctypes.data
        return o, {"fx": fx, "adj": adj}

    def result(self, system, out, bufs):
        adj = bufs["adj"]
        d = system.dim
        W = adj[:9].reshape(3, 3)[:d, :d].copy()
        nt = 0 if self.types_x is None else int(np.asarray(self.eps_table).shape[0])
        ncls = nt * (nt + 1) // 2 if nt else 1
        de, ds = adj[9:9 + ncls], adj[9 + ncls:9 + 2 * ncls]
        if nt:
            tde = np.zeros((nt, nt))
            tds = np.zeros((nt, nt))
            k = 0
            for a in range(nt):
                for b in range(a, nt):
                    tde[a, b] = tde[b, a] = de[k]
                    tds[a, b] = tds[b, a] = ds[k]
                    k += 1
            de, ds = tde, tds
        else:
            de, ds = float(de[0]), float(ds[0])
        dcell = None
        if system.unitcell is not None:
            _, M = _cell_kind_and_matrix(system.unitcell, d)
            dcell = W @ np.linalg.inv(M).T
        return LJAdjoint(out.scalar, bufs["fx"], W, dcell, de, ds)


class InverseDistanceForces(_ForcesOp):
    """energy += 1/d, forces[i] += (y - x)/d^3, forces[j] -= (y - x)/d^3 (the gradient convention of
    docs/src/ParticleSystem/single_set_compound.md:79-86).  Returned forces follow that convention."""
    op = "inv_d_forces"


class WeightedInverseDistance(_ForcesOp):
    """Per-particle weights w (masses, charges): energy u -= c w_i w_j / d and forces
    df = (c w_i w_j / d^2 / d) (x_i - x_j), f[i] -= df, f[j] += df — the gravitational potential and force
    examples with w = mass and c = 9.8 (test/examples/gravitational_potential.jl:30-33,
    test/examples/gravitational_force.jl:37-46).  `weights_y` for two sets."""
    op = "weighted_inv_d"

    def __init__(self, weights_x, c=9.8, weights_y=None):
        self.weights_x, self.weights_y, self.c = weights_x, weights_y, c

    def params(self, system):
        p = _abi.OpParams()
        p.p[0] = float(self.c)
        wx = np.ascontiguousarray(self.weights_x, dtype=np.float64).reshape(-1)
        if wx.shape[0] != system.n_x:
            raise DimensionMismatch("weights_x does not match the first set")
        p.weights_x = wx.ctypes.data
        keep = [wx]
        if system.nsets == 2:
            if self.weights_y is None:
                raise ArgumentError("weights_y is required for two sets")
            wy = np.ascontiguousarray(self.weights_y, dtype=np.float64).reshape(-1)
            if wy.shape[0] != system.n_y:
                raise DimensionMismatch("weights_y does not match the second set")
            p.weights_y = wy.ctypes.data
            keep.append(wy)
        return p, keep


class MinimumDistance(Operator):
    """Pair with the smallest distance (test/examples/nearest_neighbor.jl:9-16,43); returns (i, j, d),
    (-1, -1, inf) when no pair is within the cutoff."""
    op = "mindist"

    def __init__(self, index_base: int = 0):
        self.index_base = index_base

    def outputs(self, system):
        o = _abi.Outputs()
        o.index_base = self.index_base
        return o, {}

    def result(self, system, out, bufs):
        if not np.isfinite(out.min_d):
            return (-1, -1, float("inf"))
        return (int(out.min_i), int(out.min_j), float(out.min_d))


class RadialHistogram(Operator):
    """Per-bin pair counts and sums of dot(v_i - v_j, x - y)/r
    (test/examples/pairwise_velocities.jl:17-24).  `bins` are nbins+1 ascending edges;
    r on an edge goes to the lower bin; r <= bins[0] is dropped."""
    op = "rhist"

    def __init__(self, bins, velocities_x, velocities_y=None):
        self.bins = np.ascontiguousarray(bins, dtype=np.float64)
        self.vx = velocities_x
        self.vy = velocities_y

    def params(self, system):
        p = _abi.OpParams()
        nb = self.bins.shape[0] - 1
        if nb < 1 or nb > 256:
            raise ArgumentError("RadialHistogram supports 1..256 bins")
        p.nbins = nb
        vx = np.ascontiguousarray(self.vx, dtype=system.dtype).reshape(-1, system.dim)
        if vx.shape[0] != system.n_x:
            raise DimensionMismatch("velocities do not match the first set")
        keep = [self.bins, vx]
        p.bins, p.vel_x = self.bins.ctypes.data, vx.ctypes.data
        if system.nsets == 2:
            vy = np.ascontiguousarray(self.vy, dtype=system.dtype).reshape(-1, system.dim)
            if vy.shape[0] != system.n_y:
                raise DimensionMismatch("velocities do not match the second set")
            p.vel_y = vy.ctypes.data
            keep.append(vy)
        return p, keep

    def outputs(self, system):
        o = _abi.Outputs()
        nb = self.bins.shape[0] - 1
        hc = np.zeros(nb, np.int64)
        hs = np.zeros(nb, np.float64)
        o.hist_count, o.hist_sum = hc.ctypes.data, hs.ctypes.data
        return o, {"hc": hc, "hs": hs}

    def result(self, system, out, bufs):
        return bufs["hc"], bufs["hs"]


class NeighborList(Operator):
    """push_pair!: list of (i, j, d) (src/internals/neighborlist.jl:67-76); unordered."""
    op = "nl"

    def __init__(self, index_base: int = 0):
        self.index_base = index_base

    def result(self, system, out, bufs):
        return system._fetch_nl(self.index_base)


OPERATORS = {c.op: c for c in [Count, SumD2, SumD, SumInvD, SoftEnergy, SoftForces, LennardJones, LennardJonesForces,
                               LennardJonesAdjoint, InverseDistanceForces, MinimumDistance, RadialHistogram,
                               NeighborList]}


# ---------------------------------------------------------------------------- helpers
def _promote_dtype(unitcell, cutoff, dtype):
    """_promote_types (src/internals/Box.jl:132-142): the promoted element type of the unit cell and the
    cutoff, integers yielding to any float type (Julia's promote_type(Int, Float32) is Float32) and integers
    alone giving Float64."""
    if dtype is not None:
        return np.dtype(dtype)
    floats = [t for t in (np.asarray(v).dtype for v in (cutoff, unitcell) if v is not None)
              if np.issubdtype(t, np.floating)]
    if not floats:
        return np.dtype(np.float64)
    t = np.result_type(*floats)
    return t if t in (np.float32, np.float64) else np.dtype(np.float64)


def _as_positions(x, dim, dtype):
    """Positions as an (n, dim) contiguous array (memory = Julia's dim x n column-major).
    Returns (array_or_tensor, n, is_device, keepalive)."""
    try:
        import torch  # noqa: F401
        is_torch = hasattr(x, "is_cuda") and hasattr(x, "data_ptr")
    except ImportError:  # pragma: no cover
        is_torch = False
    if is_torch:
        import torch
        tdt = torch.float64 if dtype == np.float64 else torch.float32
        t = x.to(tdt).contiguous()
        if t.ndim != 2 or t.shape[1] != dim:
            raise DimensionMismatch(f"Positions have dimension {t.shape[-1] if t.ndim else 0}, "
                                    f"but the unit cell has dimension {dim}.")
        return t, t.shape[0], bool(t.is_cuda), t
    a = np.asarray(x, dtype=dtype)
    if a.ndim == 1 and a.size == 0:
        a = a.reshape(0, dim)
    if a.ndim != 2 or a.shape[1] != dim:
        got = a.shape[-1] if a.ndim >= 1 else 0
        raise DimensionMismatch(f"Positions have dimension {got}, but the unit cell has dimension {dim}.")
    a = np.ascontiguousarray(a)
    return a, a.shape[0], False, a


def _get_dim(unitcell, x, y=None):
    """get_dim (src/internals/auxiliary_functions.jl:8-37)."""
    ds = [np.asarray(unitcell).shape[0] if unitcell is not None else 0]
    for p in (x, y):
        if p is None:
            ds.append(0)
            continue
        shp = tuple(p.shape) if hasattr(p, "shape") else np.asarray(p).shape
        ds.append(shp[-1] if len(shp) == 2 and shp[0] > 0 else (shp[-1] if len(shp) == 2 else 0))
    D = max(ds)
    if D == 0:
        raise ArgumentError("Could not infer dimension (2 or 3) from the unitcell or coordinate arrays.")
    if D not in (2, 3):
        raise ArgumentError("Dimension must be 2 or 3.")
    if any(d not in (0, D) for d in ds):
        raise ArgumentError(f"Incompatible dimensions between unitcell and/or coordinates. Got: {ds}")
    return D


def _cell_kind_and_matrix(unitcell, dim):
    if unitcell is None:
        return _abi.CLM_NONPERIODIC, np.zeros((dim, dim))
    u = np.asarray(unitcell, dtype=np.float64)
    if u.ndim == 1:
        if u.shape[0] != dim:
            raise DimensionMismatch("unit cell sides must have one entry per dimension")
        return _abi.CLM_ORTHO, np.diag(u)
    if u.shape != (dim, dim):
        raise ArgumentError("Unit cell matrix must be square.")
    return _abi.CLM_TRICLINIC, u


class _Handle:
    """Owns one library handle."""

    def __init__(self, dtype, dim, nsets):
        L = _abi.load()
        h = C.c_void_p()
        st = L.clm_create(_abi.CLM_F64 if np.dtype(dtype) == np.float64 else _abi.CLM_F32, dim, nsets, C.byref(h))
        if st:
            _raise(None, st)
        self.h = h
        self.L = L

    def check(self, st):
        if st:
            _raise(self.h, st)

    def close(self):
        if getattr(self, "h", None):
            self.L.clm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass


# ---------------------------------------------------------------------------- ParticleSystem
class ParticleSystem:
    """Mirror of `ParticleSystem(; xpositions, ypositions, unitcell, cutoff, output, output_name, parallel,
    nbatches, lcell, validate_coordinates)` (src/API/ParticleSystem.jl:142-202).

    `output` is the initial output value (kept for API parity; operators create their own outputs).
    `parallel` and `nbatches` are accepted and ignored (the GPU grid replaces the thread batches).
    `precision` selects the exact form (bit-exact with the reference's arithmetic) or the FP32-split form.
    Positions may be numpy arrays / lists (host) or torch tensors (CUDA tensors stay on the device).
    """

    def __init__(self, *, positions=None, xpositions=None, ypositions=None, unitcell=None, cutoff, output=None,
                 output_name: str = "output", parallel: bool = True, nbatches=(0, 0), lcell: int = 1,
                 validate_coordinates=True, dtype=None, precision: str = "exact"):
        if (positions is None) == (xpositions is None):
            raise ArgumentError("Either `positions` OR `xpositions` must be defined.")
        x = positions if positions is not None else xpositions
        self.dim = _get_dim(unitcell, x, ypositions)
        self.dtype = _promote_dtype(unitcell, cutoff, dtype)
        self.nsets = 1 if ypositions is None else 2
        self.output = output
        self.output_name = output_name
        self.parallel = parallel
        self.nbatches = nbatches
        self._lcell = int(lcell)
        self._handle = _Handle(self.dtype, self.dim, self.nsets)
        self._unitcell = None if unitcell is None else np.asarray(unitcell, dtype=np.float64)
        self._cutoff = float(cutoff)
        self.set_precision(precision)
        self._apply_box()
        self._x = self._y = None
        self.n_x = self.n_y = 0
        self._set_positions(0, x)
        if ypositions is not None:
            self._set_positions(1, ypositions)
        self._handle.check(self._handle.L.clm_build(self._handle.h))

    # -- properties (src/API/ParticleSystem.jl:205-221)
    @property
    def positions(self):
        return self._x

    @property
    def xpositions(self):
        return self._x

    @xpositions.setter
    def xpositions(self, v):
        self._set_positions(0, v)

    @property
    def ypositions(self):
        return self._y

    @ypositions.setter
    def ypositions(self, v):
        if self.nsets != 2:
            raise ArgumentError("system has a single set of particles")
        self._set_positions(1, v)

    @property
    def unitcell(self):
        return self._unitcell

    @unitcell.setter
    def unitcell(self, v):
        self.update(unitcell=v)

    @property
    def cutoff(self):
        return self._cutoff

    @cutoff.setter
    def cutoff(self, v):
        self.update(cutoff=v)

    def __getattr__(self, name):
        if name != "output_name" and name == self.__dict__.get("output_name"):
            return self.__dict__.get("output")
        raise AttributeError(name)

    # -- internals
    def _apply_box(self):
        kind, M = _cell_kind_and_matrix(self._unitcell, self.dim)
        Mf = np.ascontiguousarray(M.flatten(order="F"), dtype=np.float64)
        st = self._handle.L.clm_set_box(self._handle.h, Mf.ctypes.data_as(C.POINTER(C.c_double)), kind,
                                        self._cutoff, self._lcell)
        self._handle.check(st)
        self.kind = kind

    def _set_positions(self, s, v):
        arr, n, dev, keep = _as_positions(v, self.dim, self.dtype)
        ptr = arr.data_ptr() if hasattr(arr, "data_ptr") else arr.ctypes.data
        st = self._handle.L.clm_set_positions(self._handle.h, s, ptr if n else None, n, 1 if dev else 0)
        self._handle.check(st)
        if s == 0:
            self._x, self.n_x = keep, n
        else:
            self._y, self.n_y = keep, n

    def set_precision(self, precision: str):
        p = {"exact": _abi.CLM_PREC_EXACT, "split": _abi.CLM_PREC_SPLIT}[precision]
        self._handle.check(self._handle.L.clm_set_precision(self._handle.h, p))
        self.precision = precision

    def update(self, *, xpositions=None, positions=None, ypositions=None, cutoff=None, unitcell=None,
               parallel=None):
        """update!(sys; positions, cutoff, unitcell, parallel) — src/API/updating.jl:165-187."""
        if positions is not None and xpositions is not None:
            raise ArgumentError("Either `positions` OR `xpositions` can be updated.")
        x = positions if positions is not None else xpositions
        if x is not None:
            self._set_positions(0, x)
        if ypositions is not None:
            self.ypositions = ypositions
        if unitcell is not None:
            if self.kind == _abi.CLM_NONPERIODIC:
                raise ArgumentError("Manual updating of the unit cell of non-periodic systems is not allowed.")
            self._unitcell = np.asarray(unitcell, dtype=np.float64)
        if cutoff is not None:
            self._cutoff = float(cutoff)
        if unitcell is not None or cutoff is not None:
            self._apply_box()
        if parallel is not None:
            self.parallel = parallel
        return self

    def build(self):
        """UpdateCellList! for dirty sets (normally implicit in pairwise)."""
        self._handle.check(self._handle.L.clm_build(self._handle.h))
        return self

    def _fetch_nl(self, base=0):
        L, h = self._handle.L, self._handle.h
        n = C.c_int64()
        self._handle.check(L.clm_nl_count(h, C.byref(n)))
        i = np.empty(n.value, np.int64)
        j = np.empty(n.value, np.int64)
        d = np.empty(n.value, self.dtype)
        self._handle.check(L.clm_nl_fetch(h, i.ctypes.data, j.ctypes.data, d.ctypes.data, n.value, base, 0))
        return i, j, d

    def run(self, op: Operator):
        p, keep = op.params(self)
        o, bufs = op.outputs(self)
        st = self._handle.L.clm_run(self._handle.h, _abi.OP[op.op], C.byref(p), C.byref(o))
        self._handle.check(st)
        del keep
        return op.result(self, o, bufs)

    def celllist_info(self, s: int = 0):
        a = [C.c_int64() for _ in range(4)]
        self._handle.check(self._handle.L.clm_get_celllist_info(self._handle.h, s, *[C.byref(v) for v in a]))
        return {"n_real_particles": a[0].value, "n_particles": a[1].value,
                "n_cells_with_particles": a[2].value, "n_cells_with_real_particles": a[3].value}

    def fetch_celllist(self, s: int = 0, index_base: int = 0):
        info = self.celllist_info(s)
        n = info["n_particles"]
        cell = np.empty(n, np.int64)
        idx = np.empty(n, np.int64)
        real = np.empty(n, np.int8)
        coords = np.empty((n, self.dim), self.dtype)
        self._handle.check(self._handle.L.clm_fetch_celllist(self._handle.h, s, n, cell.ctypes.data, idx.ctypes.data,
                                                             real.ctypes.data, coords.ctypes.data, index_base))
        return {"cell": cell, "index": idx, "real": real.astype(bool), "coords": coords}

    def box(self):
        return Box._from_handle(self._handle, self.dim)

    def last_timings(self):
        b, m = C.c_float(), C.c_float()
        self._handle.L.clm_last_timings(self._handle.h, C.byref(b), C.byref(m))
        return {"build_ms": b.value, "map_ms": m.value}

    def close(self):
        self._handle.close()


def pairwise(op: Operator, system: ParticleSystem, *, show_progress: bool = False, reset: bool = True):
    """pairwise!(f, sys) (src/API/pairwise.jl:48-63) for a built-in operator; stores and returns the output."""
    if not isinstance(op, Operator):
        raise ArgumentError("pairwise on the GPU takes a built-in operator from celllistmap_gb300.ops")
    out = system.run(op)
    if not reset and system.output is not None and isinstance(out, (int, float)) and \
            isinstance(system.output, (int, float)):
        out = system.output + out
    system.output = out
    return out


pairwise_ = pairwise


# ---------------------------------------------------------------------------- neighbour lists
class InPlaceNeighborList:
    """Mirror of InPlaceNeighborList (src/API/neighborlist.jl:84-111)."""

    def __init__(self, *, xpositions=None, positions=None, ypositions=None, cutoff, unitcell=None,
                 parallel: bool = True, nbatches=(0, 0), lcell: int = 1, validate_coordinates=True,
                 show_progress: bool = False, dtype=None, precision: str = "exact", index_base: int = 0):
        self.sys = ParticleSystem(xpositions=xpositions, positions=positions, ypositions=ypositions, cutoff=cutoff,
                                  unitcell=unitcell, parallel=parallel, nbatches=nbatches, lcell=lcell,
                                  output=None, output_name="nb", dtype=dtype, precision=precision)
        self.show_progress = show_progress
        self.index_base = index_base

    def update(self, **kw):
        self.sys.update(**kw)
        return self


def update(system, **kw):
    """update!(system; xpositions, ypositions, cutoff, unitcell, parallel) (src/API/updating.jl:165-187,
    src/API/neighborlist.jl:159-169)."""
    return system.update(**kw)


def neighborlist_(system: InPlaceNeighborList):
    """neighborlist!(system) (src/API/neighborlist.jl:217-231): returns (i, j, d) arrays."""
    return system.sys.run(NeighborList(system.index_base))


def neighborlist(*, xpositions=None, positions=None, ypositions=None, cutoff, unitcell=None, parallel: bool = True,
                 nbatches=(0, 0), lcell: int = 1, validate_coordinates=True, show_progress: bool = False,
                 dtype=None, precision: str = "exact", index_base: int = 0):
    """neighborlist(; xpositions, ypositions, cutoff, unitcell) (src/API/neighborlist.jl:314-340).
    Returns (i, j, d) numpy arrays; pair order is unspecified, as in the reference."""
    s = InPlaceNeighborList(xpositions=xpositions, positions=positions, ypositions=ypositions, cutoff=cutoff,
                            unitcell=unitcell, parallel=parallel, nbatches=nbatches, lcell=lcell, dtype=dtype,
                            precision=precision, index_base=index_base)
    try:
        return neighborlist_(s)
    finally:
        s.sys.close()


# ---------------------------------------------------------------------------- Box / CellList
class BatchedSystems:
    """Many independent periodic systems evaluated together: the loop
    ``for sys in systems: pairwise!(f, sys)`` of the reference (src/API/pairwise.jl:48-63) as one build and one
    launch per kernel for all systems, optionally replayed as a CUDA graph.

    positions: a list of (n_s, dim) arrays, or one (n_total, dim) array (numpy or a torch CUDA tensor) with
    ``offsets`` (n_sys + 1).  unitcells: (n_sys, dim) sides (orthorhombic) or (n_sys, dim, dim) matrices
    (triclinic, columns are the cell vectors).  A system whose cell fails the reference's check
    (Box.jl:243) gets status CLM_ERR_CELL_TOO_SMALL and NaN sums; the others are unaffected.
    """

    def __init__(self, *, positions, unitcells, cutoff, offsets=None, lcell: int = 1, dtype=None,
                 precision: str = "exact", graph: bool = False):
        uc = np.asarray(unitcells, dtype=np.float64)
        if uc.ndim not in (2, 3):
            raise ArgumentError("unitcells must be (nsys, dim) sides or (nsys, dim, dim) matrices")
        self.dim = uc.shape[1]
        if self.dim not in (2, 3) or (uc.ndim == 3 and uc.shape[2] != self.dim):
            raise ArgumentError("unit cells must be 2x2 or 3x3 (or 2 / 3 sides)")
        self.kind = _abi.CLM_ORTHO if uc.ndim == 2 else _abi.CLM_TRICLINIC
        self.dtype = _promote_dtype(uc, cutoff, dtype)
        if isinstance(positions, (list, tuple)):
            arrs = [np.asarray(a, dtype=self.dtype).reshape(-1, self.dim) for a in positions]
            sizes = [a.shape[0] for a in arrs]
            offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
            positions = np.concatenate(arrs) if arrs else np.zeros((0, self.dim), self.dtype)
        if offsets is None:
            raise ArgumentError("offsets are required with concatenated positions")
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self.nsys = len(self.offsets) - 1
        if uc.shape[0] != self.nsys:
            raise DimensionMismatch("one unit cell per system is required")
        self.cutoff = float(cutoff)
        L = _abi.load()
        h = C.c_void_p()
        st = L.clm_batched_create(_abi.CLM_F64 if self.dtype == np.float64 else _abi.CLM_F32, self.dim, C.byref(h))
        if st:
            _raise(None, st)
        self._handle = _Handle.__new__(_Handle)
        self._handle.h, self._handle.L = h, L
        # column-major cells per system (the ABI's layout)
        self._cells = np.ascontiguousarray(uc if uc.ndim == 2 else np.transpose(uc, (0, 2, 1)))
        self._handle.check(L.clm_batched_set_systems(h, self.nsys, self.offsets.ctypes.data, self._cells.ctypes.data,
                                                     self.kind, self.cutoff, int(lcell)))
        if precision != "exact":
            self.set_precision(precision)
        self.graph = graph
        self.update(positions=positions)

    @property
    def graph(self) -> bool:
        return self._graph

    @graph.setter
    def graph(self, on: bool):
        self._handle.check(self._handle.L.clm_batched_set_graph(self._handle.h, 1 if on else 0))
        self._graph = bool(on)

    def set_precision(self, precision: str):
        p = {"exact": _abi.CLM_PREC_EXACT, "split": _abi.CLM_PREC_SPLIT}[precision]
        self._handle.check(self._handle.L.clm_set_precision(self._handle.h, p))

    def set_config(self, lcell: int = 0, cell_split: int = 0, grid_div: int = 0):
        self._handle.check(self._handle.L.clm_batched_set_config(self._handle.h, lcell, cell_split, grid_div))

    def update(self, *, positions):
        arr, n, dev, keep = _as_positions(positions, self.dim, self.dtype)
        if n != int(self.offsets[-1]):
            raise DimensionMismatch("positions do not match the systems' offsets")
        ptr = arr.data_ptr() if hasattr(arr, "data_ptr") else arr.ctypes.data
        self._handle.check(self._handle.L.clm_set_positions(self._handle.h, 0, ptr if n else None, n, 1 if dev else 0))
        self._x, self.n = keep, n

    @staticmethod
    def _params(ops):
        arr = (_abi.OpParams * len(ops))()
        for k, op in enumerate(ops):
            p, _ = op.params(None) if not isinstance(op, (LennardJones,)) else (None, None)
            if isinstance(op, LennardJones):
                if op.types_x is not None:
                    raise ArgumentError("batches take no per-type tables")
                arr[k].p[0], arr[k].p[1], arr[k].p[2], arr[k].p[3] = float(op.eps), float(op.sigma), float(op.c12), \
                    float(op.c6)
            elif p is not None:
                arr[k] = p
        return arr

    def run(self, *ops):
        """One step with the given operators; returns one result per operator: per-system sums (numpy,
        NaN for a failed system), per-system counts for Count and NeighborList, and forces for the force
        operators (as EnergyAndForces with per-system energies)."""
        if not ops:
            raise ArgumentError("at least one operator")
        ids = np.array([_abi.OP[o.op] for o in ops], np.int32)
        params = self._params(ops)
        outs = (_abi.BatchOutputs * len(ops))()
        keep = []
        for k, op in enumerate(ops):
            sc = np.zeros(self.nsys, np.float64)
            ct = np.zeros(self.nsys, np.int64)
            outs[k].scalar, outs[k].count = sc.ctypes.data, ct.ctypes.data
            f = None
            if isinstance(op, _ForcesOp):
                f = np.zeros((self.n, self.dim), self.dtype)
                outs[k].forces = f.ctypes.data
            keep.append((sc, ct, f))
        self._handle.check(self._handle.L.clm_batched_run(self._handle.h, len(ops), ids.ctypes.data,
                                                          C.cast(params, C.c_void_p), C.cast(outs, C.c_void_p)))
        res = []
        for op, (sc, ct, f) in zip(ops, keep):
            if isinstance(op, NeighborList):
                res.append(BatchNeighborLists(self, ct, op.index_base))
            elif isinstance(op, Count):
                res.append(ct)
            elif f is not None:
                res.append(EnergyAndForces(sc, f))
            else:
                res.append(sc)
        return res

    def _neighbor_lists(self, base=0):
        """Per-system neighbour lists with indices local to each system (copied to the host)."""
        L, h = self._handle.L, self._handle.h
        n = C.c_int64()
        self._handle.check(L.clm_nl_count(h, C.byref(n)))
        i = np.empty(n.value, np.int64)
        j = np.empty(n.value, np.int64)
        d = np.empty(n.value, self.dtype)
        self._handle.check(L.clm_nl_fetch(h, i.ctypes.data, j.ctypes.data, d.ctypes.data, n.value, 0, 0))
        sysid = np.searchsorted(self.offsets, i, side="right") - 1
        order = np.argsort(sysid, kind="stable")
        i, j, d, sysid = i[order], j[order], d[order], sysid[order]
        bounds = np.concatenate([[0], np.cumsum(np.bincount(sysid, minlength=self.nsys))])
        out = []
        for s in range(self.nsys):
            a, b = bounds[s], bounds[s + 1]
            o = self.offsets[s]
            out.append((i[a:b] - o + base, j[a:b] - o + base, d[a:b]))
        return out

    def status(self):
        st = np.zeros(self.nsys, np.int32)
        self._handle.check(self._handle.L.clm_batched_status(self._handle.h, st.ctypes.data, self.nsys))
        return st

    def autotune(self, *ops, reps: int = 3):
        ids = np.array([_abi.OP[o.op] for o in ops], np.int32)
        params = self._params(ops)
        cfg = np.zeros(3, np.int32)
        best = C.c_float()
        self._handle.check(self._handle.L.clm_batched_autotune(self._handle.h, len(ops), ids.ctypes.data,
                                                               C.cast(params, C.c_void_p), reps, cfg.ctypes.data,
                                                               C.byref(best)))
        return {"lcell": int(cfg[0]), "cell_split": int(cfg[1]), "grid_div": int(cfg[2]), "step_ms": best.value}

    def last_step(self):
        ms, nl = C.c_float(), C.c_int64()
        self._handle.check(self._handle.L.clm_batched_last_step(self._handle.h, C.byref(ms), C.byref(nl)))
        return {"step_ms": ms.value, "launches": nl.value}

    def close(self):
        self._handle.close()


class BatchNeighborLists:
    """Neighbour lists of one batched step.  They stay on the device until a system's list is asked for
    (indexing copies all lists to the host once and splits them by system)."""

    def __init__(self, batch, counts, base):
        self._batch, self.counts, self._base, self._lists = batch, counts, base, None

    def __len__(self):
        return len(self.counts)

    def __getitem__(self, s):
        if self._lists is None:
            self._lists = self._batch._neighbor_lists(self._base)
        return self._lists[s]

    @property
    def total(self) -> int:
        return int(np.sum(self.counts))


class Box:
    """Mirror of `Box(unitcell, cutoff; lcell)` (src/internals/Box.jl:191-203, 330-335): the geometry as
    computed by the library (nc, cell_size, computing_box, aligned unit cell, rotation)."""

    def __init__(self, unitcell, cutoff, lcell: int = 1, dtype=None):
        dim = np.asarray(unitcell).shape[0]
        self.dtype = _promote_dtype(unitcell, cutoff, dtype)
        h = _Handle(self.dtype, dim, 1)
        kind, M = _cell_kind_and_matrix(unitcell, dim)
        Mf = np.ascontiguousarray(M.flatten(order="F"), dtype=np.float64)
        h.check(h.L.clm_set_box(h.h, Mf.ctypes.data_as(C.POINTER(C.c_double)), kind, float(cutoff), int(lcell)))
        self._fill(h, dim)
        self.unit_cell_type = {0: "OrthorhombicCell", 1: "TriclinicCell", 2: "NonPeriodicCell"}[kind]
        self.lcell = lcell
        self.input_unit_cell = M
        h.close()

    @classmethod
    def _from_handle(cls, h, dim):
        b = cls.__new__(cls)
        b._fill(h, dim)
        return b

    def _fill(self, h, dim):
        nc = np.zeros(3, np.int64)
        cs, lo, hi = np.zeros(3), np.zeros(3), np.zeros(3)
        al, R, Ri = np.zeros(9), np.zeros(9), np.zeros(9)
        cut = C.c_double()
        h.check(h.L.clm_get_box(h.h, nc.ctypes.data, cs.ctypes.data, lo.ctypes.data, hi.ctypes.data, al.ctypes.data,
                                R.ctypes.data, Ri.ctypes.data, C.byref(cut)))
        self.nc = nc[:dim].copy()
        self.cell_size = cs[:dim].copy()
        self.computing_box = (lo[:dim].copy(), hi[:dim].copy())
        self.aligned_unit_cell = al[:dim * dim].reshape(dim, dim, order="F")
        self.rotation = R[:dim * dim].reshape(dim, dim, order="F")
        self.inv_rotation = Ri[:dim * dim].reshape(dim, dim, order="F")
        self.cutoff = cut.value
        self.cutoff_sqr = cut.value * cut.value


def device_allocations():
    """(count, bytes) of the device and pinned allocations the library made in this process so far."""
    c, b = C.c_int64(), C.c_int64()
    _abi.load().clm_device_allocations(C.byref(c), C.byref(b))
    return c.value, b.value


def version() -> str:
    return _abi.load().clm_version().decode()
