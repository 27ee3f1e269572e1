"""ctypes front end of the CPU oracle (``oracle/clm_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg, to check results and to time the CPU baseline.  The shipped
package never imports this module.

The oracle restates CellListMap.jl's serial cell-list build and pair map
(``src/internals/CellLists.jl:940-1057``, ``src/internals/self.jl:106-184``,
``src/internals/cross.jl:81-129``, ``src/internals/vicinal_cells.jl:4-75``)
and its naive O(N^2) check (``test/modules/Testing.jl:62-104``).
Indices are 0-based here.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libclm_oracle.so")

KIND = {"ortho": 0, "orthorhombic": 0, "tri": 1, "triclinic": 1, "nonperiodic": 2, "none": 2}
OPS = {
    "nl": 1, "count": 2, "sum_d2": 3, "sum_d": 4, "sum_inv_d": 5,
    "soft_energy": 6, "soft_forces": 7, "lj_energy": 8, "lj_forces": 9,
    "mindist": 10, "rhist": 11, "inv_d_forces": 12, "lj_adjoint": 13, "weighted_inv_d": 14,
}
ERRORS = {1: "invalid argument", 2: "unit cell too small for cutoff", 3: "invalid (NaN) coordinates",
          4: "dimension mismatch", 6: "capacity", 10: "lcell must be >= 1"}


class OracleError(RuntimeError):
    def __init__(self, code):
        super().__init__(f"oracle status {code}: {ERRORS.get(code, '?')}")
        self.code = code


class _Spec(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("dim", C.c_int32), ("kind", C.c_int32), ("lcell", C.c_int32),
                ("cutoff", C.c_double), ("M", C.c_double * 9)]


class _BoxInfo(C.Structure):
    _fields_ = [("nc", C.c_int64 * 3), ("cell_size", C.c_double * 3), ("cbmin", C.c_double * 3),
                ("cbmax", C.c_double * 3), ("origin", C.c_double * 3), ("Min", C.c_double * 9),
                ("Mal", C.c_double * 9), ("R", C.c_double * 9), ("Rinv", C.c_double * 9),
                ("cutoff", C.c_double), ("cutoff_sqr", C.c_double)]


class _Op(C.Structure):
    _fields_ = [("op", C.c_int32), ("nthreads", C.c_int32), ("compensated", C.c_int32), ("ntypes", C.c_int32),
                ("types_x", C.c_void_p), ("types_y", C.c_void_p), ("p", C.c_double * 8),
                ("eps_table", C.c_void_p), ("sig_table", C.c_void_p), ("vel_x", C.c_void_p),
                ("vel_y", C.c_void_p), ("bins", C.c_void_p), ("nbins", C.c_int32), ("pad_", C.c_int32),
                ("weights_x", C.c_void_p), ("weights_y", C.c_void_p)]


class _Result(C.Structure):
    _fields_ = [("nl_cap", C.c_int64), ("nl_n", C.c_int64), ("nl_i", C.c_void_p), ("nl_j", C.c_void_p),
                ("nl_d", C.c_void_p), ("scalar", C.c_double), ("count", C.c_int64), ("forces_x", C.c_void_p),
                ("forces_y", C.c_void_p), ("min_i", C.c_int64), ("min_j", C.c_int64), ("min_d", C.c_double),
                ("hist_count", C.c_void_p), ("hist_sum", C.c_void_p), ("adj", C.c_double * 32)]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -ffp-contract=off -fopenmp)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "clm_oracle.cpp")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        for name in ("orc_map", "orc_naive"):
            fn = getattr(L, name)
            fn.argtypes = [C.POINTER(_Spec), C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.POINTER(_Op),
                           C.POINTER(_Result)]
            fn.restype = C.c_int
        L.orc_box.argtypes = [C.POINTER(_Spec), C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.POINTER(_BoxInfo)]
        L.orc_box.restype = C.c_int
        L.orc_celllist.argtypes = [C.POINTER(_Spec), C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64), C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_celllist.restype = C.c_int
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def max_threads() -> int:
    return int(lib().orc_max_threads())


def _spec(dtype, dim, kind, M, cutoff, lcell):
    s = _Spec()
    s.dtype = 1 if np.dtype(dtype) == np.float64 else 0
    s.dim = dim
    s.kind = KIND[kind] if isinstance(kind, str) else int(kind)
    s.lcell = int(lcell)
    s.cutoff = float(cutoff)
    if M is not None:
        Mm = np.asarray(M, dtype=np.float64)
        if Mm.ndim == 1:
            Mm = np.diag(Mm)
        flat = Mm.reshape(dim, dim).flatten(order="F")
        for k in range(dim * dim):
            s.M[k] = float(flat[k])
    return s


def _pos(x, dtype, dim):
    if x is None:
        return None, 0
    a = np.ascontiguousarray(np.asarray(x, dtype=dtype).reshape(-1, dim))
    return a, a.shape[0]


def box_info(x=None, y=None, *, dim=3, kind="ortho", unitcell=None, cutoff, lcell=1, dtype=np.float64):
    s = _spec(dtype, dim, kind, unitcell, cutoff, lcell)
    xa, nx = _pos(x, dtype, dim)
    ya, ny = _pos(y, dtype, dim)
    out = _BoxInfo()
    st = lib().orc_box(C.byref(s), None if xa is None else xa.ctypes.data, nx,
                       None if ya is None else ya.ctypes.data, ny, C.byref(out))
    if st:
        raise OracleError(st)
    n = dim
    return {
        "nc": np.array(out.nc[:n], dtype=np.int64),
        "cell_size": np.array(out.cell_size[:n]),
        "computing_box": (np.array(out.cbmin[:n]), np.array(out.cbmax[:n])),
        "origin": np.array(out.origin[:n]),
        "input_unit_cell": np.array(out.Min[:n * n]).reshape(n, n, order="F"),
        "aligned_unit_cell": np.array(out.Mal[:n * n]).reshape(n, n, order="F"),
        "rotation": np.array(out.R[:n * n]).reshape(n, n, order="F"),
        "inv_rotation": np.array(out.Rinv[:n * n]).reshape(n, n, order="F"),
        "cutoff": out.cutoff, "cutoff_sqr": out.cutoff_sqr,
    }


def celllist(x, *, dim=3, kind="ortho", unitcell=None, cutoff, lcell=1, dtype=np.float64):
    """Serial cell list: copies sorted by (cell linear index, in-cell order of the reference)."""
    s = _spec(dtype, dim, kind, unitcell, cutoff, lcell)
    xa, nx = _pos(x, dtype, dim)
    ncopy = C.c_int64(0)
    nreal = C.c_int64(0)
    st = lib().orc_celllist(C.byref(s), xa.ctypes.data, nx, C.byref(ncopy), C.byref(nreal), 0, None, None, None, None)
    if st:
        raise OracleError(st)
    n = ncopy.value
    cell = np.zeros(n, np.int64)
    idx = np.zeros(n, np.int64)
    real = np.zeros(n, np.int8)
    coords = np.zeros((n, dim), np.float64)
    st = lib().orc_celllist(C.byref(s), xa.ctypes.data, nx, C.byref(ncopy), C.byref(nreal), n, cell.ctypes.data,
                            idx.ctypes.data, real.ctypes.data, coords.ctypes.data)
    if st:
        raise OracleError(st)
    return {"cell": cell, "index": idx, "real": real.astype(bool), "coords": coords,
            "n_cells_with_real": nreal.value}


def run(op, x, y=None, *, dim=3, kind="ortho", unitcell=None, cutoff, lcell=1, dtype=np.float64,
        params=(), types_x=None, types_y=None, eps_table=None, sig_table=None, vel_x=None, vel_y=None,
        bins=None, nthreads=1, compensated=True, naive=False, nl_cap=None, weights_x=None, weights_y=None):
    """Run one operator over all pairs within the cutoff; returns a dict of outputs."""
    s = _spec(dtype, dim, kind, unitcell, cutoff, lcell)
    xa, nx = _pos(x, dtype, dim)
    ya, ny = _pos(y, dtype, dim)
    o = _Op()
    o.op = OPS[op] if isinstance(op, str) else int(op)
    o.nthreads = int(nthreads)
    o.compensated = 1 if compensated else 0
    keep = []
    p = list(params)
    if o.op in (OPS["soft_energy"], OPS["soft_forces"]) and not p:
        p = [float(cutoff)]
    for k, v in enumerate(p):
        o.p[k] = float(v)
    if types_x is not None:
        tx = np.ascontiguousarray(types_x, dtype=np.int32)
        keep.append(tx)
        o.types_x = tx.ctypes.data
        et = np.ascontiguousarray(eps_table, dtype=np.float64)
        stb = np.ascontiguousarray(sig_table, dtype=np.float64)
        keep += [et, stb]
        o.ntypes = et.shape[0]
        o.eps_table = et.ctypes.data
        o.sig_table = stb.ctypes.data
        if types_y is not None:
            ty = np.ascontiguousarray(types_y, dtype=np.int32)
            keep.append(ty)
            o.types_y = ty.ctypes.data
    if vel_x is not None:
        vx = np.ascontiguousarray(vel_x, dtype=np.float64).reshape(-1, dim)
        keep.append(vx)
        o.vel_x = vx.ctypes.data
        if vel_y is not None:
            vy = np.ascontiguousarray(vel_y, dtype=np.float64).reshape(-1, dim)
            keep.append(vy)
            o.vel_y = vy.ctypes.data
    if weights_x is not None:
        wx = np.ascontiguousarray(weights_x, dtype=np.float64).reshape(-1)
        keep.append(wx)
        o.weights_x = wx.ctypes.data
        if weights_y is not None:
            wy = np.ascontiguousarray(weights_y, dtype=np.float64).reshape(-1)
            keep.append(wy)
            o.weights_y = wy.ctypes.data
    if bins is not None:
        b = np.ascontiguousarray(bins, dtype=np.float64)
        keep.append(b)
        o.bins = b.ctypes.data
        o.nbins = b.shape[0] - 1
    r = _Result()
    out = {}
    if o.op == OPS["nl"]:
        cap = nl_cap if nl_cap is not None else 1024
        while True:
            ni = np.zeros(cap, np.int64)
            nj = np.zeros(cap, np.int64)
            nd = np.zeros(cap, np.float64)
            r.nl_cap = cap
            r.nl_i, r.nl_j, r.nl_d = ni.ctypes.data, nj.ctypes.data, nd.ctypes.data
            fn = lib().orc_naive if naive else lib().orc_map
            st = fn(C.byref(s), xa.ctypes.data, nx, None if ya is None else ya.ctypes.data, ny, C.byref(o), C.byref(r))
            if st == 6 and nl_cap is None:
                cap = r.nl_n
                continue
            if st:
                raise OracleError(st)
            n = r.nl_n
            return {"i": ni[:n].copy(), "j": nj[:n].copy(), "d": nd[:n].copy()}
    fx = fy = hc = hs = None
    if o.op in (OPS["soft_forces"], OPS["lj_forces"], OPS["inv_d_forces"], OPS["lj_adjoint"], OPS["weighted_inv_d"]):
        fx = np.zeros((nx, dim), np.float64)
        r.forces_x = fx.ctypes.data
        if ya is not None:
            fy = np.zeros((ny, dim), np.float64)
            r.forces_y = fy.ctypes.data
    if o.op == OPS["rhist"]:
        hc = np.zeros(o.nbins, np.int64)
        hs = np.zeros(o.nbins, np.float64)
        r.hist_count, r.hist_sum = hc.ctypes.data, hs.ctypes.data
    fn = lib().orc_naive if naive else lib().orc_map
    st = fn(C.byref(s), xa.ctypes.data, nx, None if ya is None else ya.ctypes.data, ny, C.byref(o), C.byref(r))
    if st:
        raise OracleError(st)
    out["scalar"] = r.scalar
    out["count"] = r.count
    if fx is not None:
        out["forces_x"] = fx
        if fy is not None:
            out["forces_y"] = fy
    if o.op == OPS["mindist"]:
        out["min"] = (r.min_i, r.min_j, r.min_d)
    if o.op == OPS["lj_adjoint"]:
        nt = o.ntypes
        ncls = nt * (nt + 1) // 2 if nt > 0 else 1
        out["virial"] = np.array(r.adj[:9]).reshape(3, 3)[:dim, :dim].copy()
        out["deps"] = np.array(r.adj[9:9 + ncls])
        out["dsig"] = np.array(r.adj[12:12 + ncls])
    if hc is not None:
        out["hist_count"], out["hist_sum"] = hc, hs
    return out


def canonical_pairs(i, j, d=None):
    """Sort an unordered pair list by (min(i,j), max(i,j)); returns arrays."""
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    a = np.minimum(i, j)
    b = np.maximum(i, j)
    order = np.lexsort((b, a))
    if d is None:
        return a[order], b[order]
    return a[order], b[order], np.asarray(d)[order]
