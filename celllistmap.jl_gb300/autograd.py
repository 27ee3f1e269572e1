"""The LJ energy as a differentiable function for torch autograd, backed by the adjoint operator.

This is the runnable counterpart of the ChainRulesCore ``rrule`` that a Julia package extension would
define for the GPU energy (the reference differentiates its map with ForwardDiff dual numbers,
test/examples/generic_types.jl:10-20,102): one forward call computes the energy, the forces, the virial
and the per-type parameter derivatives; the backward pass scales them by the incoming gradient.

    U = lj_energy(x, cell, eps_table, sig_table, types, cutoff)
    U.backward()   # x.grad = dU/dx, cell.grad = dU/dM (scaled coordinates fixed), eps/sig tables' grads

`cell` is the (dim, dim) unit-cell matrix (columns are the cell vectors) or (dim,) sides.  Gradients
are returned on the inputs' devices and dtypes.
"""
from __future__ import annotations

import numpy as np

from . import api


def _lj_function():
    import torch

    class LJEnergy(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, cell, eps_table, sig_table, types, cutoff, c12, c6):
            dt = np.float64 if x.dtype == torch.float64 else np.float32
            xn = x.detach().cpu().numpy().astype(dt, copy=False)
            cn = cell.detach().cpu().numpy().astype(np.float64)
            tn = types.detach().cpu().numpy().astype(np.int32)
            en = eps_table.detach().cpu().numpy().astype(np.float64)
            sn = sig_table.detach().cpu().numpy().astype(np.float64)
            op = api.LennardJonesAdjoint(c12=c12, c6=c6, types_x=tn, eps_table=en, sig_table=sn)
            system = api.ParticleSystem(positions=xn, unitcell=cn, cutoff=float(cutoff), dtype=dt)
            try:
                r = api.pairwise(op, system)
            finally:
                system.close()
            dim = xn.shape[1]
            M = np.diag(cn) if cn.ndim == 1 else cn
            dU_dM = r.virial @ np.linalg.inv(M).T
            dU_dcell = np.diag(dU_dM).copy() if cn.ndim == 1 else dU_dM
            ctx.save_for_backward(
                torch.as_tensor(-np.asarray(r.forces, np.float64).reshape(-1, dim), dtype=x.dtype, device=x.device),
                torch.as_tensor(dU_dcell, dtype=cell.dtype, device=cell.device),
                torch.as_tensor(np.asarray(r.dU_deps), dtype=eps_table.dtype, device=eps_table.device),
                torch.as_tensor(np.asarray(r.dU_dsigma), dtype=sig_table.dtype, device=sig_table.device))
            return torch.tensor(float(r.energy), dtype=torch.float64, device=x.device)

        @staticmethod
        def backward(ctx, gU):
            gx, gcell, geps, gsig = ctx.saved_tensors
            # the tables are symmetric: a parameter of the pair class (a, b) is shared by both entries,
            # so the derivative per entry is half the class derivative off the diagonal
            half = torch.full_like(geps, 0.5)
            half.fill_diagonal_(1.0)
            return (gU * gx, gU * gcell, gU * geps * half, gU * gsig * half, None, None, None, None)

    return LJEnergy


_FN = None


def lj_energy(x, cell, eps_table, sig_table, types, cutoff, c12=4.0, c6=4.0):
    """Differentiable LJ energy of one periodic system with per-type tables (at most 2 types)."""
    global _FN
    if _FN is None:
        _FN = _lj_function()
    return _FN.apply(x, cell, eps_table, sig_table, types, cutoff, c12, c6)
