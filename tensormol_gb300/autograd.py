"""The fused energy/force path behind a ``torch.autograd.Function``.

``FusedEnergy.apply(x, system)`` returns the per-molecule total energies
(Hartree) of positions ``x`` (CUDA float64 [N, 3], Angstrom). When ``x``
needs a gradient, the forward call runs the whole fused evaluation once
(neighbour lists, descriptors, both networks forward and backward, pair terms,
the descriptor adjoint), so the gradient is already known when ``backward`` is
called; otherwise (``x`` without ``requires_grad``, or under
``torch.no_grad()``) it runs the energy alone (the DoForce=False evaluation,
no adjoint). ``backward`` returns
dE/dx = -F / JOULEPERHARTREE, weighted per molecule by the incoming gradient.
This is the hand-written adjoint standing in for ``tf.gradients(Etotal,
xyzs)`` (TFNetworks/TFBehlerParinelloSymEE.py:1490). Second derivatives are
not available.
"""
from __future__ import annotations

import torch

from . import _lib
from .params import JOULEPERHARTREE


class FusedEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, system):
        if x.device.type != "cuda" or x.dtype != torch.float64 or tuple(x.shape) != (system.N, 3):
            raise ValueError("x must be a CUDA float64 tensor of shape [natoms, 3]")
        x = x.contiguous()
        lib_stream = torch.cuda.ExternalStream(int(system.ctx.stream or 0), device=x.device)
        cur = torch.cuda.current_stream(x.device)
        need_force = bool(ctx.needs_input_grad[0])
        E = torch.empty((system.nmol, 4), dtype=torch.float64, device=x.device)
        F = torch.empty((system.N, 3) if need_force else (0, 3), dtype=torch.float64, device=x.device)
        lib_stream.wait_stream(cur)            # x is ready before the library reads it
        system.energy_force_device(x.data_ptr(), E.data_ptr(), F.data_ptr() if need_force else 0,
                                   flags=0 if need_force else _lib.TM_F_ENERGY_ONLY)
        cur.wait_stream(lib_stream)            # E, F are ready before torch reads them
        E.record_stream(cur)
        F.record_stream(cur)
        mol = getattr(system, "_mol_index", None)
        if mol is None or mol.device != x.device:
            counts = torch.as_tensor(system.offsets[1:] - system.offsets[:-1])
            mol = torch.repeat_interleave(torch.arange(system.nmol), counts).to(x.device)
            system._mol_index = mol
        ctx.save_for_backward(F, mol)
        return E[:, 0].clone()

    @staticmethod
    def backward(ctx, gE):
        if ctx.needs_input_grad[0] and torch.is_grad_enabled():
            raise RuntimeError("FusedEnergy provides first derivatives only")
        F, mol = ctx.saved_tensors
        g = (-F / JOULEPERHARTREE) * gE[mol][:, None]
        return g, None


def energy(system, x):
    """Per-molecule total energy with a gradient from the fused adjoint."""
    return FusedEnergy.apply(x, system)
