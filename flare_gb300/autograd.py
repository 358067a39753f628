"""torch.autograd.Function over the fused prediction pipeline.

``SGPEnergy.apply(positions, sgp, structures)`` returns the per-structure
energies as a differentiable function of the (N, 3) FP64 CUDA positions
tensor.  The forward runs fgb_predict (energy, forces, stress); the forces
come from the library's hand-written reverse-mode adjoint (dE/dB2 -> dE/dA
-> per-pair dE/dr with recomputed radial and Y_lm terms), so the backward
is dE/dr_i = -F_i scaled by the incoming energy gradient — no torch
autograd graph is built through the descriptor.
"""
import numpy as np
import torch

from . import _lib
from .core import _prec, get_precision, pack_structures


class SGPEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, sgp, structures, precision=None):
        if not positions.is_cuda or positions.dtype != torch.float64:
            raise ValueError("positions must be a float64 CUDA tensor")
        positions = positions.contiguous()
        offsets, cells, _, sp = pack_structures(structures)
        N = int(offsets[-1])
        if positions.shape != (N, 3):
            raise ValueError("positions must be (N, 3) for the packed batch")
        m = sgp._device_model(structures[0].descriptor_calculators)
        S = len(structures)
        dev = positions.device
        d_sp = torch.from_numpy(sp).to(dev)
        e = torch.zeros(S, dtype=torch.float64, device=dev)
        f = torch.zeros((max(N, 1), 3), dtype=torch.float64, device=dev)
        st = torch.zeros((S, 6), dtype=torch.float64, device=dev)
        prec = _prec[precision or get_precision()]
        _lib.check(_lib.lib().fgb_predict(
            m.h, S, _lib.ptr(offsets), _lib.ptr(cells), _lib.ptr(positions),
            _lib.ptr(d_sp), structures[0].cutoff,
            _lib.FGB_WANT_ENERGY | _lib.FGB_WANT_FORCES | _lib.FGB_WANT_STRESS,
            prec, _lib.ptr(e), _lib.ptr(f), _lib.ptr(st), None,
            _lib.stream_ptr()), "SGPEnergy")
        owner = torch.from_numpy(np.repeat(np.arange(S), np.diff(offsets))).to(dev)
        ctx.save_for_backward(f[:N], owner)
        ctx.stress = st
        return e

    @staticmethod
    def backward(ctx, grad_e):
        forces, owner = ctx.saved_tensors
        grad_pos = -forces * grad_e[owner].unsqueeze(1)
        return grad_pos, None, None, None


def energy(positions, sgp, structures, precision=None):
    """Differentiable per-structure energies (see SGPEnergy)."""
    return SGPEnergy.apply(positions, sgp, structures, precision)
