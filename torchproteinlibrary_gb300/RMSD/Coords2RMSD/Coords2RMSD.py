"""Coords2RMSD layer: least RMSD after optimal superposition, per chain.

Mirrors TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py:12-78:
``Coords2RMSD()(input [B, 3N], target [B, 3N], num_atoms int32 [B]) -> rmsd [B]``
(the module keeps the optimal transposed rotation in ``self.UT``), and
``Coords2RMSDFunction.apply(centered_input, centered_target, num_atoms) -> (rmsd, UT)``.
The gradient flows to the input only, dL/dx = g (x - UT y) / (rmsd N).

Differences from the reference: CUDA tensors only (float32 or float64); the module
folds the centring (Coords2Center + CoordsTranslate in the reference) into the
same launch; the eigen solve runs on the GPU; the backward is one kernel instead
of a Python loop with .item() per chain; the NaN check runs only with
TPL_CHECK_NAN=1.
"""
import math
import os

import torch
from torch.autograd import Function
from torch.nn.modules.module import Module

from ... import load_extension

_RMSD = load_extension("_RMSD")


def _na(num_atoms, device):
    """num_atoms as int32 on `device`.  A host tensor's device copy is kept on the
    tensor itself and reused while the tensor is unchanged (its version counter), so
    repeated calls with the same counts make no host-to-device copy."""
    if num_atoms.device == device:
        return num_atoms.to(dtype=torch.int32).contiguous()
    hit = getattr(num_atoms, "_tpl_on_device", None)
    if hit is not None and hit[0] == num_atoms._version and hit[1].device == device:
        return hit[1]
    na = num_atoms.to(device=device, dtype=torch.int32).contiguous()
    if not torch.cuda.is_current_stream_capturing():
        num_atoms._tpl_on_device = (num_atoms._version, na)
    return na


def _check(t, where):
    if os.environ.get("TPL_CHECK_NAN", "0") == "1" and math.isnan(t.sum().item()):
        raise Exception(f"Coords2RMSDFunction: {where} Nan")


class Coords2RMSDFunction(Function):
    """Protein coords, target coords -> rmsd function (inputs already centred)."""

    @staticmethod
    def forward(ctx, centered_input, centered_target, num_atoms):
        if centered_input.dim() != 2:
            raise ValueError('Coords2RMSDFunction: ', 'Incorrect input size:', centered_input.size())
        if not centered_input.is_cuda:
            raise RuntimeError("Coords2RMSD: this build has no CPU path; move the tensors to a CUDA device")
        x = centered_input.contiguous()
        y = centered_target.contiguous()
        na = _na(num_atoms, x.device)
        B = x.size(0)
        output = torch.empty(B, dtype=x.dtype, device=x.device)
        UT = torch.empty(B, 3, 3, dtype=x.dtype, device=x.device)
        _RMSD.Coords2RMSDGPU_forward(x, y, output, na, UT)
        _check(output, "forward")
        ctx.save_for_backward(output, na, UT, x, y)
        ctx.mark_non_differentiable(UT)
        return output, UT

    @staticmethod
    def backward(ctx, gradRMSD, gradUT):
        output, na, UT, x, y = ctx.saved_tensors
        grad = torch.empty_like(x)
        _RMSD.Coords2RMSDGPU_backward(gradRMSD.contiguous(), x, y, na, output, UT, x.new_empty(0, dtype=torch.double),
                                      grad, 0)
        _check(grad, "backward")
        return grad, None, None


class _Coords2RMSDCentering(Function):
    """Same with the centring of both sets folded into the kernels."""

    @staticmethod
    def forward(ctx, input, target, num_atoms):
        x = input.contiguous()
        y = target.contiguous()
        na = _na(num_atoms, x.device)
        B = x.size(0)
        output = torch.empty(B, dtype=x.dtype, device=x.device)
        UT = torch.empty(B, 3, 3, dtype=x.dtype, device=x.device)
        cent = torch.empty(B, 6, dtype=torch.float64, device=x.device)
        _RMSD.Coords2RMSDGPU_forward_centering(x, y, output, na, UT, cent)
        _check(output, "forward")
        ctx.save_for_backward(output, na, UT, x, y, cent)
        ctx.mark_non_differentiable(UT)
        return output, UT

    @staticmethod
    def backward(ctx, gradRMSD, gradUT):
        output, na, UT, x, y, cent = ctx.saved_tensors
        grad = torch.empty_like(x)
        _RMSD.Coords2RMSDGPU_backward(gradRMSD.contiguous(), x, y, na, output, UT, cent, grad, 1)
        _check(grad, "backward")
        return grad, None, None


class Coords2RMSD(Module):
    def __init__(self):
        super(Coords2RMSD, self).__init__()
        self.UT = None

    def forward(self, input, target, num_atoms):
        if not input.is_cuda:
            raise RuntimeError("Coords2RMSD: this build has no CPU path; move the tensors to a CUDA device")
        if os.environ.get("TPL_CHECK_NAN", "0") == "1":
            rmsd, self.UT = _Coords2RMSDCentering.apply(input, target, num_atoms)
            return rmsd
        # the same entries as _Coords2RMSDCentering through the extension's C++ autograd
        # function: no Python frame in the backward
        rmsd, self.UT = _RMSD.coords2rmsd_autograd(input, target, _na(num_atoms, input.device))
        return rmsd
