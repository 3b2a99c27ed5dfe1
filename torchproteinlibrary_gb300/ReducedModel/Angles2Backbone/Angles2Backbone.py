"""Angles2Backbone layer: backbone dihedrals -> N, CA, C coordinates.

Mirrors TorchProteinLibrary/ReducedModel/Angles2Backbone/Angles2Backbone.py:8-104:
``Angles2Backbone()(angles [B,3,L], lengths int32 [B]) -> coords [B, 9L]`` (N, CA, C
xyz per residue, zero past each chain's length), with a backward returning
dL/dangles [B,3,L].

Differences from the reference:
  * CUDA only.  float32 angles run the batched FP32 kernels; float64 angles run the
    plain FP64 form.  (The reference runs float32 on CUDA and float64 on the CPU.)
    CPU tensors raise RuntimeError; there is no CPU fallback.
  * ``ctx.A`` is a small workspace (per-tile carries), not the [B, 48L] frame
    buffer, and no [B, 3, 27L^2] ``dr_dangle`` is allocated.
  * The NaN check that forces a host sync after every call
    (Angles2Backbone.py:27,49 in the reference) runs only when the environment
    variable TPL_CHECK_NAN=1; it also reads back device-detected errors.
  * dL/domega of each chain's last residue is 0 (the reference reads one matrix
    past the chain there).
  * The float32 backward works from the coordinates the forward returned (saved
    for backward, as the reference saves its frame buffer ``A``), so it does not
    walk the chain again.  Set ``Angles2BackboneGPUFunction.backward_from_coords``
    to False to recompute from the angles instead.
"""
import math
import os

import torch
from torch.autograd import Function
from torch.nn.modules.module import Module

from ... import load_extension

_ReducedModel = load_extension("_ReducedModel")


def _check_nan(t, ws, where):
    if os.environ.get("TPL_CHECK_NAN", "0") == "1":
        status = _ReducedModel.workspace_status(ws) if ws is not None else 0
        if status != 0:
            raise RuntimeError(f"Angles2BackboneFunction: {where}: device error {status}")
        if math.isnan(t.sum().item()):
            raise Exception(f"Angles2BackboneFunction: {where} Nan")


def new_workspace(batch, max_len, device):
    return torch.zeros(int(_ReducedModel.workspace_bytes(batch, max_len)), dtype=torch.uint8, device=device)


class Angles2BackboneGPUFunction(Function):
    """Backbone angles -> backbone coordinates (CUDA, float32 or float64)."""

    backward_from_coords = True

    @staticmethod
    def forward(ctx, input_angles, angles_length):
        if input_angles.dim() != 3:
            raise Exception('Angles2BackboneFunction: ', 'Incorrect input size:', input_angles.size())
        input_angles = input_angles.contiguous()
        batch_size, _, max_len = input_angles.shape
        coords = torch.empty(batch_size, 9 * max_len, dtype=input_angles.dtype, device=input_angles.device)
        ctx.A = new_workspace(batch_size, max_len, input_angles.device)
        _ReducedModel.Angles2BackboneGPU_forward(input_angles, coords, angles_length, ctx.A)
        _check_nan(coords, ctx.A, "forward")
        ctx.from_coords = (Angles2BackboneGPUFunction.backward_from_coords and
                           input_angles.dtype == torch.float32)
        ctx.save_for_backward(input_angles, angles_length, coords if ctx.from_coords else None)
        return coords

    @staticmethod
    def backward(ctx, gradOutput):
        input_angles, angles_length, coords = ctx.saved_tensors
        gradOutput = gradOutput.contiguous()
        gradInput = torch.empty_like(input_angles)
        if ctx.from_coords:
            _ReducedModel.Angles2BackboneGPU_backward_coords(gradInput, gradOutput, coords, angles_length, ctx.A)
        else:
            _ReducedModel.Angles2BackboneGPU_backward(gradInput, gradOutput, input_angles, angles_length, ctx.A,
                                                      gradInput.new_empty(0))
        _check_nan(gradInput, ctx.A, "backward")
        return gradInput, None


class Angles2BackboneCPUFunction(Function):
    """The reference's float64 CPU function, kept under its name so that code
    importing it still loads.  This build has no CPU path: calling it raises, as
    ``_ReducedModel.Angles2BackboneCPU_forward`` does.  Run float64 angles on a
    CUDA device through ``Angles2BackboneGPUFunction`` instead."""

    @staticmethod
    def forward(ctx, input, angles_length):
        raise RuntimeError("Angles2BackboneCPUFunction: this build has no CPU path; "
                           "move the tensors to a CUDA device")

    @staticmethod
    def backward(ctx, gradOutput):  # pragma: no cover - forward never succeeds
        raise RuntimeError("Angles2BackboneCPUFunction: this build has no CPU path")


class Angles2Backbone(Module):
    def __init__(self):
        super(Angles2Backbone, self).__init__()

    def forward(self, input, angles_length):
        if not input.is_cuda:
            raise RuntimeError("Angles2Backbone: this build has no CPU path; move the tensors to a CUDA device")
        return Angles2BackboneGPUFunction.apply(input, angles_length)
