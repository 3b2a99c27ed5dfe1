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
  * The float32 scan scheme and tile for the batch's shape come from the autotuner
    (``autotune.options_for``: the user's tuning cache, else the table tuned for this
    GPU and shipped with the package, else the library's built-in rule).
  * The float32 path with the backward from coordinates reuses one workspace per
    (device, stream, shape, options) instead of allocating and zeroing one per call:
    that backward reads only the workspace's status word, and the forward's chain
    records, which a later forward of the same shape rewrites, are not read by it.
"""
import math
import os
from collections import OrderedDict

import torch
from torch.autograd import Function
from torch.nn.modules.module import Module

from ... import autotune, load_extension

_ReducedModel = load_extension("_ReducedModel")

_WS_CACHE: "OrderedDict[tuple, torch.Tensor]" = OrderedDict()
_WS_CACHE_SIZE = 8


def _check_nan(t, ws, where):
    if os.environ.get("TPL_CHECK_NAN", "0") == "1":
        status = _ReducedModel.workspace_status(ws) if ws is not None else 0
        if status != 0:
            raise RuntimeError(f"Angles2BackboneFunction: {where}: device error {status}")
        if math.isnan(t.sum().item()):
            raise Exception(f"Angles2BackboneFunction: {where} Nan")


def new_workspace(batch, max_len, device, residues_per_thread=-1, threads_per_cta=-1):
    return torch.zeros(int(_ReducedModel.workspace_bytes(batch, max_len, residues_per_thread, threads_per_cta)),
                       dtype=torch.uint8, device=device)


def _shared_workspace(batch, max_len, device, fwd_opts):
    """A zeroed-once workspace per (device, current stream, shape, options), kept for
    reuse by later calls (at most _WS_CACHE_SIZE of them).  A graph being captured
    gets one of its own."""
    if torch.cuda.is_current_stream_capturing():
        return new_workspace(batch, max_len, device, *fwd_opts)
    key = (device.index, torch.cuda.current_stream(device).cuda_stream, batch, max_len) + tuple(fwd_opts)
    ws = _WS_CACHE.get(key)
    if ws is None:
        ws = new_workspace(batch, max_len, device, *fwd_opts)
        _WS_CACHE[key] = ws
        if len(_WS_CACHE) > _WS_CACHE_SIZE:
            _WS_CACHE.popitem(last=False)
    else:
        _WS_CACHE.move_to_end(key)
    return ws


class Angles2BackboneGPUFunction(Function):
    """Backbone angles -> backbone coordinates (CUDA, float32 or float64)."""

    backward_from_coords = True

    @staticmethod
    def forward(ctx, input_angles, angles_length):
        if input_angles.dim() != 3:
            raise Exception('Angles2BackboneFunction: ', 'Incorrect input size:', input_angles.size())
        input_angles = input_angles.contiguous()
        batch_size, _, max_len = input_angles.shape
        dev = input_angles.device
        coords = torch.empty(batch_size, 9 * max_len, dtype=input_angles.dtype, device=dev)
        f32 = input_angles.dtype == torch.float32
        tuned = autotune.options_for(dev, batch_size, max_len) if f32 and dev.type == "cuda" else None
        fwd_opts, bwd_opts = tuned if tuned is not None else ((-1, -1), (-1, -1, -1))
        ctx.from_coords = Angles2BackboneGPUFunction.backward_from_coords and f32
        if ctx.from_coords:
            ctx.A = _shared_workspace(batch_size, max_len, dev, fwd_opts)
        else:  # the recomputing backward reads the forward's chain records: a workspace of its own
            ctx.A = new_workspace(batch_size, max_len, dev, *fwd_opts)
        _ReducedModel.Angles2BackboneGPU_forward(input_angles, coords, angles_length, ctx.A, *fwd_opts)
        _check_nan(coords, ctx.A, "forward")
        ctx.fwd_opts, ctx.bwd_opts = fwd_opts, bwd_opts
        ctx.save_for_backward(input_angles, angles_length, coords if ctx.from_coords else None)
        return coords

    @staticmethod
    def backward(ctx, gradOutput):
        input_angles, angles_length, coords = ctx.saved_tensors
        gradOutput = gradOutput.contiguous()
        gradInput = torch.empty_like(input_angles)
        if ctx.from_coords:
            _ReducedModel.Angles2BackboneGPU_backward_coords(gradInput, gradOutput, coords, angles_length, ctx.A,
                                                             *ctx.bwd_opts)
        else:
            _ReducedModel.Angles2BackboneGPU_backward(gradInput, gradOutput, input_angles, angles_length, ctx.A,
                                                      gradInput.new_empty(0), *ctx.fwd_opts)
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
        if (input.dtype != torch.float32 or input.dim() != 3 or not Angles2BackboneGPUFunction.backward_from_coords
                or os.environ.get("TPL_CHECK_NAN", "0") == "1"):
            return Angles2BackboneGPUFunction.apply(input, angles_length)
        # the float32 path of Angles2BackboneGPUFunction (the same kernels, options and
        # shared workspace) through the extension's C++ autograd function: no Python
        # frame in the backward
        batch_size, _, max_len = input.shape
        dev = input.device
        tuned = autotune.options_for(dev, batch_size, max_len)
        fwd_opts, bwd_opts = tuned if tuned is not None else ((-1, -1), (-1, -1, -1))
        ws = _shared_workspace(batch_size, max_len, dev, fwd_opts)
        return _ReducedModel.angles2backbone_autograd(input, angles_length, ws, list(fwd_opts), list(bwd_opts))
