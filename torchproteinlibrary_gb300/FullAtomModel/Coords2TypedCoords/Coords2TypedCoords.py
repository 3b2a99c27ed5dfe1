"""Coords2TypedCoords: coordinates regrouped by the 11 atom types.

Mirrors TorchProteinLibrary/FullAtomModel/Coords2TypedCoords/Coords2TypedCoords.py:
``Coords2TypedCoords()(coords [B, 3N], res_names u8 [B, N, 4], atom_names u8 [B, N, 4],
num_atoms int32 [B]) -> (typed_coords [B, 3 max(num_atoms)], num_atoms_of_type
int32 [B, 11], offsets int32 [B, 11])``: the atoms of type k (ProtUtil::get11AtomType,
Math/nUtil.cpp:567-703) sit at slots offsets[b, k] .. offsets[b, k] +
num_atoms_of_type[b, k] - 1 in their input order.  The backward scatters the
gradient back to the input atoms.

Differences from the reference: CUDA tensors only (the reference is CPU only);
names and num_atoms are moved to the coordinates' device; the index map
``ctx.atom_indexes`` stays on the device; an unknown (residue, atom) pair is
reported through the status word (RuntimeError when TPL_CHECK_NAN=1, where the
reference throws); the gradient has the input's shape.
"""
import math
import os

import torch
from torch.autograd import Function
from torch.nn.modules.module import Module

from ... import load_extension

_FullAtomModel = load_extension("_FullAtomModel")

__all__ = ["Coords2TypedCoordsFunction", "Coords2TypedCoords"]

NUM_ATOM_TYPES = 11


def _check(t, what, device):
    if os.environ.get("TPL_CHECK_NAN", "0") == "1":
        status = _FullAtomModel.workspace_status(device.index if device.index is not None else 0)
        if status != 0:
            raise RuntimeError(f"Coords2TypedCoordsFunction: {what}: device error {status}")
        if math.isnan(t.sum().item()):
            raise Exception(f"Coords2TypedCoordsFunction: {what} Nan")


class Coords2TypedCoordsFunction(Function):
    """coordinates -> coordinates arranged in atom types function"""

    @staticmethod
    def forward(ctx, input_coords, input_resnames, input_atomnames, num_atoms):
        if input_coords.dim() != 2:
            raise ValueError('Coords2TypedCoordsFunction: ', 'Incorrect input size:', input_coords.size())
        if not input_coords.is_cuda:
            raise RuntimeError("Coords2TypedCoords: this build has no CPU path; move the tensors to a CUDA device")
        x = input_coords.contiguous()
        dev = x.device
        max_num_atoms = getattr(num_atoms, "_tpl_max_atoms", None)  # Angles2Coords' counts carry their maximum
        if max_num_atoms is None:
            max_num_atoms = int(torch.max(num_atoms)) if num_atoms.numel() else 0
        B = x.size(0)
        na = num_atoms.to(device=dev, dtype=torch.int32).contiguous()
        rn = input_resnames.to(dev).contiguous()
        an = input_atomnames.to(dev).contiguous()
        out = torch.empty(B, 3 * max_num_atoms, dtype=x.dtype, device=dev)
        n_of_type = torch.empty(B, NUM_ATOM_TYPES, dtype=torch.int32, device=dev)
        offsets = torch.empty(B, NUM_ATOM_TYPES, dtype=torch.int32, device=dev)
        atom_indexes = torch.empty(B, max_num_atoms, dtype=torch.int32, device=dev)
        _FullAtomModel.Coords2TypedCoords_forward(x, rn, an, na, out, n_of_type, offsets, atom_indexes)
        _check(out, "forward", dev)
        ctx.atom_indexes = atom_indexes
        ctx.num_coords = x.size(1)
        ctx.save_for_backward(n_of_type, offsets)
        ctx.mark_non_differentiable(n_of_type, offsets)
        return out, n_of_type, offsets

    @staticmethod
    def backward(ctx, grad_typed_coords, *kwargs):
        n_of_type, offsets = ctx.saved_tensors
        g = grad_typed_coords.contiguous()
        grad = torch.empty(g.size(0), ctx.num_coords, dtype=g.dtype, device=g.device)
        _FullAtomModel.Coords2TypedCoords_backward(g, grad, n_of_type, offsets, ctx.atom_indexes)
        _check(grad, "backward", g.device)
        return grad, None, None, None


class Coords2TypedCoords(Module):
    def __init__(self):
        super(Coords2TypedCoords, self).__init__()

    def forward(self, input_coords, input_resnames, input_atomnames, num_atoms):
        return Coords2TypedCoordsFunction.apply(input_coords, input_resnames, input_atomnames, num_atoms)
