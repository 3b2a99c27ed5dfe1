"""Angles2Coords layer: 8 angles per residue + sequences -> heavy-atom coordinates.

Mirrors TorchProteinLibrary/FullAtomModel/Angles2Coords/Angles2Coords.py:12-88:
``Angles2Coords()(angles [B,8,L], sequences: list[str]) -> (coords [B, 3*maxA],
res_names uint8 [B,maxA,4], atom_names uint8 [B,maxA,4], num_atoms int32 [B])``,
rows of ``angles`` being phi, psi, omega, chi1..chi5, with a backward returning
dL/dangles.

Differences from the reference:
  * The compute runs on CUDA (float32: batched kernels, float64: FP64 kernels);
    the reference runs on the CPU only.  CPU angles raise RuntimeError.
  * coords and the name tensors live on the angles' device; ``num_atoms`` stays a
    CPU int32 tensor as in the reference.
  * The sequence byte tensor and atom counts are cached per batch of sequences,
    so repeated calls with the same sequences skip the per-sequence Python loop.
  * Unknown residue letters raise instead of being skipped.
  * The NaN check (a host sync) runs only when TPL_CHECK_NAN=1.
  * float32: the forward saves its output coordinates and the backward reads every
    joint's origin and axis from them (tpl_a2c_backward_coords_f32) instead of
    rebuilding the tree; ``Angles2CoordsFunction.backward_from_coords = False``
    selects the rebuilding backward (the reference's entry point).
"""
import math
import os

import numpy as np
import torch
from torch.autograd import Function
from torch.nn.modules.module import Module

from ... import load_extension

_FullAtomModel = load_extension("_FullAtomModel")


def convertStringList(stringList):
    """Sequences -> uint8 tensor [len(stringList), longest + 1], one NUL-terminated row each."""
    raw = [s.encode("ascii") for s in stringList]
    width = max(map(len, raw), default=0) + 1
    packed = b"".join(r.ljust(width, b"\0") for r in raw)
    return torch.from_numpy(np.frombuffer(packed, dtype=np.uint8).reshape(len(raw), width).copy())


def convertString(string):
    """A sequence -> NUL-terminated uint8 tensor."""
    return torch.tensor(list(string.encode("ascii")) + [0], dtype=torch.uint8)


def _check_nan_enabled():
    return os.environ.get("TPL_CHECK_NAN", "0") == "1"


def _check(t, where, device):
    if os.environ.get("TPL_CHECK_NAN", "0") == "1":
        status = _FullAtomModel.workspace_status(device.index if device.index is not None else 0)
        if status != 0:
            raise RuntimeError(f"Angles2CoordsFunction: {where}: device error {status}")
        if math.isnan(t.sum().item()):
            raise Exception(f"Angles2CoordsFunction: {where} Nan")


class Angles2CoordsFunction(Function):
    """Protein angles -> coordinates function"""

    backward_from_coords = True

    @staticmethod
    def forward(ctx, input_angles, sequenceTensor, num_atoms):
        input_angles = input_angles.contiguous()
        dev = input_angles.device
        max_num_atoms = getattr(num_atoms, "_tpl_max_atoms", None)  # set by Angles2Coords' sequence cache
        if max_num_atoms is None:
            max_num_atoms = int(torch.max(num_atoms)) if num_atoms.numel() else 0
        batch_size = input_angles.size(0)
        seq = sequenceTensor if sequenceTensor.device == dev else sequenceTensor.to(dev)
        coords = torch.empty(batch_size, 3 * max_num_atoms, dtype=input_angles.dtype, device=dev)
        res_names = torch.empty(batch_size, max_num_atoms, 4, dtype=torch.uint8, device=dev)
        atom_names = torch.empty(batch_size, max_num_atoms, 4, dtype=torch.uint8, device=dev)
        _FullAtomModel.Angles2Coords_forward(seq, input_angles, coords, res_names, atom_names)
        _check(coords, "forward", dev)
        ctx.from_coords = Angles2CoordsFunction.backward_from_coords and input_angles.dtype == torch.float32
        if ctx.from_coords:
            ctx.save_for_backward(input_angles, seq, coords)
        else:
            ctx.save_for_backward(input_angles, seq)
        ctx.mark_non_differentiable(res_names, atom_names, num_atoms)
        return coords, res_names, atom_names, num_atoms

    @staticmethod
    def backward(ctx, grad_atoms, *kwargs):
        saved = ctx.saved_tensors
        input_angles, seq = saved[0], saved[1]
        grad_atoms = grad_atoms.contiguous()
        grad_angles = torch.empty_like(input_angles)
        if ctx.from_coords:
            _FullAtomModel.Angles2Coords_backward_coords(grad_atoms, grad_angles, seq, saved[2])
        else:
            _FullAtomModel.Angles2Coords_backward(grad_atoms, grad_angles, seq, input_angles)
        _check(grad_angles, "backward", input_angles.device)
        return grad_angles, None, None


class Angles2Coords(Module):
    def __init__(self):
        super(Angles2Coords, self).__init__()
        self.num_atoms = None
        self._cache_key = None
        self._cache = None

    def _prepare(self, sequences, device):
        key = (tuple(sequences), device)
        if key != self._cache_key:
            seq = convertStringList(sequences).to(device)
            counts = [_FullAtomModel.getSeqNumAtoms(s) for s in sequences]
            num_atoms = torch.IntTensor(counts)
            num_atoms._tpl_max_atoms = max(counts, default=0)
            self._cache = (seq, num_atoms, counts)
            self._cache_key = key
        return self._cache

    def forward(self, input_angles_cpu, sequences):
        if not input_angles_cpu.is_cuda:
            raise RuntimeError("Angles2Coords: this build has no CPU path; move the angles to a CUDA device")
        seq, num_atoms, counts = self._prepare(sequences, input_angles_cpu.device)
        self.num_atoms = counts
        if not Angles2CoordsFunction.backward_from_coords or _check_nan_enabled():
            return Angles2CoordsFunction.apply(input_angles_cpu, seq, num_atoms)
        # the same entries as Angles2CoordsFunction, through the extension's C++ autograd
        # function: no Python frame in the backward, less host time per call
        coords, res_names, atom_names = _FullAtomModel.angles2coords_autograd(input_angles_cpu, seq,
                                                                               num_atoms._tpl_max_atoms, True)
        return coords, res_names, atom_names, num_atoms
