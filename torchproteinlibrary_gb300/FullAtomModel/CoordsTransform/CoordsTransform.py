"""CoordsTransform: translate, rotate and centre batched coordinates, bounding boxes
and rotation helpers.

Mirrors TorchProteinLibrary/FullAtomModel/CoordsTransform/CoordsTransform.py: the
same function and class names, argument order and shapes.  Coordinates are
[batch, 3 * atoms]; the first num_atoms[b] atoms of each row are transformed and the
rest of the row is zero.

Differences from the reference:
  * The layers and getBBox run on CUDA tensors only (sm_103a kernels behind the C ABI);
    CPU coordinates raise RuntimeError.  ``num_atoms`` may live on the CPU; it is
    moved to the coordinates' device.
  * getRotation / getRandomRotation / getRandomTranslation are the same formulas
    (Math/nUtil.cpp:60-100) written as tensor arithmetic, so they run on any device.
    getRandomRotation and getRandomTranslation take an optional ``device`` /
    generator (torch.rand), where the reference draws on the CPU.
  * Coords2Center of an empty chain is 0 (the reference divides by zero and its NaN
    check raises).
  * The NaN checks that force a host sync after every call run only when
    TPL_CHECK_NAN=1.
"""
import math
import os

import torch
from torch.autograd import Function
from torch.nn.modules.module import Module

from ... import load_extension

_FullAtomModel = load_extension("_FullAtomModel")

__all__ = ["getBBox", "getRandomTranslation", "getRandomRotation", "getRotation", "CoordsTranslateFunction",
           "CoordsTranslate", "CoordsRotateFunction", "CoordsRotate", "Coords2CenterFunction", "Coords2Center"]


def _check(t, what):
    if os.environ.get("TPL_CHECK_NAN", "0") == "1" and math.isnan(t.sum().item()):
        raise Exception(f"{what} Nan")


def _coords(x, what):
    if x.dim() != 2:
        raise ValueError(f'{what}: ', 'Incorrect input size:', x.size())
    if not x.is_cuda:
        raise RuntimeError(f"{what}: this build has no CPU path; move the tensors to a CUDA device")
    return x.contiguous()


def _num_atoms(num_atoms, device):
    return num_atoms.to(device=device, dtype=torch.int32).contiguous()


def getBBox(input_coords, num_atoms):
    """Per-chain bounding box: a = min, b = max over the first num_atoms[b] atoms."""
    x = _coords(input_coords, "getBBox")
    a = torch.empty(x.size(0), 3, dtype=x.dtype, device=x.device)
    b = torch.empty_like(a)
    _FullAtomModel.getBBox(x, a, b, _num_atoms(num_atoms, x.device))
    return a, b


def getRandomTranslation(a, b, volume_size, generator=None):
    """Random translation keeping a box [a, b] inside a cube of side volume_size
    (Math/nUtil.cpp:88-100): T_k ~ U[-d_k, d_k], d_k = max(0, volume_size/2 - (b_k - a_k)/2) / 2."""
    if a.dim() != 2:
        raise ValueError('getRandomTranslation: ', 'Incorrect input size:', a.size())
    d = torch.clamp(volume_size / 2.0 - (b - a) / 2.0, min=0.0) * 0.5
    u = torch.rand(a.shape, dtype=torch.float64, device=a.device, generator=generator)
    return (u * (2.0 * d.double()) - d.double()).to(a.dtype)


def getRotation(u):
    """Rotation matrices [B, 3, 3] (float64) from u [B, 3] in [0, 1)^3: the unit
    quaternion q = (sqrt(1-u1) sin 2 pi u2, sqrt(1-u1) cos 2 pi u2, sqrt(u1) sin 2 pi u3,
    sqrt(u1) cos 2 pi u3) of Math/nUtil.cpp:60-79, uniform over SO(3) for uniform u."""
    u = u.double()
    s1, s2 = torch.sqrt(1.0 - u[:, 0]), torch.sqrt(u[:, 0])
    q0 = s1 * torch.sin(2.0 * math.pi * u[:, 1])
    q1 = s1 * torch.cos(2.0 * math.pi * u[:, 1])
    q2 = s2 * torch.sin(2.0 * math.pi * u[:, 2])
    q3 = s2 * torch.cos(2.0 * math.pi * u[:, 2])
    R = torch.stack([
        q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3, 2.0 * (q1 * q2 - q0 * q3), 2.0 * (q1 * q3 + q0 * q2),
        2.0 * (q1 * q2 + q0 * q3), q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3, 2.0 * (q2 * q3 - q0 * q1),
        2.0 * (q1 * q3 - q0 * q2), 2.0 * (q2 * q3 + q0 * q1), q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3], dim=1)
    return R.view(-1, 3, 3)


def getRandomRotation(batch_size, device=None, generator=None):
    """batch_size uniformly random rotations, float64 [B, 3, 3]."""
    return getRotation(torch.rand(batch_size, 3, dtype=torch.float64, device=device, generator=generator))


class CoordsTranslateFunction(Function):
    """coordinates translation: out = in + T[b] for the first num_atoms[b] atoms."""

    @staticmethod
    def forward(ctx, input_coords, T, num_atoms):
        x = _coords(input_coords, "CoordsTranslateFunction")
        na = _num_atoms(num_atoms, x.device)
        T = T.to(device=x.device, dtype=x.dtype).contiguous()
        ctx.save_for_backward(T, na)
        out = torch.empty_like(x)
        _FullAtomModel.CoordsTranslateGPU_forward(x, out, T, na)
        _check(out, "CoordsTranslateFunction: forward")
        return out

    @staticmethod
    def backward(ctx, grad_output_coords):
        T, na = ctx.saved_tensors
        g = grad_output_coords.contiguous()
        grad = torch.empty_like(g)
        _FullAtomModel.CoordsTranslateGPU_backward(g, grad, T, na)
        return grad, None, None


class CoordsTranslate(Module):
    def __init__(self):
        super(CoordsTranslate, self).__init__()

    def forward(self, input_coords, T, num_atoms):
        return CoordsTranslateFunction.apply(input_coords, T, num_atoms)


class CoordsRotateFunction(Function):
    """coordinates rotation: out = R[b] in for the first num_atoms[b] atoms."""

    @staticmethod
    def forward(ctx, input_coords, R, num_atoms):
        x = _coords(input_coords, "CoordsRotateFunction")
        na = _num_atoms(num_atoms, x.device)
        R = R.to(device=x.device, dtype=x.dtype).contiguous()
        ctx.save_for_backward(R, na)
        out = torch.empty_like(x)
        _FullAtomModel.CoordsRotateGPU_forward(x, out, R, na)
        _check(out, "CoordsRotateFunction: forward")
        return out

    @staticmethod
    def backward(ctx, grad_output_coords):
        R, na = ctx.saved_tensors
        g = grad_output_coords.contiguous()
        grad = torch.empty_like(g)
        _FullAtomModel.CoordsRotateGPU_backward(g, grad, R, na)
        _check(grad, "CoordsRotateFunction: backward")
        return grad, None, None


class CoordsRotate(Module):
    def __init__(self):
        super(CoordsRotate, self).__init__()

    def forward(self, input_coords, R, num_atoms):
        return CoordsRotateFunction.apply(input_coords, R, num_atoms)


class Coords2CenterFunction(Function):
    """Geometric centre of the first num_atoms[b] atoms, [batch, 3]."""

    @staticmethod
    def forward(ctx, input_coords, num_atoms):
        x = _coords(input_coords, "Coords2CenterFunction")
        na = _num_atoms(num_atoms, x.device)
        ctx.save_for_backward(na)
        ctx.num_coords = x.size(1)
        center = torch.empty(x.size(0), 3, dtype=x.dtype, device=x.device)
        _FullAtomModel.Coords2CenterGPU_forward(x, center, na)
        _check(center, "Coords2CenterFunction: forward")
        return center

    @staticmethod
    def backward(ctx, grad_output_center):
        na, = ctx.saved_tensors
        g = grad_output_center.contiguous()
        grad = torch.empty(g.size(0), ctx.num_coords, dtype=g.dtype, device=g.device)
        _FullAtomModel.Coords2CenterGPU_backward(g, grad, na)
        return grad, None


class Coords2Center(Module):
    def __init__(self):
        super(Coords2Center, self).__init__()

    def forward(self, input_coords, num_atoms):
        return Coords2CenterFunction.apply(input_coords, num_atoms)
