"""CoordsTransform, Coords2TypedCoords and Coords2RMSD on the GPU against the
reference's own outputs (tests/golden/{transform,typed,rmsd}_ref.npz, written by
the reference's Python layers over its CPU interfaces; tests/golden/make_golden.py).

Tolerances: translate, bounding box and typed coordinates (copies) exact; rotate
1e-14 (FP64) / 2 ulp (FP32) of the coordinate scale; centre 1e-14 / 8 ulp (the
kernel accumulates in FP64 across warps, the reference serially in the coordinate
type); Coords2RMSD 1e-9 relative in FP64."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name))


@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_transform_layers_match_reference(built, tag):
    from torchproteinlibrary_gb300.FullAtomModel import CoordsTransform as ct
    d = _load("transform_ref.npz")
    dev = torch.device("cuda")
    x = d[f"{tag}_x"]
    ulp = 2.0 ** -52 if tag == "f64" else 2.0 ** -23
    scale = np.abs(x).max()
    na = torch.tensor(d["num_atoms"])
    xt = torch.tensor(x, device=dev, requires_grad=True)
    g = torch.tensor(d[f"{tag}_grad_out"], device=dev)
    R = torch.tensor(d["rotation"].astype(x.dtype), device=dev)

    y = ct.CoordsTranslate()(xt, torch.tensor(d[f"{tag}_T"], device=dev), na)
    y.backward(g)
    assert np.array_equal(y.detach().cpu().numpy(), d[f"{tag}_translate"])
    assert np.array_equal(xt.grad.cpu().numpy(), d[f"{tag}_translate_grad"])

    xt.grad = None
    y = ct.CoordsRotate()(xt, R, na)
    y.backward(g)
    rot_tol = 1e-14 if tag == "f64" else 2 * ulp
    assert np.abs(y.detach().cpu().numpy() - d[f"{tag}_rotate"]).max() <= rot_tol * scale
    assert np.abs(xt.grad.cpu().numpy() - d[f"{tag}_rotate_grad"]).max() <= 4 * rot_tol * np.abs(d[f"{tag}_grad_out"]).max()

    xt.grad = None
    c = ct.Coords2Center()(xt, na)
    c.backward(torch.tensor(d[f"{tag}_grad_center"], device=dev))
    c_tol = 1e-14 if tag == "f64" else 8 * ulp
    assert np.abs(c.detach().cpu().numpy() - d[f"{tag}_center"]).max() <= c_tol * scale
    assert np.array_equal(xt.grad.cpu().numpy(), d[f"{tag}_center_grad"])

    lo, hi = ct.getBBox(xt.detach(), na)
    assert np.array_equal(lo.cpu().numpy(), d[f"{tag}_bbox_lo"])
    assert np.array_equal(hi.cpu().numpy(), d[f"{tag}_bbox_hi"])


def test_rotation_from_u_matches_reference(built):
    from torchproteinlibrary_gb300.FullAtomModel import CoordsTransform as ct
    d = _load("transform_ref.npz")
    R = ct.getRotation(torch.tensor(d["u"], device="cuda"))
    assert np.abs(R.cpu().numpy() - d["rotation"]).max() <= 1e-15


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_typed_coords_match_reference(built, dtype):
    from torchproteinlibrary_gb300.FullAtomModel import Coords2TypedCoords
    d = _load("typed_ref.npz")
    dev = torch.device("cuda")
    x = torch.tensor(d["coords"], dtype=dtype, device=dev, requires_grad=True)
    typed, counts, offsets = Coords2TypedCoords()(x, torch.tensor(d["res_names"], device=dev),
                                                  torch.tensor(d["atom_names"], device=dev),
                                                  torch.tensor(d["num_atoms"], device=dev))
    assert np.array_equal(counts.cpu().numpy(), d["num_atoms_of_type"])
    assert np.array_equal(offsets.cpu().numpy(), d["offsets"])
    ref = torch.tensor(d["typed"], dtype=dtype).numpy()
    assert np.array_equal(typed.detach().cpu().numpy(), ref)
    typed.backward(torch.tensor(d["grad_typed"], dtype=dtype, device=dev))
    assert np.array_equal(x.grad.cpu().numpy(), torch.tensor(d["grad_coords"], dtype=dtype).numpy())


def test_rmsd_matches_reference(built):
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    d = _load("rmsd_ref.npz")
    dev = torch.device("cuda")
    layer = Coords2RMSD()
    x = torch.tensor(d["src"], device=dev, requires_grad=True)
    r = layer(x, torch.tensor(d["dst"], device=dev), torch.tensor(d["num_atoms"]))
    r.backward(torch.tensor(d["grad_rmsd"], device=dev))
    np.testing.assert_allclose(r.detach().cpu().numpy(), d["rmsd"], rtol=1e-9, atol=0)
    assert np.abs(layer.UT.detach().cpu().numpy() - d["ut"]).max() <= 1e-9
    assert np.abs(x.grad.cpu().numpy() - d["grad_src"]).max() <= 1e-9 * np.abs(d["grad_src"]).max()
