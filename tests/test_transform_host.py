"""CoordsTransform host-side helpers (no GPU): getRotation / getRandomRotation /
getRandomTranslation are tensor formulas that run on any device; they are checked
here on CPU tensors against the oracle's restatement of Math/nUtil.cpp:60-100."""
import numpy as np
import pytest
import torch

import oracle


@pytest.fixture(scope="module")
def ct(built):
    from torchproteinlibrary_gb300.FullAtomModel import CoordsTransform
    return CoordsTransform


def test_get_rotation_matches_oracle_and_is_orthonormal(ct):
    u = np.random.default_rng(3).uniform(0, 1, (64, 3))
    R = ct.getRotation(torch.tensor(u)).numpy()
    assert R.dtype == np.float64 and R.shape == (64, 3, 3)
    assert np.allclose(R, oracle.rotation_from_u(u), atol=1e-14)
    assert np.allclose(R @ R.transpose(0, 2, 1), np.eye(3), atol=1e-13)
    assert np.allclose(np.linalg.det(R), 1.0, atol=1e-13)


def test_random_rotation_and_translation_ranges(ct):
    g = torch.Generator().manual_seed(5)
    R = ct.getRandomRotation(16, generator=g)
    assert R.shape == (16, 3, 3) and torch.allclose(R @ R.transpose(1, 2), torch.eye(3, dtype=torch.float64).expand(16, 3, 3), atol=1e-12)
    a = torch.tensor([[0.0, -5.0, 2.0], [10.0, 10.0, 10.0]])
    b = torch.tensor([[4.0, 5.0, 2.0], [90.0, 12.0, 10.0]])
    T = ct.getRandomTranslation(a, b, 40.0, generator=g)
    d = torch.clamp(20.0 - (b - a) / 2.0, min=0.0) * 0.5
    assert T.shape == a.shape and bool((T.abs() <= d + 1e-6).all())
    assert float(T[1, 0]) == 0.0  # a box wider than the volume leaves no room


def test_extension_pose_helpers_match_the_layer_module(ct):
    """The reference-signature entry points of _FullAtomModel fill caller tensors
    (coordsTransform_interface.cpp:201-259) with the same formulas."""
    from torchproteinlibrary_gb300 import load_extension
    ext = load_extension("_FullAtomModel")
    u = torch.tensor(np.random.default_rng(4).uniform(0, 1, (8, 3)))
    R = torch.zeros(8, 3, 3, dtype=torch.float64)
    ext.getRotation(R, u)
    assert torch.allclose(R, ct.getRotation(u), atol=1e-14)
    R32 = torch.zeros(8, 3, 3, dtype=torch.float32)
    ext.getRandomRotation(R32)
    eye = torch.eye(3).expand(8, 3, 3)
    assert torch.allclose(R32 @ R32.transpose(1, 2), eye, atol=1e-5)
    torch.manual_seed(11)
    ext.getRandomRotation(R)
    torch.manual_seed(11)
    assert torch.allclose(R, ct.getRotation(torch.rand(8, 3, dtype=torch.float64)), atol=1e-14)
    a = torch.tensor([[0.0, -5.0, 2.0], [10.0, 10.0, 10.0]], dtype=torch.float64)
    b = torch.tensor([[4.0, 5.0, 2.0], [90.0, 12.0, 10.0]], dtype=torch.float64)
    T = torch.full((2, 3), 99.0, dtype=torch.float64)
    ext.getRandomTranslation(T, a, b, 40.0)
    d = torch.clamp(20.0 - (b - a) / 2.0, min=0.0) * 0.5
    assert bool((T.abs() <= d + 1e-12).all()) and float(T[1, 0]) == 0.0
    with pytest.raises(RuntimeError):
        ext.getRotation(torch.zeros(2, 3), u)
