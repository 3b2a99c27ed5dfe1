"""Coords2RMSD on the GPU (the loss of the training-step workload).

The reference's _RMSD extension does not build against torch 2.x (Tensor::eig was
removed), so the oracle is a numpy restatement of its CPU path; it is pinned by the
properties the reference's own tests check (UnitTests/RMSD/Coords2RMSD/test.py:
RMSD of a rigidly moved copy is 0, gradcheck).  Tolerances: FP64 1e-9 relative,
FP32 1e-4 relative (rmsd) and 1e-3 relative (gradients)."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def case(B=8, N=300, seed=0):
    rng = np.random.default_rng(seed)
    na = rng.integers(3, N + 1, B).astype(np.int32)
    src = rng.standard_normal((B, 3 * N)) * 10
    dst = rng.standard_normal((B, 3 * N)) * 10
    return src, dst, na


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-9), (torch.float32, 1e-4)])
def test_matches_oracle(built, dtype, tol):
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    src, dst, na = case()
    layer = Coords2RMSD()
    x = torch.tensor(src, dtype=dtype, device="cuda", requires_grad=True)
    y = torch.tensor(dst, dtype=dtype, device="cuda")
    r = layer(x, y, torch.tensor(na, device="cuda"))
    r.sum().backward()
    ro, UTo, go = oracle.rmsd(src, dst, na)
    assert np.allclose(r.detach().double().cpu().numpy(), ro, rtol=tol, atol=0)
    g = x.grad.double().cpu().numpy()
    assert np.abs(g - go).max() <= 10 * tol * np.abs(go).max()
    # UT agrees up to the sign convention of the eigenvector (U(q) = U(-q))
    assert np.allclose(layer.UT.double().cpu().numpy(), UTo, atol=100 * tol)


def test_rigid_copy_has_zero_rmsd(built):
    """UnitTests/RMSD/Coords2RMSD/test.py: a rotated and translated copy gives RMSD ~ 0."""
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    rng = np.random.default_rng(1)
    B, N = 6, 200
    src = rng.standard_normal((B, N, 3)) * 15
    dst = np.stack([src[b] @ random_rotation(rng).T + rng.standard_normal(3) * 20 for b in range(B)])
    na = np.full(B, N, np.int32)
    r = Coords2RMSD()(torch.tensor(src.reshape(B, -1), device="cuda"), torch.tensor(dst.reshape(B, -1), device="cuda"),
                      torch.tensor(na, device="cuda"))
    assert r.max().item() < 1e-4


def test_gradcheck_and_function_api(built):
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    from torchproteinlibrary_gb300.RMSD.Coords2RMSD import Coords2RMSDFunction
    src, dst, na = case(B=3, N=12, seed=5)
    x = torch.tensor(src, device="cuda", requires_grad=True)
    y = torch.tensor(dst, device="cuda")
    n = torch.tensor(na, device="cuda")
    assert torch.autograd.gradcheck(lambda a: Coords2RMSD()(a, y, n), (x,), eps=1e-6, atol=1e-6, rtol=1e-5)
    # Function API on already-centred inputs (reference Coords2RMSDFunction)
    xc = x.detach().clone()
    yc = y.clone()
    for b in range(3):
        m = na[b]
        xc[b, :3 * m] -= xc[b, :3 * m].view(m, 3).mean(0).repeat(m)
        yc[b, :3 * m] -= yc[b, :3 * m].view(m, 3).mean(0).repeat(m)
    r1, UT = Coords2RMSDFunction.apply(xc, yc, n)
    r2 = Coords2RMSD()(x.detach(), y, n)
    assert torch.allclose(r1, r2, rtol=1e-9)


def test_host_num_atoms_reused_and_refreshed(built):
    """A host num_atoms tensor is copied to the device once and reused on later calls;
    changing it in place makes the next call copy the new counts."""
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    src, dst, na = case(B=4, N=50, seed=3)
    layer = Coords2RMSD()
    x = torch.tensor(src, device="cuda")
    y = torch.tensor(dst, device="cuda")
    n = torch.tensor(na, dtype=torch.int32)
    r1 = layer(x, y, n)
    r2 = layer(x, y, n)
    assert torch.equal(r1, r2)
    n[0] = 3
    r3 = layer(x, y, n)
    ref, _, _ = oracle.rmsd(src, dst, n.numpy())
    assert np.allclose(r3.cpu().numpy(), ref, rtol=1e-9, atol=0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_small_and_degenerate_chains(built, dtype):
    """Chains of 0, 1, 2 and 3 atoms, collinear and planar chains (repeated
    eigenvalues of the key matrix), identical structures (rmsd 0) and a mirrored copy:
    rmsd against the oracle, finite gradients everywhere and zero gradient past each
    chain.  rmsd = sqrt((R2 - 2 lambda + 1e-10) / N) cancels for near-identical
    structures, so its absolute resolution is about sqrt(eps R2 / N): the tolerance is
    2e-2 A in float32 and 1e-5 A in float64 (coordinates of about 10 A here)."""
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    rng = np.random.default_rng(77)
    N = 40
    src = rng.standard_normal((10, N, 3)) * 8
    dst = rng.standard_normal((10, N, 3)) * 8
    na = np.array([0, 1, 2, 3, N, N, N, N, N, N], np.int32)
    line = np.linspace(-20, 20, N)[:, None] * np.array([0.3, 0.5, 0.8])
    src[4], dst[4] = line, line[::-1] + 5.0                      # collinear
    src[5, :, 2] = 0.0
    dst[5] = src[5] @ random_rotation(rng).T + 3.0                # planar, rigid copy
    dst[6] = src[6]                                               # identical
    dst[7] = src[7] * np.array([-1.0, 1.0, 1.0])                  # mirror image
    src[8, :, 2] = 0.0
    dst[8, :, 2] = 0.0                                            # both planar
    x = torch.tensor(src.reshape(10, -1), dtype=dtype, device="cuda", requires_grad=True)
    y = torch.tensor(dst.reshape(10, -1), dtype=dtype, device="cuda")
    r = Coords2RMSD()(x, y, torch.tensor(na, device="cuda"))
    r.sum().backward()
    ro, _, _ = oracle.rmsd(src.reshape(10, -1), dst.reshape(10, -1), na)
    atol = 2e-2 if dtype == torch.float32 else 1e-5
    np.testing.assert_allclose(r.detach().double().cpu().numpy(), ro, atol=atol, rtol=0)
    g = x.grad.double().cpu().numpy()
    assert np.isfinite(g).all()
    for b in range(10):
        assert np.all(g[b, 3 * na[b]:] == 0.0)
