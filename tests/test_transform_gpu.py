"""CoordsTransform on the GPU against the oracle (restatement of
Layers/FullAtomModel/TransformCUDAKernels.cu:4-107 and Math/nUtil.cpp:27-57).

Tolerances: translate and its backward are single additions (bit-exact in both
dtypes); rotate 1e-12 (FP64) / 2e-6 (FP32) relative to the coordinate scale;
centre 1e-12 / 1e-6 (FP64 accumulation in the kernel); bounding box bit-exact."""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def case(dtype, B=9, S=700, seed=0):
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal((B, 3 * S)) * 30).astype(np.float64)
    na = rng.integers(0, S + 1, B).astype(np.int32)
    na[0], na[1], na[2] = S, 0, 1
    T = rng.standard_normal((B, 3)) * 10
    R = oracle.rotation_from_u(rng.uniform(0, 1, (B, 3)))
    if dtype == torch.float32:
        x, T, R = x.astype(np.float32), T.astype(np.float32), R.astype(np.float32)
    return x, na, T, R


@pytest.fixture(scope="module")
def ct(built):
    from torchproteinlibrary_gb300.FullAtomModel import CoordsTransform
    return CoordsTransform


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_translate_rotate_center_layers(ct, dtype):
    x, na, T, R = case(dtype)
    dev = torch.device("cuda")
    xt = torch.tensor(x, device=dev, requires_grad=True)
    nat = torch.tensor(na)
    tol_rot = 2e-6 if dtype == torch.float32 else 1e-12
    scale = np.abs(x).max()

    y = ct.CoordsTranslate()(xt, torch.tensor(T, device=dev), nat)
    assert np.array_equal(y.detach().cpu().numpy(), oracle.coords_translate(x, T, na))
    g = torch.tensor(np.random.default_rng(1).standard_normal(x.shape).astype(x.dtype), device=dev)
    y.backward(g)
    assert np.array_equal(xt.grad.cpu().numpy(), oracle.coords_translate(g.cpu().numpy(), None, na))

    xt.grad = None
    y = ct.CoordsRotate()(xt, torch.tensor(R, device=dev), nat)
    assert np.abs(y.detach().cpu().numpy() - oracle.coords_rotate(x, R, na)).max() <= tol_rot * scale
    y.backward(g)
    gref = oracle.coords_rotate(g.cpu().numpy(), R, na, transpose=True)
    assert np.abs(xt.grad.cpu().numpy() - gref).max() <= tol_rot * np.abs(gref).max()

    xt.grad = None
    c = ct.Coords2Center()(xt, nat)
    tol_c = 1e-6 if dtype == torch.float32 else 1e-12
    assert np.abs(c.detach().cpu().numpy() - oracle.coords_center(x, na)).max() <= tol_c * scale
    gc = torch.tensor(np.random.default_rng(2).standard_normal((x.shape[0], 3)).astype(x.dtype), device=dev)
    c.backward(gc)
    gref = oracle.coords_center_backward(gc.cpu().numpy(), na, x.shape[1] // 3)
    assert np.allclose(xt.grad.cpu().numpy(), gref, rtol=1e-6 if dtype == torch.float32 else 1e-14, atol=0)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_bbox_and_centering_composition(ct, dtype):
    """getBBox against the oracle; translating by minus the centre centres the chain
    (the reference's Coords2Center + CoordsTranslate idiom)."""
    x, na, _, _ = case(dtype, seed=4)
    dev = torch.device("cuda")
    xt = torch.tensor(x, device=dev)
    lo, hi = ct.getBBox(xt, torch.tensor(na))
    rlo, rhi = oracle.coords_bbox(x, na)
    assert np.array_equal(lo.cpu().numpy(), rlo) and np.array_equal(hi.cpu().numpy(), rhi)
    c = ct.Coords2Center()(xt, torch.tensor(na))
    y = ct.CoordsTranslate()(xt, -c, torch.tensor(na))
    c2 = ct.Coords2Center()(y, torch.tensor(na)).cpu().numpy()
    assert np.abs(c2).max() <= (1e-4 if dtype == torch.float32 else 1e-11)


def test_c_abi_translate_rotate(built):
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    x, na, T, R = case(torch.float32, B=5, S=33, seed=7)
    dev = torch.device("cuda")
    xt = torch.tensor(x, device=dev)
    nat = torch.tensor(na, device=dev)
    out = torch.full_like(xt, float("nan"))
    capi.check(lib.tpl_coords_translate_f32(xt.data_ptr(), out.data_ptr(), torch.tensor(T, device=dev).data_ptr(),
                                            nat.data_ptr(), 5, 33, capi.stream_ptr()), "translate")
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.coords_translate(x, T, na))
    Rt = torch.tensor(R, device=dev)
    capi.check(lib.tpl_coords_rotate_f32(xt.data_ptr(), out.data_ptr(), Rt.data_ptr(), 0, nat.data_ptr(), 5, 33,
                                         capi.stream_ptr()), "rotate")
    torch.cuda.synchronize()
    assert np.abs(out.cpu().numpy() - oracle.coords_rotate(x, R, na)).max() <= 2e-6 * np.abs(x).max()
    assert lib.tpl_coords_rotate_f32(None, out.data_ptr(), Rt.data_ptr(), 0, nat.data_ptr(), 5, 33, None) == -1


@pytest.mark.parametrize("S", [700, 33, 4000])
def test_center_vector_and_scalar_paths(ct, S):
    """Coords2Center in float32 reads 16-byte rows (stride a multiple of 4 atoms) as
    float4 groups of four atoms plus a scalar tail, and other strides atom by atom;
    both against the oracle within 1e-6 of the coordinate scale, with counts of every
    residue mod 4 and a chain far from the origin."""
    x, na, _, _ = case(torch.float32, B=12, S=S, seed=11)
    na[3:7] = [max(0, S - 1), max(0, S - 2), max(0, S - 3), min(5, S)]
    x[4] += 500.0
    c = ct.Coords2Center()(torch.tensor(x, device="cuda"), torch.tensor(na)).cpu().numpy()
    assert np.abs(c - oracle.coords_center(x, na)).max() <= 1e-6 * np.abs(x).max()
