"""Coords2TypedCoords on the GPU against the oracle (restatement of
coords2typedcoords_interface.cpp and ProtUtil::get11AtomType).  Integer and byte
work plus coordinate copies: everything is compared bit-exactly."""
import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

AA = "ACDEFGHIKLMNPQRSTVWY"


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_forward_backward_match_oracle(built, dtype):
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords, Coords2TypedCoords
    rng = np.random.default_rng(11)
    lengths = [60, 1, 37, 120, 5]
    seqs = ["".join(rng.choice(list(AA), n)) for n in lengths]
    seqs[0] = (AA * 3)[:60]
    L = max(lengths)
    ang = torch.tensor(rng.uniform(-np.pi, np.pi, (len(seqs), 8, L)), dtype=dtype, device="cuda")
    coords, rn, an, na = Angles2Coords()(ang, seqs)
    x = coords.detach().clone().requires_grad_()
    typed, counts, offsets = Coords2TypedCoords()(x, rn, an, na)
    xc, rc, ac = coords.detach().cpu().numpy(), rn.cpu().numpy(), an.cpu().numpy()
    rt, rcnt, roff, ridx = oracle.typed_coords(xc, rc, ac, na.numpy())
    assert np.array_equal(typed.detach().cpu().numpy(), rt)
    assert np.array_equal(counts.cpu().numpy(), rcnt) and np.array_equal(offsets.cpu().numpy(), roff)
    g = torch.tensor(rng.standard_normal(typed.shape), dtype=dtype, device="cuda")
    typed.backward(g)
    ref = oracle.typed_coords_backward(g.cpu().numpy(), rcnt, ridx, xc.shape[1] // 3)
    assert np.array_equal(x.grad.cpu().numpy(), ref)


def test_unknown_name_is_reported(built):
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    dev = torch.device("cuda")
    x = torch.zeros(1, 6, device=dev)
    rn = torch.tensor([[list(b"ALA\0"), list(b"ALA\0")]], dtype=torch.uint8, device=dev)
    an = torch.tensor([[list(b"CB\0\0"), list(b"QQ\0\0")]], dtype=torch.uint8, device=dev)
    na = torch.tensor([2], dtype=torch.int32, device=dev)
    out = torch.empty(1, 6, device=dev)
    cnt = torch.empty(1, 11, dtype=torch.int32, device=dev)
    off = torch.empty_like(cnt)
    idx = torch.empty(1, 2, dtype=torch.int32, device=dev)
    ws = torch.zeros(64, dtype=torch.uint8, device=dev)
    capi.check(lib.tpl_typed_coords_forward_f32(x.data_ptr(), rn.data_ptr(), an.data_ptr(), na.data_ptr(), 1, 2, 2,
                                                out.data_ptr(), cnt.data_ptr(), off.data_ptr(), idx.data_ptr(),
                                                ws.data_ptr(), 64, capi.stream_ptr()), "typed")
    st = capi.ctypes.c_int()
    capi.check(lib.tpl_workspace_status(ws.data_ptr(), capi.stream_ptr(), capi.ctypes.byref(st)), "status")
    assert st.value == -10
    assert int(cnt.sum()) == 1 and int(cnt[0, 10]) == 1


def test_padded_names_take_the_slow_path(built):
    """Atom names with spaces or a tab inside their 4 bytes (PDB-style ' CA ', 'CB  ')
    are squeezed as the reference does (whitespace erased) and typed like the packed
    names; the packed names take the word-at-a-time path, the padded ones the byte
    loop.  Against the oracle, bit for bit."""
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    dev = torch.device("cuda")
    names = [b"N\0\0\0", b" CA ", b"C\0\0\0", b"O  \0", b"CB  ", b"\tCG\0", b"CD1\0", b"C D2", b"CE\0\0", b"NZ\0\0"]
    res = [b"LEU\0"] * 4 + [b"LEU\0", b"LEU\0", b"LEU\0", b"LEU\0", b"LYS\0", b"LYS\0"]
    n = len(names)
    rng = np.random.default_rng(5)
    x = torch.tensor(rng.standard_normal((1, 3 * n)), dtype=torch.float32, device=dev)
    rn = torch.tensor([[list(r) for r in res]], dtype=torch.uint8, device=dev)
    an = torch.tensor([[list(a) for a in names]], dtype=torch.uint8, device=dev)
    na = torch.tensor([n], dtype=torch.int32, device=dev)
    out = torch.full((1, 3 * n), float("nan"), device=dev)
    cnt = torch.empty(1, 11, dtype=torch.int32, device=dev)
    off = torch.empty_like(cnt)
    idx = torch.empty(1, n, dtype=torch.int32, device=dev)
    ws = torch.zeros(64, dtype=torch.uint8, device=dev)
    capi.check(lib.tpl_typed_coords_forward_f32(x.data_ptr(), rn.data_ptr(), an.data_ptr(), na.data_ptr(), 1, n, n,
                                                out.data_ptr(), cnt.data_ptr(), off.data_ptr(), idx.data_ptr(),
                                                ws.data_ptr(), 64, capi.stream_ptr()), "typed")
    st = capi.ctypes.c_int()
    capi.check(lib.tpl_workspace_status(ws.data_ptr(), capi.stream_ptr(), capi.ctypes.byref(st)), "status")
    assert st.value == 0
    rt, rcnt, roff, ridx = oracle.typed_coords(x.cpu().numpy(), rn.cpu().numpy(), an.cpu().numpy(), [n])
    assert int(rcnt.sum()) == n
    np.testing.assert_array_equal(cnt.cpu().numpy(), rcnt)
    np.testing.assert_array_equal(off.cpu().numpy(), roff)
    np.testing.assert_array_equal(idx.cpu().numpy(), ridx)
    np.testing.assert_array_equal(out.cpu().numpy(), rt)


def test_long_chain_path(built):
    """Rows of more than 32768 atoms take the one-CTA-per-chain kernel (no per-row type
    cache in shared memory): a 4100-residue chain beside a short one, forward and
    backward against the oracle bit for bit."""
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords, Coords2TypedCoords
    rng = np.random.default_rng(17)
    seqs = ["".join(rng.choice(list(AA), 4100)), "".join(rng.choice(list(AA), 12))]
    ang = torch.tensor(rng.uniform(-np.pi, np.pi, (2, 8, 4100)), dtype=torch.float32, device="cuda")
    coords, rn, an, na = Angles2Coords()(ang, seqs)
    assert coords.shape[1] // 3 > 32768
    x = coords.detach().clone().requires_grad_()
    typed, counts, offsets = Coords2TypedCoords()(x, rn, an, na)
    xc, rc, ac = coords.detach().cpu().numpy(), rn.cpu().numpy(), an.cpu().numpy()
    rt, rcnt, roff, ridx = oracle.typed_coords(xc, rc, ac, na.numpy())
    assert np.array_equal(typed.detach().cpu().numpy(), rt)
    assert np.array_equal(counts.cpu().numpy(), rcnt) and np.array_equal(offsets.cpu().numpy(), roff)
    g = torch.tensor(rng.standard_normal(typed.shape), dtype=torch.float32, device="cuda")
    typed.backward(g)
    ref = oracle.typed_coords_backward(g.cpu().numpy(), rcnt, ridx, xc.shape[1] // 3)
    assert np.array_equal(x.grad.cpu().numpy(), ref)
