"""The no-allocation Angles2Backbone forward (tpl_a2b_forward_f32_noalloc).

It serves callers that cannot allocate device memory, such as an FFI host that
owns only the buffers it passes in, or a process whose framework has already
reserved the GPU's memory.  It keeps its scratch in a fixed array inside the
library instead of a caller workspace.  These tests drive it through the C ABI
and compare it with the workspace entry point, tpl_a2b_forward_f32.  The
tolerance is the FP32 one used elsewhere (1e-3 A); the two paths run the same
kernel and are expected to agree exactly.  The file is named to be collected
last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

COORD_TOL_F32 = 1e-3


def _inputs(B, L, seed):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L)).astype(np.float32)
    lengths = rng.integers(0, L + 1, B).astype(np.int32)
    lengths[0] = L
    dev = torch.device("cuda")
    return torch.tensor(ang, device=dev), torch.tensor(lengths, device=dev)


def _with_workspace(lib, capi, ang, lengths):
    B, _, L = ang.shape
    n = lib.tpl_a2b_workspace_bytes(B, L, None)
    ws = torch.zeros(n, dtype=torch.uint8, device=ang.device)
    out = torch.full((B, 9 * L), float("nan"), device=ang.device)
    capi.check(lib.tpl_a2b_forward_f32(ang.data_ptr(), lengths.data_ptr(), out.data_ptr(), ws.data_ptr(), n, B, L,
                                       None, capi.stream_ptr()), "tpl_a2b_forward_f32")
    torch.cuda.synchronize()
    return out


def _no_alloc(lib, capi, ang, lengths):
    B, _, L = ang.shape
    out = torch.full((B, 9 * L), float("nan"), device=ang.device)
    capi.check(lib.tpl_a2b_forward_f32_noalloc(ang.data_ptr(), lengths.data_ptr(), out.data_ptr(), B, L, None,
                                               capi.stream_ptr()), "tpl_a2b_forward_f32_noalloc")
    torch.cuda.synchronize()
    return out


def test_no_alloc_matches_workspace_entry_on_two_calls(built):
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    # two calls in a row with different inputs: the shared scratch keeps the first
    # call's contents and is cleared by the second
    for seed, (B, L) in [(1, (64, 300)), (2, (48, 517))]:
        ang, lengths = _inputs(B, L, seed)
        ref = _with_workspace(lib, capi, ang, lengths)
        got = _no_alloc(lib, capi, ang, lengths)
        assert torch.isfinite(got).all()
        err = (got.double() - ref.double()).view(B, -1, 3).norm(dim=-1).max().item()
        assert err <= COORD_TOL_F32, err


def test_no_alloc_rejects_sizes_beyond_its_scratch(built):
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    dummy = ctypes.c_void_p(256)
    # 8192 chains of 1000 residues need far more than the 4 MiB scratch; nothing is launched
    assert lib.tpl_a2b_forward_f32_noalloc(dummy, dummy, dummy, 8192, 1000, None, None) == -9
    assert b"no-allocation" in lib.tpl_status_string(-9)
