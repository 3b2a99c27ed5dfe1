"""The no-allocation Angles2Backbone forward (tpl_a2b_forward_f32_noalloc).

It serves callers that cannot allocate device memory, such as an FFI host that
owns only the buffers it passes in, or a process whose framework has already
reserved the GPU's memory.  It keeps its scratch in a fixed array inside the
library instead of a caller workspace.  These tests drive it through the C ABI
and compare it with the workspace entry point, tpl_a2b_forward_f32.  Both run the
same kernel on the same inputs, so the outputs must be bitwise equal
(torch.equal), a stricter bar than the 1e-3 A FP32 tolerance of the other tests.
The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 4 << 20  # the fixed array's size, as documented in include/tpl_gb300.h
TPL_ERR_LENGTH = -4
TPL_ERR_TOO_LARGE = -9

# option sets: the automatic choice, warp tiles of 32 residues (the most look-back
# records per chain), one warp per chain and one CTA of four warps per chain
OPTION_SETS = {
    "default": {},
    "warp_tiles_r1": {"threads_per_cta": 1, "residues_per_thread": 1},
    "one_warp_r4": {"threads_per_cta": 32, "residues_per_thread": 4},
    "four_warps_r8": {"threads_per_cta": 4, "residues_per_thread": 8},
}


def _inputs(B, L, seed):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L)).astype(np.float32)
    lengths = rng.integers(0, L + 1, B).astype(np.int32)
    lengths[0] = L
    dev = torch.device("cuda")
    return torch.tensor(ang, device=dev), torch.tensor(lengths, device=dev)


def _opt(capi, kw):
    return ctypes.byref(capi.options(**kw)) if kw else None


def _with_workspace(lib, capi, ang, lengths, kw):
    B, _, L = ang.shape
    n = lib.tpl_a2b_workspace_bytes(B, L, _opt(capi, kw))
    ws = torch.zeros(n, dtype=torch.uint8, device=ang.device)
    out = torch.full((B, 9 * L), float("nan"), device=ang.device)
    capi.check(lib.tpl_a2b_forward_f32(ang.data_ptr(), lengths.data_ptr(), out.data_ptr(), ws.data_ptr(), n, B, L,
                                       _opt(capi, kw), capi.stream_ptr()), "tpl_a2b_forward_f32")
    torch.cuda.synchronize()
    return out


def _no_alloc(lib, capi, ang, lengths, kw):
    B, _, L = ang.shape
    out = torch.full((B, 9 * L), float("nan"), device=ang.device)
    capi.check(lib.tpl_a2b_forward_f32_noalloc(ang.data_ptr(), lengths.data_ptr(), out.data_ptr(), B, L,
                                               _opt(capi, kw), capi.stream_ptr()), "tpl_a2b_forward_f32_noalloc")
    return out


def _status(lib, capi):
    st = ctypes.c_int(123)
    capi.check(lib.tpl_a2b_noalloc_status(capi.stream_ptr(), ctypes.byref(st)), "tpl_a2b_noalloc_status")
    return st.value


def _largest_batch(lib, capi, L, kw):
    """Largest batch whose scratch fits the fixed array at stride L."""
    one = lib.tpl_a2b_workspace_bytes(1, L, _opt(capi, kw))
    two = lib.tpl_a2b_workspace_bytes(2, L, _opt(capi, kw))
    per_chain, head = two - one, 2 * one - two
    B = (SCRATCH_BYTES - head) // per_chain
    assert lib.tpl_a2b_workspace_bytes(B, L, _opt(capi, kw)) <= SCRATCH_BYTES
    assert lib.tpl_a2b_workspace_bytes(B + 1, L, _opt(capi, kw)) > SCRATCH_BYTES
    return B


@pytest.mark.parametrize("name", list(OPTION_SETS))
def test_no_alloc_matches_workspace_entry_on_two_calls(built, name):
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    kw = OPTION_SETS[name]
    # two calls in a row with different inputs: the shared scratch keeps the first
    # call's contents and is cleared by the second
    for seed, (B, L) in [(1, (64, 300)), (2, (48, 517))]:
        ang, lengths = _inputs(B, L, seed)
        ref = _with_workspace(lib, capi, ang, lengths, kw)
        got = _no_alloc(lib, capi, ang, lengths, kw)
        assert _status(lib, capi) == 0
        assert torch.isfinite(got).all()
        assert torch.equal(got, ref)


@pytest.mark.parametrize("name", list(OPTION_SETS))
def test_no_alloc_size_limit_boundary(built, name):
    """The largest batch that fits runs and matches; one more chain, or one more
    tile per chain, is refused with TPL_ERR_TOO_LARGE before anything is enqueued."""
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    kw = OPTION_SETS[name]
    L = 640
    B = _largest_batch(lib, capi, L, kw)
    ang, lengths = _inputs(B, L, 7)
    ref = _with_workspace(lib, capi, ang, lengths, kw)
    got = _no_alloc(lib, capi, ang, lengths, kw)
    assert _status(lib, capi) == 0
    assert torch.equal(got, ref)

    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    tile = lib.tpl_a2b_workspace_bytes(1, L + 1, _opt(capi, kw)) - lib.tpl_a2b_workspace_bytes(1, L, _opt(capi, kw))
    assert tile > 0  # L is a multiple of every tile, so L + 1 starts a new record per chain
    assert lib.tpl_a2b_forward_f32_noalloc(dummy, dummy, dummy, B + 1, L, _opt(capi, kw), None) == TPL_ERR_TOO_LARGE
    assert lib.tpl_a2b_forward_f32_noalloc(dummy, dummy, dummy, B, L + 1, _opt(capi, kw), None) == TPL_ERR_TOO_LARGE
    assert b"no-allocation" in lib.tpl_status_string(TPL_ERR_TOO_LARGE)


def test_no_alloc_reports_device_detected_errors(built):
    """A length past max_len is recorded on the device; the status reader returns
    it once, and the next clean call reports success."""
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    B, L = 32, 200
    ang, lengths = _inputs(B, L, 3)
    bad = lengths.clone()
    bad[5] = L + 1  # the kernels clamp it to L and record TPL_ERR_LENGTH
    _no_alloc(lib, capi, ang, bad, {})
    assert _status(lib, capi) == TPL_ERR_LENGTH
    assert _status(lib, capi) == 0  # reading clears the record
    ref = _with_workspace(lib, capi, ang, lengths, {})
    got = _no_alloc(lib, capi, ang, lengths, {})
    assert _status(lib, capi) == 0
    assert torch.equal(got, ref)
