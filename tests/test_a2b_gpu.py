"""Angles2Backbone on the GPU against the oracle (FP64 restatement of the
reference CPU path, itself pinned to the reference in test_oracle_pin.py).

Tolerances (stated here, used below):
  * FP64 plain form vs oracle: coordinates 1e-9 A, gradients 1e-9 x max|grad|.
  * FP32 batched form vs oracle on the same float32 angles: coordinates 1e-3 A
    (the target for chains up to 1000 residues), gradients 1e-4 x max|grad|.
"""
import ctypes

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

COORD_TOL_F32 = 1e-3
GRAD_TOL_F32 = 1e-4
COORD_TOL_F64 = 1e-9
GRAD_TOL_F64 = 1e-9


@pytest.fixture(scope="module")
def rm(built):
    from torchproteinlibrary_gb300 import load_extension
    m = load_extension("_ReducedModel")
    m.set_options(0, 0, 0, 0)
    yield m
    m.set_options(0, 0, 0, 0)


def make_case(B, L, seed, lengths=None, omega="pi"):
    rng = np.random.default_rng(seed)
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    if omega == "pi":
        ang[:, 2] = np.pi
    else:
        ang[:, 2] = rng.normal(np.pi, 0.05, (B, L))
    if lengths is None:
        lengths = rng.integers(0, L + 1, B)
    lengths = np.asarray(lengths, dtype=np.int32)
    g = rng.standard_normal((B, 9 * L))
    return ang, lengths, g


def run_gpu(rm, ang, lengths, g, dtype):
    dev = torch.device("cuda")
    a = torch.tensor(ang, dtype=dtype, device=dev)
    ln = torch.tensor(lengths, dtype=torch.int32, device=dev)
    B, _, L = a.shape
    ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
    coords = torch.full((B, 9 * L), float("nan"), dtype=dtype, device=dev)
    rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
    gi = torch.full((B, 3, L), float("nan"), dtype=dtype, device=dev)
    gt = torch.tensor(g, dtype=dtype, device=dev)
    rm.Angles2BackboneGPU_backward(gi, gt, a, ln, ws, torch.empty(0, device=dev))
    assert rm.workspace_status(ws) == 0
    return coords.double().cpu().numpy(), gi.double().cpu().numpy()


def oracle_ref(ang, lengths, g, as_float32):
    a = ang.astype(np.float32).astype(np.float64) if as_float32 else ang
    c, A = oracle.a2b_forward(a, lengths)
    return c, oracle.a2b_backward(g if not as_float32 else g.astype(np.float32).astype(np.float64), a, lengths, A)


def check(got_c, got_g, ref_c, ref_g, lengths, L, ctol, gtol):
    B = len(lengths)
    for b in range(B):
        n = lengths[b]
        assert np.all(got_c[b, 9 * n:] == 0.0), "coordinates past the chain must be exactly zero"
        assert np.all(got_g[b, :, n:] == 0.0), "gradients past the chain must be exactly zero"
    d = np.abs(got_c - ref_c).reshape(B, -1, 3)
    err = np.sqrt((d ** 2).sum(-1)).max()
    assert err <= ctol, f"max coordinate error {err:.3e} A"
    scale = max(1.0, np.abs(ref_g).max())
    gerr = np.abs(got_g - ref_g).max() / scale
    assert gerr <= gtol, f"max gradient error {gerr:.3e} of max|grad|"
    return err, gerr


@pytest.mark.parametrize("B,L,seed", [(16, 50, 1), (5, 7, 2), (3, 130, 3), (9, 257, 4)])
def test_fp32_matches_oracle(rm, B, L, seed):
    ang, lengths, g = make_case(B, L, seed)
    lengths[0] = L
    c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
    rc, rg = oracle_ref(ang, lengths, g, True)
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


@pytest.mark.parametrize("B,L,seed", [(16, 50, 1), (3, 300, 5), (2, 513, 6)])
def test_fp64_plain_matches_oracle(rm, B, L, seed):
    ang, lengths, g = make_case(B, L, seed, omega="noise")
    lengths[0] = L
    c, gi = run_gpu(rm, ang, lengths, g, torch.float64)
    rc, rg = oracle_ref(ang, lengths, g, False)
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F64, GRAD_TOL_F64)


@pytest.mark.parametrize("rpt,cta", [(1, 1), (2, 1), (4, 1), (8, 1), (1, 128), (4, 128), (8, 128), (4, 32),
                                      (8, 32), (4, 4), (8, 4), (0, 0)])
def test_tile_shapes_and_lookback(rm, rpt, cta):
    """Chains of 1000 residues split into up to 32 warp tiles (R=1: 32-residue tiles)
    or CTA tiles (128 R residues, one tile at R=8), or walked in chunks of 32 R
    residues by one warp per chain (cta=32) or by the four warps of one CTA per
    chain (cta=4); all within tolerance of the oracle."""
    B, L = 6, 1000
    ang, lengths, g = make_case(B, L, 40 + rpt, lengths=[1000, 999, 129, 128, 127, 1])
    rm.set_options(rpt, 0, 0, 0, cta)
    try:
        c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
    finally:
        rm.set_options(0, 0, 0, 0)
    rc, rg = oracle_ref(ang, lengths, g, True)
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


@pytest.mark.parametrize("rpt,cta", [(4, 32), (8, 32), (4, 4), (8, 4), (4, 1), (4, 128)])
def test_angles_beyond_the_fast_sincos_range(rm, rpt, cta):
    """Angles far outside [-pi, pi] (one in eight phi and psi moved by up to 1e5 turns)
    send their four-residue groups down the rare path of the walk (sincosf instead of
    the polynomial sin/cos): inlined in most forwards, a call in the one-warp C = 4
    form.  Every scheme's forward and recomputing backward, and the backward from the
    coordinates, against the oracle on the same float32 angles."""
    B, L = 6, 600
    ang, lengths, g = make_case(B, L, 61 + rpt, lengths=[600, 599, 257, 128, 33, 1])
    rng = np.random.default_rng(7 + rpt + cta)
    pick = rng.random((B, 2, L)) < 0.125
    turns = rng.integers(-100000, 100001, (B, 2, L)) * (2 * np.pi)
    ang[:, :2] = np.where(pick, ang[:, :2] + turns, ang[:, :2])
    assert np.abs(ang).max() > 1e4
    rm.set_options(rpt, 0, 0, 0, cta)
    try:
        c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
        c2, gi2 = run_gpu_coords_backward(rm, ang, lengths, g, 4)
    finally:
        rm.set_options(0, 0, 0, 0)
    rc, rg = oracle_ref(ang, lengths, g, True)
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)
    check(c2, gi2, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


def test_fp64_carry_threshold_and_renorm_off(rm):
    """FP32 inter-tile carries (fp64_carry_min_len=-1) or a threshold of 256 keep the
    1e-3 A bound; switching the Newton-Schulz renormalisation off is an ablation
    (coherent scale drift of FP32 frames), held to 5e-3 A only."""
    B, L = 4, 600
    ang, lengths, g = make_case(B, L, 77, lengths=[600, 450, 300, 20])
    rc, rg = oracle_ref(ang, lengths, g, True)
    for carry, renorm, ctol in [(-1, 0, COORD_TOL_F32), (256, 0, COORD_TOL_F32), (0, -1, 5e-3)]:
        rm.set_options(1, carry, renorm, 0, 1)
        try:
            c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
        finally:
            rm.set_options(0, 0, 0, 0)
        check(c, gi, rc, rg, lengths, L, ctol, GRAD_TOL_F32)


@pytest.mark.parametrize("rpt", [4, 8])
def test_four_warp_fp64_carry_threshold(rm, rpt):
    """The four-warp forward with an FP64 chain-frame carry for chains of at least
    300 residues (a positive fp64_carry_min_len): chains above and below the
    threshold in one batch, coordinates within 1e-3 A of the oracle and the
    recomputing backward (which starts from the forward's recorded frames) within
    1e-4; the FP32 carry (threshold 0, the default) on the same batch for contrast.
    The FP64 carry must not be less accurate than the FP32 one: its maximum and RMS
    coordinate errors over the 1000-residue chains stay within 10 % of the FP32
    carry's (an FP64 product of chunk totals that are not renormalised drifts in
    scale, to about 1.5e-3 A at 1000 residues)."""
    B, L = 40, 1000
    lengths = [1000] * 35 + [700, 300, 299, 40, 1000]
    ang, lengths, g = make_case(B, L, 91 + rpt, lengths=lengths)
    rc, rg = oracle_ref(ang, lengths, g, True)
    errs = {}
    for carry in (300, 0):
        rm.set_options(rpt, carry, 0, 0, 4)
        try:
            c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
        finally:
            rm.set_options(0, 0, 0, 0)
        check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)
        e = np.linalg.norm((c - rc).reshape(B, -1, 3), axis=-1)[:35]
        errs[carry] = (e.max(), np.sqrt((e ** 2).mean()))
    assert errs[300][0] <= 1.1 * errs[0][0], errs
    assert errs[300][1] <= 1.1 * errs[0][1], errs


@pytest.mark.parametrize("rpt,cta", [(0, 1), (8, 32), (4, 32)])
def test_padding_nan_does_not_leak(rm, rpt, cta):
    B, L = 4, 64
    ang, lengths, g = make_case(B, L, 9, lengths=[64, 30, 1, 0])
    for b, n in enumerate(lengths):
        ang[b, :, n:] = np.nan
        g[b, 9 * n:] = np.nan
    ang[1, 2, 29] = np.nan  # omega of the last residue is never used
    rm.set_options(rpt, 0, 0, 0, cta)
    try:
        c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
    finally:
        rm.set_options(0, 0, 0, 0)
    a2 = np.nan_to_num(ang, nan=0.0)
    g2 = np.nan_to_num(g, nan=0.0)
    rc, rg = oracle_ref(a2, lengths, g2, True)
    assert np.isfinite(c).all() and np.isfinite(gi).all()
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


def test_empty_inputs(rm):
    dev = torch.device("cuda")
    for B, L in [(0, 10), (3, 0)]:
        a = torch.zeros(B, 3, L, device=dev)
        ln = torch.zeros(B, dtype=torch.int32, device=dev)
        ws = torch.zeros(max(64, rm.workspace_bytes(B, L)), dtype=torch.uint8, device=dev)
        out = torch.zeros(B, 9 * L, device=dev)
        rm.Angles2BackboneGPU_forward(a, out, ln, ws)
    c, gi = run_gpu(rm, np.zeros((3, 3, 5)), np.zeros(3, np.int32), np.ones((3, 45)), torch.float32)
    assert np.all(c == 0) and np.all(gi == 0)


def test_layer_empty_batch_and_zero_lengths(rm):
    """The float32 layer (its C++ autograd function) on an empty batch and on chains of
    length 0: empty or all-zero coordinates, and a backward that returns zeros of the
    angles' shape."""
    from torchproteinlibrary_gb300.ReducedModel import Angles2Backbone
    dev = torch.device("cuda")
    layer = Angles2Backbone()
    x = torch.zeros(0, 3, 16, device=dev, requires_grad=True)
    out = layer(x, torch.zeros(0, dtype=torch.int32, device=dev))
    assert out.shape == (0, 144)
    out.sum().backward()
    assert x.grad.shape == (0, 3, 16)
    x = torch.rand(3, 3, 16, device=dev, requires_grad=True)
    out = layer(x, torch.zeros(3, dtype=torch.int32, device=dev))
    assert torch.all(out == 0)
    out.backward(torch.ones_like(out))
    assert torch.all(x.grad == 0)


def test_errors_raise(rm):
    dev = torch.device("cuda")
    a = torch.zeros(2, 3, 8, device=dev)
    ln = torch.full((2,), 8, dtype=torch.int32, device=dev)
    out = torch.zeros(2, 72, device=dev)
    ws = torch.zeros(rm.workspace_bytes(2, 8), dtype=torch.uint8, device=dev)
    with pytest.raises(RuntimeError):
        rm.Angles2BackboneGPU_forward(a.cpu(), out.cpu(), ln.cpu(), ws.cpu())
    with pytest.raises(RuntimeError):
        rm.Angles2BackboneGPU_forward(a, out, ln.long(), ws)
    with pytest.raises(RuntimeError):
        rm.Angles2BackboneGPU_forward(a, out, ln, ws[:10])
    # a length beyond max_len is clamped on the device and reported
    bad = torch.tensor([8, 9], dtype=torch.int32, device=dev)
    rm.Angles2BackboneGPU_forward(a, out, bad, ws)
    assert rm.workspace_status(ws) == -4
    assert rm.workspace_status(ws) == 0  # reading clears it


def test_lookback_timeout_is_reported(rm, built):
    """Fault injection on the host side of the kernel: the first tile of chain 0
    never publishes, so the next tile's bounded wait runs out.  The kernel ends,
    records TPL_ERR_LOOKBACK_TIMEOUT, and the context stays usable."""
    from torchproteinlibrary_gb300 import capi
    dev = torch.device("cuda")
    B, L = 2, 300
    a = torch.rand(B, 3, L, device=dev)
    ln = torch.full((B,), L, dtype=torch.int32, device=dev)
    out = torch.zeros(B, 9 * L, device=dev)
    rm.set_options(4, 0, 0, 0, 1)  # 128-residue warp tiles: 3 tiles per chain
    try:
        ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
        ws[4 * 8:4 * 9].view(torch.int32).fill_(1)  # WsHeader.test_skip_publish
        rm.Angles2BackboneGPU_forward(a, out, ln, ws)
        assert rm.workspace_status(ws) == -6
        ws.zero_()
        rm.Angles2BackboneGPU_forward(a, out, ln, ws)
        assert rm.workspace_status(ws) == 0
    finally:
        rm.set_options(0, 0, 0, 0)
    assert torch.isfinite(out).all()


def test_c_abi_direct_matches_extension(rm, built):
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    ang, lengths, g = make_case(7, 90, 21)
    c_ext, g_ext = run_gpu(rm, ang, lengths, g, torch.float32)
    dev = torch.device("cuda")
    a = torch.tensor(ang, dtype=torch.float32, device=dev)
    ln = torch.tensor(lengths, device=dev)
    n = lib.tpl_a2b_workspace_bytes(7, 90, None)
    ws = torch.zeros(n, dtype=torch.uint8, device=dev)
    coords = torch.empty(7, 810, device=dev)
    st = capi.stream_ptr()
    capi.check(lib.tpl_a2b_forward_f32(a.data_ptr(), ln.data_ptr(), coords.data_ptr(), ws.data_ptr(), n, 7, 90,
                                       None, st))
    gi = torch.empty(7, 3, 90, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    capi.check(lib.tpl_a2b_backward_f32(gi.data_ptr(), gt.data_ptr(), a.data_ptr(), ln.data_ptr(), ws.data_ptr(), n,
                                        7, 90, None, st))
    status = ctypes.c_int(123)
    capi.check(lib.tpl_workspace_status(ws.data_ptr(), st, ctypes.byref(status)))
    assert status.value == 0
    assert np.array_equal(coords.double().cpu().numpy(), c_ext)
    assert np.array_equal(gi.double().cpu().numpy(), g_ext)


def test_autograd_layer_and_gradcheck(built):
    from torchproteinlibrary_gb300.ReducedModel import Angles2Backbone
    layer = Angles2Backbone()
    dev = torch.device("cuda")
    # reference test setup (UnitTests/ReducedModel/Angles2Backbone/test.py:72-82), here in FP64
    torch.manual_seed(0)
    x = torch.randn(8, 3, 8, dtype=torch.float64, device=dev, requires_grad=True)
    n = torch.randint(4, 8, (8,), dtype=torch.int32, device=dev)
    assert torch.autograd.gradcheck(layer, (x, n), eps=1e-6, atol=1e-6, rtol=1e-5)
    # FP32 with the reference's own tolerances
    x32 = x.detach().float().requires_grad_()
    assert torch.autograd.gradcheck(layer, (x32, n), eps=1e-3, atol=1e-2, rtol=0.01)
    with pytest.raises(RuntimeError):
        layer(x.detach().cpu(), n.cpu())


def test_cuda_graph_replay(rm):
    """Persistent launches reset their tickets/epochs themselves, so a captured
    forward+backward replays correctly without memsets."""
    dev = torch.device("cuda")
    B, L = 64, 400
    ang, lengths, g = make_case(B, L, 5)
    a = torch.tensor(ang, dtype=torch.float32, device=dev)
    ln = torch.tensor(lengths, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
    coords = torch.empty(B, 9 * L, device=dev)
    gi = torch.empty(B, 3, L, device=dev)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
        rm.Angles2BackboneGPU_backward(gi, gt, a, ln, ws, torch.empty(0, device=dev))
    torch.cuda.current_stream().wait_stream(s)
    ref_c, ref_g = coords.clone(), gi.clone()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
        rm.Angles2BackboneGPU_backward(gi, gt, a, ln, ws, torch.empty(0, device=dev))
    for _ in range(3):
        coords.zero_(); gi.zero_()
        graph.replay()
        torch.cuda.synchronize()
        assert torch.equal(coords, ref_c) and torch.equal(gi, ref_g)
    assert rm.workspace_status(ws) == 0


def _ragged_config3(seed=1003):
    rng = np.random.default_rng(seed)
    B, L = 1024, 700
    lengths = rng.integers(20, 701, B).astype(np.int32)
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    ang[:, 2] = rng.normal(np.pi, 0.05, (B, L))
    for b, n in enumerate(lengths):
        ang[b, :, n:] = 0.0
    g = rng.standard_normal((B, 9 * L))
    return ang, lengths, g


def test_config3_full_size_against_fp64_form(rm):
    """1024 ragged chains of 20..700 residues: the FP32 batched path agrees with the
    FP64 plain form (pinned to the oracle above) within the stated tolerances, and
    a few chains are checked against the CPU oracle directly."""
    ang, lengths, g = _ragged_config3()
    c32, g32 = run_gpu(rm, ang, lengths, g.astype(np.float32).astype(np.float64), torch.float32)
    a32 = ang.astype(np.float32).astype(np.float64)
    c64, g64 = run_gpu(rm, a32, lengths, g.astype(np.float32).astype(np.float64), torch.float64)
    check(c32, g32, c64, g64, lengths, 700, COORD_TOL_F32, GRAD_TOL_F32)
    idx = np.argsort(lengths)[-2:]
    rc, rg = oracle_ref(ang[idx], lengths[idx], g[idx], True)
    check(c64[idx], g64[idx], rc, rg, lengths[idx], 700, COORD_TOL_F64, GRAD_TOL_F64)


@pytest.mark.parametrize("cta", [32, 4])
@pytest.mark.parametrize("rpt", [4, 8])
@pytest.mark.parametrize("L", [1001, 258, 1000, 1400])
def test_one_warp_per_chain_ragged_and_unaligned(rm, rpt, L, cta):
    """One warp per chain (cta=32) or one CTA of four warps per chain (cta=4) over
    ragged lengths at chunk edges, with rows that are not 16-byte aligned (L % 4 != 0:
    scalar loads and stores) and aligned (float4).  L = 1400 is 11 chunks of 128
    residues (4 per lane) or 6 of 256: the four-warp handoff goes round its ring
    more than once."""
    lens = [L, L - 1, 257, 256, 255, 129, 128, 127, 1, 0]
    ang, lengths, g = make_case(len(lens), L, 300 + L + rpt, lengths=lens)
    rm.set_options(rpt, 0, 0, 0, cta)
    try:
        c, gi = run_gpu(rm, ang, lengths, g, torch.float32)
    finally:
        rm.set_options(0, 0, 0, 0)
    rc, rg = oracle_ref(ang, lengths, g, True)
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


def test_one_warp_per_chain_mixed_chunk_sizes_through_c_abi(built):
    """The backward starts its chunks from frames the forward recorded every 128
    residues, so a forward with 256-residue chunks and a backward with 128-residue
    chunks (and the reverse) agree with the oracle, whether one warp or the four
    warps of one CTA walked the chain in the forward."""
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    dev = torch.device("cuda")
    B, L = 8, 640
    ang, lengths, g = make_case(B, L, 91, lengths=[640, 639, 600, 384, 257, 128, 3, 0])
    rc, rg = oracle_ref(ang, lengths, g, True)
    a = torch.tensor(ang, dtype=torch.float32, device=dev)
    ln = torch.tensor(lengths, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    for cf, tf, cb in [(8, 32, 4), (4, 32, 8), (8, 4, 4), (4, 4, 8)]:
        of, ob = capi.options(residues_per_thread=cf, threads_per_cta=tf), \
            capi.options(residues_per_thread=cb, threads_per_cta=32)
        n = max(lib.tpl_a2b_workspace_bytes(B, L, ctypes.byref(of)), lib.tpl_a2b_workspace_bytes(B, L, ctypes.byref(ob)))
        ws = torch.zeros(n, dtype=torch.uint8, device=dev)
        coords = torch.full((B, 9 * L), float("nan"), device=dev)
        gi = torch.full((B, 3, L), float("nan"), device=dev)
        st = capi.stream_ptr()
        capi.check(lib.tpl_a2b_forward_f32(a.data_ptr(), ln.data_ptr(), coords.data_ptr(), ws.data_ptr(), n, B, L,
                                           ctypes.byref(of), st), "forward")
        capi.check(lib.tpl_a2b_backward_f32(gi.data_ptr(), gt.data_ptr(), a.data_ptr(), ln.data_ptr(), ws.data_ptr(),
                                            n, B, L, ctypes.byref(ob), st), "backward")
        torch.cuda.synchronize()
        check(coords.double().cpu().numpy(), gi.double().cpu().numpy(), rc, rg, lengths, L, COORD_TOL_F32,
              GRAD_TOL_F32)


@pytest.mark.parametrize("cta", [32, 4])
def test_one_warp_per_chain_graph_replay(rm, cta):
    dev = torch.device("cuda")
    B, L = 96, 500
    ang, lengths, g = make_case(B, L, 17)
    a = torch.tensor(ang, dtype=torch.float32, device=dev)
    ln = torch.tensor(lengths, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    rm.set_options(8, 0, 0, 0, cta)
    try:
        ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
        coords = torch.empty(B, 9 * L, device=dev)
        gi = torch.empty(B, 3, L, device=dev)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
            rm.Angles2BackboneGPU_backward(gi, gt, a, ln, ws, torch.empty(0, device=dev))
        torch.cuda.current_stream().wait_stream(s)
        ref_c, ref_g = coords.clone(), gi.clone()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
            rm.Angles2BackboneGPU_backward(gi, gt, a, ln, ws, torch.empty(0, device=dev))
        for _ in range(2):
            coords.zero_(); gi.zero_()
            graph.replay()
            torch.cuda.synchronize()
            assert torch.equal(coords, ref_c) and torch.equal(gi, ref_g)
        assert rm.workspace_status(ws) == 0
    finally:
        rm.set_options(0, 0, 0, 0)
    rc, rg = oracle_ref(ang, lengths, g, True)
    check(ref_c.double().cpu().numpy(), ref_g.double().cpu().numpy(), rc, rg, lengths, L, COORD_TOL_F32,
          GRAD_TOL_F32)


def test_sincos_error_bound(built):
    """The kernels' own sin/cos (Cody-Waite reduction by pi/2, Taylor series)
    against FP64: within 2.5e-7 absolute on [-pi, pi] and up to |a| = 1e4, and
    within 3e-7 of unit norm."""
    from torchproteinlibrary_gb300 import capi
    lib = capi.lib()
    dev = torch.device("cuda")
    rng = np.random.default_rng(12)
    x = np.concatenate([rng.uniform(-np.pi, np.pi, 200000), rng.uniform(-1e4, 1e4, 50000),
                        np.linspace(-np.pi, np.pi, 4097), np.array([0.0, -0.0, np.pi / 4, -np.pi / 4, np.pi / 2])])
    x = x.astype(np.float32)
    a = torch.tensor(x, device=dev)
    s = torch.empty_like(a)
    c = torch.empty_like(a)
    capi.check(lib.tpl_sincos_f32(a.data_ptr(), s.data_ptr(), c.data_ptr(), a.numel(), capi.stream_ptr()), "sincos")
    torch.cuda.synchronize()
    xs = x.astype(np.float64)
    sv, cv = s.double().cpu().numpy(), c.double().cpu().numpy()
    assert np.abs(sv - np.sin(xs)).max() <= 2.5e-7
    assert np.abs(cv - np.cos(xs)).max() <= 2.5e-7
    assert np.abs(sv * sv + cv * cv - 1.0).max() <= 3e-7


def run_gpu_coords_backward(rm, ang, lengths, g, rpt, buffers=0, scheme=0):
    """Forward with the current options, then the backward from its coordinates."""
    dev = torch.device("cuda")
    a = torch.tensor(ang, dtype=torch.float32, device=dev)
    ln = torch.tensor(lengths, dtype=torch.int32, device=dev)
    B, _, L = a.shape
    ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
    coords = torch.full((B, 9 * L), float("nan"), device=dev)
    rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
    gi = torch.full((B, 3, L), float("nan"), device=dev)
    rm.set_backward_options(rpt, buffers, scheme)
    try:
        rm.Angles2BackboneGPU_backward_coords(gi, torch.tensor(g, dtype=torch.float32, device=dev), coords, ln, ws)
    finally:
        rm.set_backward_options(0)
    assert rm.workspace_status(ws) == 0
    return coords.double().cpu().numpy(), gi.double().cpu().numpy()


@pytest.mark.parametrize("scheme", [32, 4, 0])
@pytest.mark.parametrize("rpt,buffers", [(4, 1), (4, 2), (8, 1)])
@pytest.mark.parametrize("L", [1000, 1001, 258, 1400])
def test_backward_from_coordinates_matches_oracle(rm, rpt, buffers, L, scheme):
    """The float32 backward from the forward's output coordinates (bulk-copied chunk
    rows when L % 4 == 0, single or double buffered; plain loads otherwise), by one
    warp per chain (scheme 32), by the four warps of one CTA per chain with the
    carried sums handed round them (scheme 4) or as chosen from the length (0),
    against the oracle."""
    lens = [L, L - 1, 257, 256, 255, 129, 128, 127, 2, 1, 0]
    ang, lengths, g = make_case(len(lens), L, 500 + L + rpt, lengths=lens)
    c, gi = run_gpu_coords_backward(rm, ang, lengths, g, rpt, buffers, scheme)
    rc, rg = oracle_ref(ang, lengths, g, True)
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


def test_backward_from_coordinates_ignores_padding(rm):
    B, L = 4, 64
    ang, lengths, g = make_case(B, L, 19, lengths=[64, 30, 1, 0])
    for b, n in enumerate(lengths):
        g[b, 9 * n:] = np.nan
    c, gi = run_gpu_coords_backward(rm, ang, lengths, g, 4)
    rc, rg = oracle_ref(ang, lengths, np.nan_to_num(g, nan=0.0), True)
    assert np.isfinite(gi).all()
    check(c, gi, rc, rg, lengths, L, COORD_TOL_F32, GRAD_TOL_F32)


def test_backward_from_coordinates_c_abi_and_layer(built):
    """Through the C ABI (status-word workspace only) and through the autograd
    layer, which saves its output coordinates for the backward; both agree with the
    backward that recomputes the chain from the angles."""
    from torchproteinlibrary_gb300 import capi
    from torchproteinlibrary_gb300.ReducedModel import Angles2Backbone
    from torchproteinlibrary_gb300.ReducedModel.Angles2Backbone.Angles2Backbone import Angles2BackboneGPUFunction
    lib = capi.lib()
    dev = torch.device("cuda")
    B, L = 12, 300
    ang, lengths, g = make_case(B, L, 23)
    lengths[0] = L
    a = torch.tensor(ang, dtype=torch.float32, device=dev)
    ln = torch.tensor(lengths, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    layer = Angles2Backbone()
    grads = []
    for from_coords in (True, False):
        Angles2BackboneGPUFunction.backward_from_coords = from_coords
        try:
            x = a.clone().requires_grad_()
            out = layer(x, ln)
            out.backward(gt)
            grads.append(x.grad.clone())
        finally:
            Angles2BackboneGPUFunction.backward_from_coords = True
    scale = grads[1].abs().max().item()
    assert (grads[0] - grads[1]).abs().max().item() <= GRAD_TOL_F32 * scale
    # C ABI: 64-byte status workspace
    ws = torch.zeros(64, dtype=torch.uint8, device=dev)
    coords = layer(a, ln).detach().contiguous()
    gi = torch.full((B, 3, L), float("nan"), device=dev)
    capi.check(lib.tpl_a2b_backward_coords_f32(gi.data_ptr(), gt.data_ptr(), coords.data_ptr(), ln.data_ptr(),
                                               ws.data_ptr(), 64, B, L, None, capi.stream_ptr()), "backward_coords")
    torch.cuda.synchronize()
    assert (gi - grads[1]).abs().max().item() <= GRAD_TOL_F32 * scale
    assert lib.tpl_a2b_backward_coords_f32(gi.data_ptr(), gt.data_ptr(), coords.data_ptr(), ln.data_ptr(),
                                           ws.data_ptr(), 16, B, L, None, capi.stream_ptr()) == -2


def _bond_angle(p, q, r):
    """Angle at q between q->p and q->r (float64 tensors [..., 3])."""
    u, v = p - q, r - q
    c = (u * v).sum(-1) / (u.norm(dim=-1) * v.norm(dim=-1))
    return torch.acos(c.clamp(-1.0, 1.0))


def test_full_size_geometry_and_fp64_slice(rm):
    """The measured workload, 4096 chains x 1000 residues in FP32 with the default
    (automatic) scheme and the float32 layer's backward: every bond length and
    bond angle of every residue equals the joint geometry (size-independent
    invariants; the reference values are read off the FP64 oracle), and 32 chains
    match the FP64 form within the FP32 tolerances."""
    dev = torch.device("cuda")
    B, L = 4096, 1000
    rng = np.random.default_rng(1005)
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L)).astype(np.float32)
    ang[:, 2] = np.float32(np.pi)
    lengths = np.full(B, L, np.int32)
    up = rng.standard_normal((B, 9 * L)).astype(np.float32)
    a = torch.tensor(ang, device=dev)
    ln = torch.tensor(lengths, device=dev)
    u = torch.tensor(up, device=dev)
    ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
    coords = torch.empty(B, 9 * L, device=dev)
    gi = torch.empty(B, 3, L, device=dev)
    rm.Angles2BackboneGPU_forward(a, coords, ln, ws)
    rm.Angles2BackboneGPU_backward_coords(gi, u, coords, ln, ws)
    assert rm.workspace_status(ws) == 0
    x = coords.double().view(B, L, 3, 3)
    N, CA, C = x[:, :, 0], x[:, :, 1], x[:, :, 2]
    # reference geometry from the FP64 oracle on a short chain
    rc, _ = oracle.a2b_forward(ang[:1, :, :8].astype(np.float64), np.array([8], np.int32))
    r = torch.tensor(rc, dtype=torch.float64).view(8, 3, 3)
    rN, rCA, rC = r[:, 0], r[:, 1], r[:, 2]
    bonds = [((CA - N).norm(dim=-1), (rCA - rN).norm(dim=-1)[0]),
             ((C - CA).norm(dim=-1), (rC - rCA).norm(dim=-1)[0]),
             ((N[:, 1:] - C[:, :-1]).norm(dim=-1), (rN[1] - rC[0]).norm())]
    for got, want in bonds:
        assert (got - float(want)).abs().max().item() <= 1e-4
    angles = [(_bond_angle(N, CA, C), _bond_angle(rN, rCA, rC)[0]),
              (_bond_angle(CA[:, :-1], C[:, :-1], N[:, 1:]), _bond_angle(rCA[0], rC[0], rN[1])),
              (_bond_angle(C[:, :-1], N[:, 1:], CA[:, 1:]), _bond_angle(rC[0], rN[1], rCA[1]))]
    for got, want in angles:
        assert (got - float(want)).abs().max().item() <= 1e-4
    # 32 chains against the FP64 form on the same float32 angles
    n = 32
    a64 = a[:n].double().contiguous()
    c64 = torch.empty(n, 9 * L, dtype=torch.float64, device=dev)
    g64 = torch.empty(n, 3, L, dtype=torch.float64, device=dev)
    ws64 = torch.zeros(rm.workspace_bytes(n, L), dtype=torch.uint8, device=dev)
    rm.Angles2BackboneGPU_forward(a64, c64, ln[:n].contiguous(), ws64)
    rm.Angles2BackboneGPU_backward(g64, u[:n].double().contiguous(), a64, ln[:n].contiguous(), ws64,
                                   torch.empty(0, device=dev))
    check(coords[:n].double().cpu().numpy(), gi[:n].double().cpu().numpy(), c64.cpu().numpy(),
          g64.cpu().numpy(), lengths[:n], L, COORD_TOL_F32, GRAD_TOL_F32)


def test_config1_exact_shape_fp64_and_fp32(rm):
    """The reference's CPU configuration exactly: 32 chains of 64 residues (lengths all
    64), phi, psi ~ U[-pi, pi), omega = pi, float64, upstream gradient ~ N(0, 1).  The
    plain FP64 form matches the oracle to 1e-9 A and 1e-9 of the largest gradient
    entry; the batched FP32 path to 1e-3 A and 1e-4 of the largest entry.  omega of
    the last residue is compared too: the oracle returns 0 there, as this build does."""
    rng = np.random.default_rng(1001)
    B, L = 32, 64
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    ang[:, 2] = np.pi
    lengths = np.full(B, L, dtype=np.int32)
    up = rng.standard_normal((B, 9 * L))
    rc, A = oracle.a2b_forward(ang, lengths)
    rg = oracle.a2b_backward(up, ang, lengths, A)
    dev = torch.device("cuda")
    ln = torch.tensor(lengths, device=dev)
    for dt, ctol, gtol in ((torch.float64, 1e-9, 1e-9), (torch.float32, 1e-3, 1e-4)):
        a = torch.tensor(ang, dtype=dt, device=dev)
        c = torch.empty(B, 9 * L, dtype=dt, device=dev)
        g = torch.empty(B, 3, L, dtype=dt, device=dev)
        ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
        rm.Angles2BackboneGPU_forward(a, c, ln, ws)
        rm.Angles2BackboneGPU_backward(g, torch.tensor(up, dtype=dt, device=dev), a, ln, ws,
                                       torch.empty(0, device=dev))
        cerr = (c.double().cpu().numpy() - rc).reshape(B, -1, 3)
        assert np.linalg.norm(cerr, axis=-1).max() <= ctol
        assert np.abs(g.double().cpu().numpy() - rg).max() <= gtol * np.abs(rg).max()


def test_layer_runs_the_tuned_options(rm):
    """The float32 layer asks the autotuner for its shape's options (the table shipped
    for this GPU) and passes them to the kernels: its output equals the extension's
    with those options given explicitly, bit for bit, and the backward matches too."""
    from torchproteinlibrary_gb300 import autotune
    from torchproteinlibrary_gb300.ReducedModel import Angles2Backbone
    dev = torch.device("cuda")
    B, L = 2048, 256
    tuned = autotune.options_for(dev, B, L)
    if tuned is None:
        pytest.skip(f"no tuned table for {torch.cuda.get_device_name(dev)}")
    (rpt, cta), bwd = tuned
    ang, lengths, g = make_case(B, L, 5)
    a = torch.tensor(ang, dtype=torch.float32, device=dev, requires_grad=True)
    ln = torch.tensor(lengths, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    c = Angles2Backbone()(a, ln)
    c.backward(gt)
    ws = torch.zeros(rm.workspace_bytes(B, L, rpt, cta), dtype=torch.uint8, device=dev)
    c2 = torch.empty_like(c)
    rm.Angles2BackboneGPU_forward(a.detach(), c2, ln, ws, rpt, cta)
    g2 = torch.empty_like(a)
    rm.Angles2BackboneGPU_backward_coords(g2, gt, c2, ln, ws, *bwd)
    assert torch.equal(c.detach(), c2)
    assert torch.equal(a.grad, g2)


def test_layer_uses_cpp_autograd_function(rm):
    """The float32 layer records the extension's C++ autograd node (no Python frame
    in the backward); float64 and the recomputing backward keep the Python function.
    Both float32 routes give the same coordinates and the same gradient within the
    float32 tolerance."""
    from torchproteinlibrary_gb300.ReducedModel import Angles2Backbone
    from torchproteinlibrary_gb300.ReducedModel.Angles2Backbone.Angles2Backbone import Angles2BackboneGPUFunction
    dev = torch.device("cuda")
    B, L = 6, 90
    ang, lengths, g = make_case(B, L, 41)
    ln = torch.tensor(lengths, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    layer = Angles2Backbone()
    x = torch.tensor(ang, dtype=torch.float32, device=dev, requires_grad=True)
    out = layer(x, ln)
    assert "Angles2BackboneAutograd" in out.grad_fn.name()
    out.backward(gt)
    Angles2BackboneGPUFunction.backward_from_coords = False
    try:
        x2 = torch.tensor(ang, dtype=torch.float32, device=dev, requires_grad=True)
        out2 = layer(x2, ln)
        assert "Angles2BackboneGPUFunction" in out2.grad_fn.name()
        out2.backward(gt)
    finally:
        Angles2BackboneGPUFunction.backward_from_coords = True
    assert torch.equal(out.detach(), out2.detach())
    scale = x2.grad.abs().max().item()
    assert (x.grad - x2.grad).abs().max().item() <= GRAD_TOL_F32 * scale
    x64 = torch.tensor(ang, dtype=torch.float64, device=dev, requires_grad=True)
    assert "Angles2BackboneGPUFunction" in layer(x64, ln).grad_fn.name()


def test_layer_on_two_streams_concurrently(rm):
    """The float32 layer keeps one shared workspace per (device, stream, shape): two
    streams running forward and backward of the same shape at the same time get
    their own, and give exactly the results of the same calls run one after the
    other on the default stream (the recomputing backward too, whose workspace is
    per call)."""
    from torchproteinlibrary_gb300.ReducedModel import Angles2Backbone
    from torchproteinlibrary_gb300.ReducedModel.Angles2Backbone.Angles2Backbone import Angles2BackboneGPUFunction
    dev = torch.device("cuda")
    B, L = 512, 300
    layer = Angles2Backbone()
    cases = [make_case(B, L, 71 + i) for i in range(2)]
    ln = [torch.tensor(c[1], device=dev) for c in cases]
    gt = [torch.tensor(c[2], dtype=torch.float32, device=dev) for c in cases]
    for from_coords in (True, False):
        Angles2BackboneGPUFunction.backward_from_coords = from_coords
        try:
            ref = []
            for i, c in enumerate(cases):
                x = torch.tensor(c[0], dtype=torch.float32, device=dev, requires_grad=True)
                out = layer(x, ln[i])
                out.backward(gt[i])
                ref.append((out.detach().clone(), x.grad.clone()))
            xs = [torch.tensor(c[0], dtype=torch.float32, device=dev, requires_grad=True) for c in cases]
            streams = [torch.cuda.Stream() for _ in cases]
            outs = [None, None]
            for s in streams:
                s.wait_stream(torch.cuda.current_stream())
            for i, s in enumerate(streams):
                with torch.cuda.stream(s):
                    outs[i] = layer(xs[i], ln[i])
                    outs[i].backward(gt[i])
            for s in streams:
                torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
        finally:
            Angles2BackboneGPUFunction.backward_from_coords = True
        for i in range(2):
            assert torch.equal(outs[i].detach(), ref[i][0])
            assert torch.equal(xs[i].grad, ref[i][1])
