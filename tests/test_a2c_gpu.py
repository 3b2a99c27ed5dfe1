"""Angles2Coords on the GPU against the oracle and the reference's golden fixtures.

Tolerances (stated here, used below):
  * FP64 kernels vs oracle / golden: coordinates 1e-9 A, gradients 1e-9 x max|grad|.
  * FP32 kernels vs oracle on the same float32 angles: coordinates 1e-3 A,
    gradients 1e-4 x max|grad|.
Names and atom counts are compared bit-exactly.
"""
import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
AA = "ACDEFGHIKLMNPQRSTVWY"
COORD_TOL_F32, GRAD_TOL_F32 = 1e-3, 1e-4
COORD_TOL_F64, GRAD_TOL_F64 = 1e-9, 1e-9


@pytest.fixture(scope="module")
def fm(built):
    from torchproteinlibrary_gb300 import load_extension
    return load_extension("_FullAtomModel")


def run_gpu(fm, ang, seqs, g, dtype, from_coords=False):
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords import convertStringList
    dev = torch.device("cuda")
    a = torch.tensor(ang, dtype=dtype, device=dev)
    seq = convertStringList(seqs).to(dev)
    na = [fm.getSeqNumAtoms(s) for s in seqs]
    maxA = max(na) if na else 0
    B = len(seqs)
    coords = torch.full((B, 3 * maxA), float("nan"), dtype=dtype, device=dev)
    rn = torch.full((B, maxA, 4), 255, dtype=torch.uint8, device=dev)
    an = torch.full((B, maxA, 4), 255, dtype=torch.uint8, device=dev)
    fm.Angles2Coords_forward(seq, a, coords, rn, an)
    gi = torch.full_like(a, float("nan"))
    gt = torch.tensor(g, dtype=dtype, device=dev) if g is not None else torch.zeros_like(coords)
    if from_coords:
        fm.Angles2Coords_backward_coords(gt, gi, seq, coords)
    else:
        fm.Angles2Coords_backward(gt, gi, seq, a)
    assert fm.workspace_status(0) == 0
    return (coords.double().cpu().numpy(), rn.cpu().numpy(), an.cpu().numpy(), np.array(na, np.int32),
            gi.double().cpu().numpy())


def check(c, gi, rc, rg, na, ctol, gtol):
    for b, n in enumerate(na):
        assert np.all(c[b, 3 * n:] == 0.0)
    d = np.sqrt(((c - rc).reshape(len(na), -1, 3) ** 2).sum(-1)).max() if c.size else 0.0
    assert d <= ctol, f"max coordinate error {d:.3e} A"
    scale = max(1.0, np.abs(rg).max())
    ge = np.abs(gi - rg).max() / scale
    assert ge <= gtol, f"max gradient error {ge:.3e} of max|grad|"
    return d, ge


def test_golden_fp64(fm):
    d = np.load(os.path.join(GOLD, "a2c_ref.npz"))
    seqs = [str(s) for s in d["sequences"]]
    c, rn, an, na, gi = run_gpu(fm, d["angles"], seqs, d["grad_coords"], torch.float64)
    np.testing.assert_array_equal(na, d["num_atoms"])
    np.testing.assert_array_equal(rn, d["res_names"])
    np.testing.assert_array_equal(an, d["atom_names"])
    check(c, gi, d["coords"], d["grad_angles"], na, COORD_TOL_F64, GRAD_TOL_F64)


@pytest.mark.parametrize("dtype,threads,tree", [(torch.float32, 0, False), (torch.float32, 0, True),
                                                (torch.float32, 4, False), (torch.float32, 8, False),
                                                (torch.float32, 128, True), (torch.float32, 256, True),
                                                (torch.float32, 512, True), (torch.float64, 0, False)])
def test_random_batch_matches_oracle(fm, dtype, threads, tree):
    """Forward and the reference-signature backward against the oracle.  float32:
    Angles2Coords_backward recomputes the coordinates and runs the backward from them,
    or (tree = True) rebuilds the tree per joint; float64 always rebuilds it."""
    rng = np.random.default_rng(31)
    seqs = ["".join(rng.choice(list(AA), rng.integers(1, 300))) for _ in range(7)] + ["G", "P", "W", AA]
    L = 300
    ang = rng.uniform(-np.pi, np.pi, (len(seqs), 8, L))
    ang[:, 2] = rng.normal(np.pi, 0.05, (len(seqs), L))
    rc, rrn, ran, na = oracle.a2c_forward(ang.astype(np.float32).astype(np.float64) if dtype == torch.float32 else ang,
                                          seqs)
    g = rng.standard_normal(rc.shape)
    for b, n in enumerate(na):
        g[b, 3 * n:] = 0
    if dtype == torch.float32:
        g = g.astype(np.float32).astype(np.float64)
        a_ref = ang.astype(np.float32).astype(np.float64)
    else:
        a_ref = ang
    rg = oracle.a2c_backward(g, a_ref, seqs)
    fm.set_options(threads)
    fm.set_backward_tree(tree)
    try:
        c, rn, an, na2, gi = run_gpu(fm, ang, seqs, g, dtype)
    finally:
        fm.set_options(0)
        fm.set_backward_tree(False)
    np.testing.assert_array_equal(rn, rrn)
    np.testing.assert_array_equal(an, ran)
    tol = (COORD_TOL_F32, GRAD_TOL_F32) if dtype == torch.float32 else (COORD_TOL_F64, GRAD_TOL_F64)
    check(c, gi, rc, rg, na, *tol)
    # padding of the angle tensor past each chain gets zero gradient
    for b, s in enumerate(seqs):
        assert np.all(gi[b, :, len(s):] == 0)


def test_config2_fd_check(fm):
    """Full-atom config: 64 chains of 150 random residues, FP64, omega = pi; gradient
    of 16 random angle entries per chain against central differences (h = 1e-6) of
    the GPU forward."""
    rng = np.random.default_rng(1002)
    B, L = 64, 150
    seqs = ["".join(rng.choice(list(AA), L)) for _ in range(B)]
    ang = rng.uniform(-np.pi, np.pi, (B, 8, L))
    ang[:, 2] = np.pi
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords import convertStringList
    dev = torch.device("cuda")
    c, rn, an, na, _ = run_gpu(fm, ang, seqs, None, torch.float64)
    g = rng.standard_normal(c.shape)
    _, _, _, _, gi = run_gpu(fm, ang, seqs, g, torch.float64)
    # oracle on a few chains
    idx = [0, 17, 63]
    rc, _, _, _ = oracle.a2c_forward(ang[idx], [seqs[i] for i in idx])
    rg = oracle.a2c_backward(g[idx][:, :rc.shape[1]], ang[idx], [seqs[i] for i in idx])
    check(c[idx][:, :rc.shape[1]], gi[idx], rc, rg, na[idx], COORD_TOL_F64, GRAD_TOL_F64)
    # central differences, all chains at once: perturb entry (b, k_b, j_b) of every chain
    seq = convertStringList(seqs).to(dev)
    maxA = int(na.max())
    gt = torch.tensor(g, dtype=torch.float64, device=dev)

    def forward(a_np):
        a = torch.tensor(a_np, dtype=torch.float64, device=dev)
        out = torch.empty(B, 3 * maxA, dtype=torch.float64, device=dev)
        e = torch.empty(0, dtype=torch.uint8, device=dev)
        fm.Angles2Coords_forward(seq, a, out, e, e)
        return (out * gt).sum(1).cpu().numpy()

    h = 1e-6
    worst = 0.0
    for _ in range(16):
        k = rng.integers(0, 8, B)
        j = rng.integers(0, L, B)
        ap = ang.copy(); am = ang.copy()
        ap[np.arange(B), k, j] += h
        am[np.arange(B), k, j] -= h
        fd = (forward(ap) - forward(am)) / (2 * h)
        an_ = gi[np.arange(B), k, j]
        worst = max(worst, float((np.abs(fd - an_) / np.maximum(1.0, np.abs(fd))).max()))
    assert worst < 1e-5, worst


def test_backbone_matches_angles2backbone(fm, built):
    """Reference self-consistency test (UnitTests/ReducedModel/Angles2Backbone/test.py:32-70):
    all-Gly chains through Angles2Coords give the same N, CA, C as Angles2Backbone."""
    from torchproteinlibrary_gb300 import load_extension
    rm = load_extension("_ReducedModel")
    dev = torch.device("cuda")
    rng = np.random.default_rng(5)
    B, L = 16, 32
    lengths = rng.integers(L // 2, L, B).astype(np.int32)
    # FP64: identical up to rounding.  FP32: the reference's criterion (mean error
    # below 5e-6 A, assertAlmostEqual(places=5)) plus a 1e-4 A bound on the maximum.
    for dtype, tol in [(torch.float64, 1e-10), (torch.float32, 1e-4)]:
        bb = rng.standard_normal((B, 3, L))
        a = torch.tensor(bb, dtype=dtype, device=dev)
        ws = torch.zeros(rm.workspace_bytes(B, L), dtype=torch.uint8, device=dev)
        cb = torch.empty(B, 9 * L, dtype=dtype, device=dev)
        rm.Angles2BackboneGPU_forward(a, cb, torch.tensor(lengths, device=dev), ws)
        fa = np.zeros((B, 8, L))
        fa[:, :3] = bb
        seqs = ["G" * n for n in lengths]
        c, rn, an, na, _ = run_gpu(fm, fa, seqs, None, dtype)
        cbb = cb.double().cpu().numpy()
        err, tot, cnt = 0.0, 0.0, 0
        for b in range(B):
            n = lengths[b]
            x = c[b, :3 * 4 * n].reshape(n, 4, 3)[:, :3].reshape(-1, 3)  # N, CA, C of each Gly
            d = np.linalg.norm(x - cbb[b, :9 * n].reshape(-1, 3), axis=1)
            err = max(err, d.max())
            tot += d.sum()
            cnt += d.size
        assert err <= tol, (dtype, err)
        assert tot / cnt < 5e-6, (dtype, tot / cnt)


def test_edge_cases(fm):
    dev = torch.device("cuda")
    seqs = ["", "G", "P", "W", "GP"]
    rng = np.random.default_rng(3)
    ang = rng.uniform(-np.pi, np.pi, (len(seqs), 8, 4))
    rc, rrn, ran, na = oracle.a2c_forward(ang, seqs)
    g = rng.standard_normal(rc.shape)
    rg = oracle.a2c_backward(g, ang, seqs)
    c, rn, an, na2, gi = run_gpu(fm, ang, seqs, g, torch.float64)
    np.testing.assert_array_equal(na, na2)
    np.testing.assert_array_equal(an, ran)
    check(c, gi, rc, rg, na, COORD_TOL_F64, GRAD_TOL_F64)
    assert np.all(c[0] == 0) and np.all(gi[0] == 0)


def test_unknown_letter_and_overflow_reported(fm):
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords import convertStringList
    dev = torch.device("cuda")
    with pytest.raises(RuntimeError):
        fm.getSeqNumAtoms("GAXG")
    seq = convertStringList(["GAXG", "GG"]).to(dev)
    a = torch.zeros(2, 8, 4, device=dev)
    out = torch.full((2, 3 * 8), 7.0, device=dev)
    e = torch.empty(0, dtype=torch.uint8, device=dev)
    fm.Angles2Coords_forward(seq, a, out, e, e)
    assert fm.workspace_status(0) == -5
    assert torch.all(out[0] == 0) and torch.all(out[1] != 7.0)
    # more atoms than slots: clipped and reported
    seq = convertStringList(["WWW"]).to(dev)
    out = torch.zeros(1, 3 * 20, device=dev)
    fm.Angles2Coords_forward(seq, torch.zeros(1, 8, 3, device=dev), out, e, e)
    assert fm.workspace_status(0) == -7
    # angles tensor shorter than the sequence
    seq = convertStringList(["GGGGG"]).to(dev)
    out = torch.zeros(1, 3 * 20, device=dev)
    fm.Angles2Coords_forward(seq, torch.zeros(1, 8, 3, device=dev), out, e, e)
    assert fm.workspace_status(0) == -4
    # the backward from the coordinates rejects the same chains, with zero gradients
    for seqs, L, slots, status in ((["GAXG", "GG"], 4, 8, -5), (["WWW"], 3, 20, -7), (["GGGGG"], 3, 20, -4)):
        seq = convertStringList(seqs).to(dev)
        ga = torch.full((len(seqs), 8, L), float("nan"), device=dev)
        fm.Angles2Coords_backward_coords(torch.ones(len(seqs), 3 * slots, device=dev), ga, seq,
                                         torch.randn(len(seqs), 3 * slots, device=dev))
        assert fm.workspace_status(0) == status
        assert torch.all(ga[0] == 0)
        if len(seqs) > 1:
            assert torch.isfinite(ga[1]).all() and torch.any(ga[1] != 0)


def test_layer_api_and_gradcheck(built):
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords
    layer = Angles2Coords()
    dev = torch.device("cuda")
    seqs = ["ACDEFG", "WYP"]
    x = torch.randn(2, 8, 6, dtype=torch.float64, device=dev, requires_grad=True)
    coords, res, atoms, num = layer(x, seqs)
    assert coords.shape == (2, 3 * int(num.max())) and coords.device == x.device
    assert res.dtype == torch.uint8 and res.shape == (2, int(num.max()), 4)
    assert num.dtype == torch.int32 and num.device.type == "cpu"
    assert [int(v) for v in num] == [oracle.num_atoms(s) for s in seqs]
    assert bytes(atoms[0, 1].cpu().numpy()).rstrip(b"\0") == b"CA"
    assert bytes(res[1, 0].cpu().numpy()).rstrip(b"\0") == b"TRP"

    def f(a):
        return layer(a, seqs)[0]

    assert torch.autograd.gradcheck(f, (x,), eps=1e-6, atol=1e-6, rtol=1e-5)
    with pytest.raises(RuntimeError):
        layer(x.detach().cpu(), seqs)


def test_config4_ragged_fp32_vs_fp64(fm):
    """Training-step workload shapes: 256 chains of U{50..500} random residues;
    the FP32 kernels agree with the FP64 kernels within the stated tolerances."""
    rng = np.random.default_rng(1004)
    B = 256
    lens = rng.integers(50, 501, B)
    L = int(lens.max())
    seqs = ["".join(rng.choice(list(AA), n)) for n in lens]
    ang = rng.uniform(-np.pi, np.pi, (B, 8, L)).astype(np.float32).astype(np.float64)
    c64, _, _, na, _ = run_gpu(fm, ang, seqs, None, torch.float64)
    g = rng.standard_normal(c64.shape).astype(np.float32).astype(np.float64)
    c64, _, _, _, g64 = run_gpu(fm, ang, seqs, g, torch.float64)
    for threads in (0, 4, 8, 128, 512):
        fm.set_options(threads)
        try:
            c32, _, _, _, g32 = run_gpu(fm, ang, seqs, g, torch.float32)
        finally:
            fm.set_options(0)
        check(c32, g32, c64, g64, na, COORD_TOL_F32, GRAD_TOL_F32)
    c32, _, _, _, g32 = run_gpu(fm, ang, seqs, g, torch.float32, from_coords=True)
    check(c32, g32, c64, g64, na, COORD_TOL_F32, GRAD_TOL_F32)


@pytest.mark.parametrize("warps", [4, 8])
def test_four_warp_forward_chunk_edges(fm, warps):
    """Forward with four or eight warps per chain (threads_per_cta = 4 or 8): chains
    ending on and beside the 32-residue chunks and the rounds of 128 and 256
    residues, an empty chain, with names, against the oracle; padding past each
    chain is zero."""
    rng = np.random.default_rng(44)
    lens = [0, 1, 2, 31, 32, 33, 64, 65, 127, 128, 129, 160, 161, 255, 256, 257, 300]
    seqs = ["".join(rng.choice(list(AA), n)) for n in lens]
    L = max(lens)
    ang = rng.uniform(-np.pi, np.pi, (len(seqs), 8, L)).astype(np.float32).astype(np.float64)
    rc, rrn, ran, na = oracle.a2c_forward(ang, seqs)
    fm.set_options(warps)
    try:
        c, rn, an, na2, _ = run_gpu(fm, ang, seqs, None, torch.float32)
    finally:
        fm.set_options(0)
    np.testing.assert_array_equal(na2, na)
    np.testing.assert_array_equal(rn, rrn)
    np.testing.assert_array_equal(an, ran)
    for b, n in enumerate(na):
        assert np.abs(c[b, :3 * n] - rc[b, :3 * n]).max(initial=0.0) <= COORD_TOL_F32
        assert np.all(c[b, 3 * n:] == 0)


def coords_case(seed):
    """Chains ending on and beside the 32-residue chunks and 128-residue rounds of the
    four-warp kernels and the 256-residue tiles of the CTA kernels, one- and
    two-residue chains, an empty one, and one with all 20 residue types."""
    rng = np.random.default_rng(seed)
    lens = [0, 1, 2, 31, 32, 33, 127, 128, 129, 255, 256, 257, 300, 513]
    seqs = ["".join(rng.choice(list(AA), n)) for n in lens] + [AA, "GP" * 10, "W" * 40]
    L = 520
    ang = rng.uniform(-np.pi, np.pi, (len(seqs), 8, L)).astype(np.float32).astype(np.float64)
    ang[:, 2] = rng.normal(np.pi, 0.05, (len(seqs), L)).astype(np.float32)
    rc, rrn, ran, na = oracle.a2c_forward(ang, seqs)
    g = rng.standard_normal(rc.shape).astype(np.float32).astype(np.float64)
    for b, n in enumerate(na):
        g[b, 3 * n:] = 0
    return seqs, ang, rc, na, g


def test_backward_from_coordinates_matches_oracle(fm):
    """The float32 backward from the forward's output coordinates (what the
    float32 layer runs) against the oracle, with NaN in dL/dx past every chain's
    atoms (ignored)."""
    seqs, ang, rc, na, g = coords_case(61)
    rg = oracle.a2c_backward(g, ang, seqs)
    g_nan = g.copy()
    for b, n in enumerate(na):
        g_nan[b, 3 * n:] = np.nan
    c, _, _, _, gi = run_gpu(fm, ang, seqs, g_nan, torch.float32, from_coords=True)
    assert np.isfinite(gi).all()
    check(c, gi, rc, rg, na, COORD_TOL_F32, GRAD_TOL_F32)
    assert np.all(gi[0] == 0.0)


def test_four_warp_kernels_at_batch_size(fm):
    """Below 4 x (number of SMs) chains the automatic choice runs the forward with
    names and the backward from the coordinates with eight warps per chain, from
    there with four: the chains of coords_case, repeated to that batch size, against
    the oracle in every replica (the other tests of this file run the eight-warp
    kernels)."""
    seqs, ang, rc, na, g = coords_case(63)
    rg = oracle.a2c_backward(g, ang, seqs)
    reps = -(-4 * torch.cuda.get_device_properties(0).multi_processor_count // len(seqs))
    c, _, _, na2, gi = run_gpu(fm, np.tile(ang, (reps, 1, 1)), seqs * reps, np.tile(g, (reps, 1)), torch.float32,
                               from_coords=True)
    n = len(seqs)
    for r in range(reps):
        check(c[r * n:(r + 1) * n], gi[r * n:(r + 1) * n], rc, rg, na, COORD_TOL_F32, GRAD_TOL_F32)
    # replicas of a chain see the same kernel path: identical results
    np.testing.assert_array_equal(gi[:n], gi[(reps - 1) * n:])


def test_persistent_kernels_take_several_chains_per_cta(fm):
    """The four- and eight-warp kernels are persistent: a grid of (resident CTAs per
    SM) x (SMs) takes the chains in turn.  With 60 replicas of coords_case (1020
    chains) every kernel's CTAs take more than one chain: the forward with names (four
    warps, at most 6 x SMs CTAs), the reference-signature backward's forward without
    names (eight warps, 3 x SMs) and the backward from the coordinates.  Every
    replica must equal the first bit for bit, and the first the oracle."""
    seqs, ang, rc, na, g = coords_case(67)
    rg = oracle.a2c_backward(g, ang, seqs)
    reps, n = 60, len(seqs)
    assert reps * n > 6 * torch.cuda.get_device_properties(0).multi_processor_count
    for from_coords in (True, False):
        c, rn, an, _, gi = run_gpu(fm, np.tile(ang, (reps, 1, 1)), seqs * reps, np.tile(g, (reps, 1)),
                                   torch.float32, from_coords=from_coords)
        check(c[:n], gi[:n], rc, rg, na, COORD_TOL_F32, GRAD_TOL_F32)
        for r in range(1, reps):
            sl = slice(r * n, (r + 1) * n)
            np.testing.assert_array_equal(c[sl], c[:n])
            np.testing.assert_array_equal(gi[sl], gi[:n])
            np.testing.assert_array_equal(rn[sl], rn[:n])
            np.testing.assert_array_equal(an[sl], an[:n])


def test_backward_from_coordinates_c_abi_and_layer(fm, built):
    """Through the C ABI (status-word workspace only), bit-identical to the
    extension entry; and the float32 autograd layer's gradient (from its saved
    coordinates) against the reference-signature backward selected by
    backward_from_coords = False, which recomputes the same coordinates (identical
    gradient) or, with set_backward_tree(True), rebuilds the tree per joint."""
    import ctypes
    from torchproteinlibrary_gb300 import capi
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords import convertStringList
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords.Angles2Coords import Angles2CoordsFunction
    seqs, ang, rc, na, g = coords_case(62)
    dev = torch.device("cuda")
    c, _, _, _, gi = run_gpu(fm, ang, seqs, g, torch.float32, from_coords=True)
    lib = capi.lib()
    seq = convertStringList(seqs).to(dev)
    B, _, L = ang.shape
    maxA = int(max(na))
    ct = torch.tensor(c, dtype=torch.float32, device=dev)
    gt = torch.tensor(g, dtype=torch.float32, device=dev)
    out = torch.full((B, 8, L), float("nan"), device=dev)
    ws = torch.zeros(64, dtype=torch.uint8, device=dev)
    capi.check(lib.tpl_a2c_backward_coords_f32(out.data_ptr(), gt.data_ptr(), ct.data_ptr(), seq.data_ptr(),
                                               seq.shape[1], ws.data_ptr(), 64, B, L, maxA, capi.stream_ptr()),
               "a2c backward from coordinates")
    torch.cuda.synchronize()
    assert ws[:4].view(torch.int32).item() == 0
    np.testing.assert_array_equal(out.double().cpu().numpy(), gi)
    layer = Angles2Coords()
    grads = {}
    for flag, tree in ((True, False), (False, False), (False, True)):
        Angles2CoordsFunction.backward_from_coords = flag
        fm.set_backward_tree(tree)
        try:
            x = torch.tensor(ang, dtype=torch.float32, device=dev, requires_grad=True)
            coords = layer(x, seqs)[0]
            coords.backward(gt)
            grads[flag, tree] = x.grad.double().cpu().numpy()
        finally:
            Angles2CoordsFunction.backward_from_coords = True
            fm.set_backward_tree(False)
    np.testing.assert_array_equal(grads[True, False], gi)
    np.testing.assert_array_equal(grads[False, False], gi)
    scale = max(1.0, np.abs(grads[False, True]).max())
    assert np.abs(grads[True, False] - grads[False, True]).max() <= GRAD_TOL_F32 * scale


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_cpp_autograd_path_matches_python_function(built, dtype):
    """The Angles2Coords and Coords2RMSD modules run the extensions' C++ autograd
    functions; their outputs and gradients equal those of the Python autograd
    functions (Angles2CoordsFunction, _Coords2RMSDCentering) bit for bit, since both
    call the same entry points."""
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords import Angles2CoordsFunction
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    from torchproteinlibrary_gb300.RMSD.Coords2RMSD.Coords2RMSD import _Coords2RMSDCentering
    rng = np.random.default_rng(12)
    seqs = ["".join(rng.choice(list(AA), n)) for n in (40, 17, 33)]
    dev = torch.device("cuda")
    ang = rng.uniform(-np.pi, np.pi, (3, 8, 40))
    layer = Angles2Coords()
    x1 = torch.tensor(ang, dtype=dtype, device=dev, requires_grad=True)
    c1, r1, a1, n1 = layer(x1, seqs)
    assert "Angles2CoordsAutograd" in c1.grad_fn.name()
    tgt = (c1.detach() + 0.5 * torch.randn_like(c1)).contiguous()
    rmsd1 = Coords2RMSD()(c1, tgt, n1)
    assert "Coords2RMSDAutograd" in rmsd1.grad_fn.name()
    loss1 = rmsd1.sum()
    loss1.backward()
    x2 = torch.tensor(ang, dtype=dtype, device=dev, requires_grad=True)
    seq, num_atoms, _ = layer._prepare(seqs, dev)
    c2, r2, a2, n2 = Angles2CoordsFunction.apply(x2, seq, num_atoms)
    rmsd2, _ = _Coords2RMSDCentering.apply(c2, tgt, n2)
    rmsd2.sum().backward()
    assert torch.equal(c1, c2) and torch.equal(r1, r2) and torch.equal(a1, a2)
    assert torch.equal(loss1.detach(), rmsd2.sum().detach())
    assert torch.equal(x1.grad, x2.grad)


def test_full_size_backbone_geometry(fm):
    """At the 4096-chain x 500-residue scale (random sequences, angles U[-pi, pi)),
    properties that hold whatever the size: every N-CA, CA-C and C-N(next) bond of
    every chain has its template length (1.46, 1.525 and 1.33 A) within 2e-4 A in
    FP32, each residue's N-CA-C angle is the template's, and the rows past each
    chain's atoms are exactly zero.  The FP32 forward against the FP64 form on a
    16-chain slice within the float32 tolerance."""
    from torchproteinlibrary_gb300.FullAtomModel.Angles2Coords import convertStringList
    rng = np.random.default_rng(2024)
    B, L = 4096, 500
    aa = np.array(list(AA))
    seqs = ["".join(rng.choice(aa, L)) for _ in range(B)]
    nat_of = {c: fm.getSeqNumAtoms(c) for c in AA}
    dev = torch.device("cuda")
    ang = torch.tensor(rng.uniform(-np.pi, np.pi, (B, 8, L)), dtype=torch.float32, device=dev)
    seq = convertStringList(seqs).to(dev)
    counts = np.array([[nat_of[c] for c in s] for s in seqs], dtype=np.int64)
    maxA = int(counts.sum(1).max())
    coords = torch.full((B, 3 * maxA), float("nan"), device=dev)
    e = torch.empty(0, dtype=torch.uint8, device=dev)
    fm.Angles2Coords_forward(seq, ang, coords, e, e)
    assert fm.workspace_status(0) == 0
    off = np.concatenate([np.zeros((B, 1), np.int64), np.cumsum(counts, 1)[:, :-1]], 1)
    n_idx = torch.tensor(off, device=dev)
    ca_idx = n_idx + 1
    c_idx = torch.tensor(off + counts - 2, device=dev)
    X = coords.view(B, maxA, 3).double()

    def at(idx):
        return torch.gather(X, 1, idx.unsqueeze(-1).expand(-1, -1, 3))

    N, CA, C = at(n_idx), at(ca_idx), at(c_idx)
    for p, q, d in ((N, CA, 1.46), (CA, C, 1.525), (C[:, :-1], N[:, 1:], 1.33)):
        err = ((p - q).norm(dim=-1) - d).abs().max().item()
        assert err <= 2e-4, (d, err)
    u, v = N - CA, C - CA
    cosang = (u * v).sum(-1) / (u.norm(dim=-1) * v.norm(dim=-1))
    ang_err = (torch.acos(cosang.clamp(-1, 1)) - torch.acos(cosang[0, 0].clamp(-1, 1))).abs().max().item()
    assert ang_err <= 1e-4, ang_err
    tot = counts.sum(1)
    for b in (0, B // 2, B - 1):
        assert torch.all(coords[b, 3 * int(tot[b]):] == 0)
    # a 16-chain slice against the FP64 form
    sl = slice(0, 16)
    c64 = torch.empty(16, 3 * maxA, dtype=torch.float64, device=dev)
    fm.Angles2Coords_forward(seq[sl], ang[sl].double(), c64, e, e)
    d = (coords[sl].double() - c64).view(16, maxA, 3).norm(dim=-1).max().item()
    assert d <= COORD_TOL_F32, d


def test_angles_beyond_the_fast_sincos_range(fm):
    """One in eight of the eight angle rows moved by up to 1e5 turns: those residues take
    sincosf instead of the polynomial sin/cos; the forward and both float32 backwards
    against the oracle on the same float32 angles."""
    seqs, ang, _, _, _ = coords_case(83)
    rng = np.random.default_rng(83)
    pick = rng.random(ang.shape) < 0.125
    ang = np.where(pick, ang + rng.integers(-100000, 100001, ang.shape) * (2 * np.pi), ang)
    ang = ang.astype(np.float32).astype(np.float64)
    assert np.abs(ang).max() > 1e4
    rc, _, _, na = oracle.a2c_forward(ang, seqs)
    g = rng.standard_normal(rc.shape).astype(np.float32).astype(np.float64)
    for b, n in enumerate(na):
        g[b, 3 * n:] = 0
    rg = oracle.a2c_backward(g, ang, seqs)
    for from_coords in (True, False):
        c, _, _, _, gi = run_gpu(fm, ang, seqs, g, torch.float32, from_coords=from_coords)
        check(c, gi, rc, rg, na, COORD_TOL_F32, GRAD_TOL_F32)
