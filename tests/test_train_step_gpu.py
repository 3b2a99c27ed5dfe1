"""The training step: Angles2Coords -> Coords2RMSD (mean over chains) -> backward.

The gradient dL/dangles of the whole step is compared with the oracle: the
reference's a2c CPU backward (restated in oracle/tpl_oracle.c) fed with the
upstream dL/dx of the oracle's Kabsch/quaternion RMSD (oracle.rmsd), as the
training-step workload prescribes while the reference's own _RMSD does not build.
Tolerances: FP64 1e-8 x max|grad|; FP32 1e-4 x max|grad| (the workload's bound for
gradients), on a small batch and on the training-step workload's full shape
(256 chains of U{50..500} residues).
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

AA = "ACDEFGHIKLMNPQRSTVWY"


def case(lengths, seed):
    rng = np.random.default_rng(seed)
    seqs = ["".join(rng.choice(list(AA), n)) for n in lengths]
    L = max(lengths)
    ang = rng.uniform(-np.pi, np.pi, (len(lengths), 8, L))
    ang[:, 2] = np.pi
    for b, n in enumerate(lengths):
        ang[b, :, n:] = 0.0
    target_ang = ang + rng.normal(0.0, 0.3, ang.shape)
    return seqs, ang, target_ang


def oracle_step(seqs, ang, target_ang):
    tgt, _, _, na = oracle.a2c_forward(target_ang, seqs)
    x, _, _, _ = oracle.a2c_forward(ang, seqs)
    r, _, g = oracle.rmsd(x, tgt, na)
    B = len(seqs)
    return r.mean(), oracle.a2c_backward(g / B, ang, seqs), tgt


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-8), (torch.float32, 1e-4)])
def test_training_step_gradient_matches_oracle(built, dtype, tol):
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    lengths = [23, 41, 8, 57, 30]
    seqs, ang, target_ang = case(lengths, 4)
    loss_o, grad_o, tgt = oracle_step(seqs, ang, target_ang)
    dev = torch.device("cuda")
    a2c, rmsd = Angles2Coords(), Coords2RMSD()
    x = torch.tensor(ang, dtype=dtype, device=dev, requires_grad=True)
    coords, _, _, num_atoms = a2c(x, seqs)
    target = torch.tensor(tgt, dtype=dtype, device=dev)
    loss = rmsd(coords, target, num_atoms.to(dev)).mean()
    loss.backward()
    assert abs(loss.item() - loss_o) <= tol * max(1.0, abs(loss_o))
    g = x.grad.double().cpu().numpy()
    scale = np.abs(grad_o).max()
    assert np.abs(g - grad_o).max() <= tol * scale, np.abs(g - grad_o).max() / scale


def oracle_step_threaded(seqs, ang, target_ang):
    """oracle_step, one chain per host thread (the oracle's C calls release the GIL)."""
    B = len(seqs)

    def one(b):
        sl = slice(b, b + 1)
        tgt, _, _, na = oracle.a2c_forward(target_ang[sl], seqs[sl])
        x, _, _, _ = oracle.a2c_forward(ang[sl], seqs[sl])
        r, _, g = oracle.rmsd(x, tgt, na)
        return r[0], oracle.a2c_backward(g / B, ang[sl], seqs[sl])[0], tgt[0]

    with ThreadPoolExecutor() as ex:
        rows = list(ex.map(one, range(B)))
    width = max(len(t) for _, _, t in rows)
    tgt = np.zeros((B, width))
    for b, (_, _, t) in enumerate(rows):
        tgt[b, :len(t)] = t
    return float(np.mean([r for r, _, _ in rows])), np.stack([g for _, g, _ in rows]), tgt


def test_training_step_full_shape_fp32_matches_oracle(built):
    """The training-step workload at its full shape: 256 chains, lengths U{50..500},
    random sequences over the 20 amino acids, target = Angles2Coords(angles + N(0, 0.3)).
    The FP32 batched step's dL/dangles lies within 1e-4 of the largest gradient entry
    of the FP64 oracle, and its loss within 1e-4 relative."""
    from torchproteinlibrary_gb300.FullAtomModel import Angles2Coords
    from torchproteinlibrary_gb300.RMSD import Coords2RMSD
    rng = np.random.default_rng(1004)
    lengths = list(rng.integers(50, 501, 256))
    seqs, ang, target_ang = case(lengths, 1004)
    loss_o, grad_o, tgt = oracle_step_threaded(seqs, ang, target_ang)
    dev = torch.device("cuda")
    a2c, rmsd = Angles2Coords(), Coords2RMSD()
    x = torch.tensor(ang, dtype=torch.float32, device=dev, requires_grad=True)
    coords, _, _, num_atoms = a2c(x, seqs)
    assert coords.shape[1] == tgt.shape[1]
    target = torch.tensor(tgt, dtype=torch.float32, device=dev)
    loss = rmsd(coords, target, num_atoms).mean()
    loss.backward()
    assert abs(loss.item() - loss_o) <= 1e-4 * abs(loss_o)
    g = x.grad.double().cpu().numpy()
    scale = np.abs(grad_o).max()
    assert np.abs(g - grad_o).max() <= 1e-4 * scale, np.abs(g - grad_o).max() / scale
