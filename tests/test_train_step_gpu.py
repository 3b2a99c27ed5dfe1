"""The training step: Angles2Coords -> Coords2RMSD (mean over chains) -> backward.

The gradient dL/dangles of the whole step is compared with the oracle: the
reference's a2c CPU backward (restated in oracle/tpl_oracle.c) fed with the
upstream dL/dx of the oracle's Kabsch/quaternion RMSD (oracle.rmsd), as the
training-step workload prescribes while the reference's own _RMSD does not build.
Tolerances: FP64 1e-8 x max|grad|; FP32 2e-3 x max|grad| (two FP32 layers in a row).
"""
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


@pytest.mark.parametrize("dtype,tol", [(torch.float64, 1e-8), (torch.float32, 2e-3)])
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
