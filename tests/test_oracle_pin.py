"""Pin the oracle (oracle/tpl_oracle.c) to the reference.

* Against the golden fixtures of tests/golden/, produced by the reference's own
  CPU kinematics (tests/golden/make_golden.py).
* Against the reference compiled from its sources (oracle/_ref), when present.
* Against central finite differences (h = 1e-6).
"""
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
AA = "ACDEFGHIKLMNPQRSTVWY"


def omega_last_mask(lengths, L):
    """False at omega[len-1]: the reference reads one matrix past the chain there
    (Layers/ReducedModel/cBackboneProteinCPUKernels.cpp:83); the oracle returns 0."""
    m = np.ones((len(lengths), 3, L), bool)
    for b, n in enumerate(lengths):
        if n > 0:
            m[b, 2, n - 1] = False
    return m


def test_a2b_golden(oracle_lib):
    d = np.load(os.path.join(GOLD, "a2b_ref.npz"))
    coords, A = oracle.a2b_forward(d["angles"], d["lengths"])
    np.testing.assert_array_equal(coords, d["coords"])  # same FP64 operation order: bit-exact
    grad = oracle.a2b_backward(d["grad_coords"], d["angles"], d["lengths"], A)
    m = omega_last_mask(d["lengths"], d["angles"].shape[2])
    np.testing.assert_allclose(grad[m], d["grad_angles"][m], rtol=0, atol=1e-12)
    # the masked entries are exactly zero in the oracle
    assert np.all(grad[~m] == 0.0)


def test_a2c_golden(oracle_lib):
    d = np.load(os.path.join(GOLD, "a2c_ref.npz"))
    seqs = [str(s) for s in d["sequences"]]
    coords, rn, an, na = oracle.a2c_forward(d["angles"], seqs)
    np.testing.assert_array_equal(na, d["num_atoms"])
    np.testing.assert_array_equal(rn, d["res_names"])
    np.testing.assert_array_equal(an, d["atom_names"])
    np.testing.assert_allclose(coords, d["coords"], rtol=0, atol=1e-12)
    grad = oracle.a2c_backward(d["grad_coords"], d["angles"], seqs)
    scale = np.abs(d["grad_angles"]).max()
    np.testing.assert_allclose(grad, d["grad_angles"], rtol=0, atol=1e-12 * scale)


def test_atom_counts():
    # Math/nUtil.cpp:192-517 (no OXT)
    counts = dict(G=4, A=5, S=6, C=6, V=7, I=8, L=8, T=7, R=11, K=9, D=8, N=8, E=9, Q=9, M=8, H=10, P=7, F=11, Y=12,
                  W=14)
    for k, v in counts.items():
        assert oracle.num_atoms(k) == v
    assert oracle.num_atoms(AA) == sum(counts.values())
    with pytest.raises(ValueError):
        oracle.num_atoms("ACDX")


@pytest.mark.skipif(not oracle.ref_available() and oracle.reference_dir() is None,
                    reason="reference sources not present")
def test_port_matches_reference_build(oracle_lib):
    if not oracle.ref_available():
        pytest.skip("reference build unavailable")
    rng = np.random.default_rng(7)
    B, L = 6, 50
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    lengths = rng.integers(0, L + 1, B).astype(np.int32)
    lengths[0] = L
    c1, A1 = oracle.a2b_forward(ang, lengths)
    c2, A2 = oracle.a2b_forward(ang, lengths, impl="ref")
    np.testing.assert_array_equal(c1, c2)
    g = rng.standard_normal((B, 9 * L))
    m = omega_last_mask(lengths, L)
    np.testing.assert_allclose(oracle.a2b_backward(g, ang, lengths, A1)[m],
                               oracle.a2b_backward(g, ang, lengths, A2, impl="ref")[m], atol=1e-12, rtol=0)
    seqs = ["".join(rng.choice(list(AA), rng.integers(1, 40))) for _ in range(5)]
    a8 = rng.uniform(-np.pi, np.pi, (5, 8, 40))
    x1, rn1, an1, na = oracle.a2c_forward(a8, seqs)
    x2, rn2, an2, _ = oracle.a2c_forward(a8, seqs, impl="ref")
    np.testing.assert_allclose(x1, x2, atol=1e-12, rtol=0)
    assert (rn1 == rn2).all() and (an1 == an2).all()
    gc = rng.standard_normal(x1.shape)
    G1 = oracle.a2c_backward(gc, a8, seqs)
    G2 = oracle.a2c_backward(gc, a8, seqs, impl="ref")
    np.testing.assert_allclose(G1, G2, atol=1e-11 * np.abs(G2).max(), rtol=0)


def test_a2b_central_differences(oracle_lib):
    rng = np.random.default_rng(11)
    B, L = 3, 20
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    lengths = np.array([20, 13, 7], np.int32)
    g = rng.standard_normal((B, 9 * L))
    _, A = oracle.a2b_forward(ang, lengths)
    grad = oracle.a2b_backward(g, ang, lengths, A)
    h = 1e-6
    for _ in range(16):
        b, k, j = rng.integers(B), rng.integers(3), rng.integers(L)
        a = ang.copy(); a[b, k, j] += h
        cp, _ = oracle.a2b_forward(a, lengths)
        a[b, k, j] -= 2 * h
        cm, _ = oracle.a2b_forward(a, lengths)
        fd = (cp - cm)[b] @ g[b] / (2 * h)
        assert abs(fd - grad[b, k, j]) <= 1e-6 * max(1.0, abs(fd))


def test_a2c_central_differences(oracle_lib):
    # the finite-difference check of the 64-chain x 150-residue full-atom case, scaled down:
    # 16 random entries per chain, h = 1e-6
    rng = np.random.default_rng(12)
    seqs = [AA, "".join(rng.choice(list(AA), 25))]
    L = 25 if len(AA) < 25 else len(AA)
    ang = rng.uniform(-np.pi, np.pi, (2, 8, L))
    ang[:, 2] = np.pi
    x, _, _, na = oracle.a2c_forward(ang, seqs)
    g = rng.standard_normal(x.shape)
    grad = oracle.a2c_backward(g, ang, seqs)
    h = 1e-6
    for b in range(2):
        for _ in range(16):
            k, j = rng.integers(8), rng.integers(len(seqs[b]))
            a = ang.copy(); a[b, k, j] += h
            xp, _, _, _ = oracle.a2c_forward(a, seqs)
            a[b, k, j] -= 2 * h
            xm, _, _, _ = oracle.a2c_forward(a, seqs)
            fd = (xp - xm)[b] @ g[b] / (2 * h)
            assert abs(fd - grad[b, k, j]) <= 1e-6 * max(1.0, abs(fd)), (b, k, j, fd, grad[b, k, j])


def test_a2c_gradient_slots(oracle_lib):
    """Angles without a joint get exactly 0 (cConformation.cpp:206-211 assigns only
    joints with a gradient slot): unused chi, Ala/Gly/Pro chi, omega of the last residue."""
    seqs = ["GAPSR"]
    ang = np.random.default_rng(3).uniform(-np.pi, np.pi, (1, 8, 5))
    x, _, _, _ = oracle.a2c_forward(ang, seqs)
    g = np.ones_like(x)
    grad = oracle.a2c_backward(g, ang, seqs)[0]
    assert np.all(grad[3:, 0] == 0) and np.all(grad[3:, 1] == 0) and np.all(grad[3:, 2] == 0)  # G, A, P
    assert grad[3, 3] != 0 and np.all(grad[4:, 3] == 0)  # S: chi1 only
    assert np.all(grad[3:, 4] != 0)  # R: chi1..chi5
    assert grad[2, 4] == 0  # omega of the last residue
