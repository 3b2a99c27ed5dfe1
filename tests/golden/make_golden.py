"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own CPU kinematics, compiled unmodified from its sources
by ``make -C oracle ref REF=<reference checkout>`` (oracle/_ref/libtplref.so),
on small seeded inputs and stores inputs and outputs as .npz.  The fixtures pin
the oracle (tests/test_oracle_pin.py) on machines where the reference sources
are absent.

    python tests/golden/make_golden.py [--ref /path/to/reference]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

AA = "ACDEFGHIKLMNPQRSTVWY"


def a2b_case():
    rng = np.random.default_rng(20261203)
    B, L = 5, 24
    lengths = np.array([24, 17, 1, 0, 9], dtype=np.int32)
    ang = rng.uniform(-np.pi, np.pi, (B, 3, L))
    ang[:2, 2] = np.pi
    ang[2:, 2] = rng.normal(np.pi, 0.05, (B - 2, L))
    g = rng.standard_normal((B, 9 * L))
    coords, A = oracle.a2b_forward(ang, lengths, impl="ref")
    grad = oracle.a2b_backward(g, ang, lengths, A, impl="ref")
    return dict(angles=ang, lengths=lengths, grad_coords=g, coords=coords, grad_angles=grad)


def a2c_case():
    rng = np.random.default_rng(20261204)
    seqs = [AA, "G", "GP", "".join(rng.choice(list(AA), 12)), "".join(rng.choice(list(AA), 30))]
    L = 30
    ang = rng.uniform(-np.pi, np.pi, (len(seqs), 8, L))
    ang[:, 2] = np.pi
    # the reference's own backward test setup for the all-residue chain
    # (UnitTests/FullAtomModel/Angles2Coords/test.py:107-111)
    ang[0, 0], ang[0, 1], ang[0, 2], ang[0, 3:] = -1.047, -0.698, np.pi, 110.4 * np.pi / 180.0
    coords, rn, an, na = oracle.a2c_forward(ang, seqs, impl="ref")
    g = rng.standard_normal(coords.shape)
    for b, n in enumerate(na):
        g[b, 3 * n:] = 0.0
    grad = oracle.a2c_backward(g, ang, seqs, impl="ref")
    return dict(angles=ang, sequences=np.array(seqs), coords=coords, res_names=rn, atom_names=an, num_atoms=na,
                grad_coords=g, grad_angles=grad)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    oracle.build(args.ref)
    if not oracle.ref_available():
        sys.exit("reference sources could not be built; fixtures not regenerated")
    np.savez_compressed(os.path.join(HERE, "a2b_ref.npz"), **a2b_case())
    np.savez_compressed(os.path.join(HERE, "a2c_ref.npz"), **a2c_case())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
