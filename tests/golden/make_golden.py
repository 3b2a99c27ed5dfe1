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


def pdb_sample() -> str:
    """A synthetic PDB text (not taken from any database): the reference's full-atom
    geometry for a short chain in the writePDB record format, plus records the reader
    must skip or normalise: HETATM, hydrogens, header/TER/END lines, a second chain,
    negative residue numbers, an insertion code, left-justified atom names."""
    rng = np.random.default_rng(20261205)
    seq = "MKWVDESHG"
    ang = rng.uniform(-np.pi, np.pi, (1, 8, len(seq)))
    ang[:, 2] = np.pi
    coords, rn, an, na = oracle.a2c_forward(ang, [seq], impl="ref")
    lines = ["HEADER    SYNTHETIC TEST STRUCTURE", "REMARK   1 generated by tests/golden/make_golden.py", "MODEL 0"]
    name = lambda a: bytes(a).split(b"\0", 1)[0].decode()
    for j in range(int(na[0])):
        res_num = j // 4 - 2  # runs through negative residue numbers
        x, y, z = coords[0, 3 * j:3 * j + 3] * 7.3
        lines.append("ATOM  %5d  %-3s %3s %c%4d    %8.3f%8.3f%8.3f  1.00  0.00" % (
            j + 1, name(an[0, j]), name(rn[0, j]), "A", res_num, x, y, z))
        if j % 5 == 0:
            lines.append("ATOM  %5d  H   %3s %c%4d    %8.3f%8.3f%8.3f" % (j + 1, name(rn[0, j]), "A", res_num, x, y, z))
    lines.append("TER")
    lines.append("ATOM    900 N    GLY B 101A     -1.250 -22.100  33.333  1.00 10.00           N")
    lines.append("ATOM    901 CA   GLY B 101A     -0.500 -21.000  34.000  1.00 10.00           C")
    lines.append("ATOM    902 SG   CYS B 102      10.125   0.001 -99.999  1.00 10.00           S")
    lines.append("HETATM  903  O   HOH B 201       1.000   2.000   3.000  1.00 20.00           O")
    lines.append("ATOM    904 HG1  THR B 103       1.000   2.000   3.000  1.00 20.00           H")
    lines.append("ENDMDL")
    lines.append("END")
    return "\n".join(lines) + "\n"


def pdb_case():
    path = os.path.join(HERE, "sample.pdb")
    with open(path, "w") as f:
        f.write(pdb_sample())
    coords, chains, res, atoms, nums = oracle.pdb_read(path, impl="ref")
    return dict(coords=coords, chain_names=np.array(chains), res_names=np.array(res), atom_names=np.array(atoms),
                res_nums=nums)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--which", default="all", choices=["all", "a2b", "a2c", "pdb"])
    args = ap.parse_args()
    oracle.build(args.ref)
    if not oracle.ref_available():
        sys.exit("reference sources could not be built; fixtures not regenerated")
    if args.which in ("all", "a2b"):
        np.savez_compressed(os.path.join(HERE, "a2b_ref.npz"), **a2b_case())
    if args.which in ("all", "a2c"):
        np.savez_compressed(os.path.join(HERE, "a2c_ref.npz"), **a2c_case())
    if args.which in ("all", "pdb"):
        np.savez_compressed(os.path.join(HERE, "pdb_ref.npz"), **pdb_case())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
