"""Atom typing of the oracle (restatement of ProtUtil::get11AtomType) covers every
atom that Angles2Coords names for the 20 residues, and the type groups match the
reference's comments (N amide = 1, CA sp3 = 10, ...).  CPU only."""
import numpy as np

import oracle

AA = "ACDEFGHIKLMNPQRSTVWY"


def test_every_angles2coords_atom_has_a_type(oracle_lib):
    ang = np.zeros((1, 8, len(AA)))
    _, rn, an, na = oracle.a2c_forward(ang, [AA])
    types = [oracle.atom_type_11(oracle._name(rn[0, j]), oracle._name(an[0, j])) for j in range(na[0])]
    assert min(types) >= 0
    counts = np.bincount(types, minlength=11)
    assert counts.sum() == na[0]
    # backbone: one N, CA, C, O per residue
    assert counts[1] >= len(AA) and counts[8] >= len(AA) and counts[5] >= len(AA) and counts[10] >= len(AA)


def test_type_table_spot_checks():
    t = oracle.atom_type_11
    assert (t("GLY", "N"), t("GLY", "CA"), t("GLY", "C"), t("GLY", "O")) == (1, 10, 8, 5)
    assert (t("CYS", "SG"), t("LYS", "NZ"), t("TYR", "OH"), t("GLU", "OE2"), t("TRP", "CZ3")) == (0, 4, 6, 7, 9)
    assert t("ALA", " CB ") == 10 and t("ALA", "XX") == -1 and t("XYZ", "CB") == -1


def test_typed_regrouping_is_stable_and_invertible(oracle_lib):
    rng = np.random.default_rng(2)
    seqs = ["".join(rng.choice(list(AA), n)) for n in (7, 19, 3)]
    L = max(map(len, seqs))
    x, rn, an, na = oracle.a2c_forward(rng.uniform(-np.pi, np.pi, (3, 8, L)), seqs)
    typed, counts, offsets, index = oracle.typed_coords(x, rn, an, na)
    for b in range(3):
        assert counts[b].sum() == na[b]
        assert sorted(index[b, :na[b]]) == list(range(na[b]))
        for k in range(11):
            sl = index[b, offsets[b, k]:offsets[b, k] + counts[b, k]]
            assert list(sl) == sorted(sl)  # stable within a type
    back = oracle.typed_coords_backward(typed, counts, index, x.shape[1] // 3)
    assert np.array_equal(back, x)
