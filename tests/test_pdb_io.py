"""PDB reading and writing (host code, no GPU).

The native reader (libtpl_gb300's tpl_pdb_read_batch behind
FullAtomModel.PDB2Coords.PDB2CoordsUnordered) is compared bit-exactly with the
reference's own cPDBLoader: through the committed fixture tests/golden/pdb_ref.npz
(generated from tests/golden/sample.pdb by tests/golden/make_golden.py) and, where
the reference sources are present, live.  writePDB -> read round trips keep
coordinates to the format's 1e-3 A and names exactly."""
import os

import numpy as np
import pytest
import torch

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
SAMPLE = os.path.join(HERE, "golden", "sample.pdb")


@pytest.fixture(scope="module")
def pdb(built):
    from torchproteinlibrary_gb300.FullAtomModel import PDB2Coords
    return PDB2Coords


def names(t, n):
    return [bytes(t[j].numpy()).split(b"\0", 1)[0].decode() for j in range(n)]


def test_reader_matches_reference_fixture(pdb):
    ref = np.load(os.path.join(HERE, "golden", "pdb_ref.npz"))
    coords, chains, res, nums, atoms, n = pdb.PDB2CoordsUnordered()([SAMPLE])
    n = int(n[0])
    assert n == len(ref["coords"]) == 78
    assert coords.dtype == torch.float64 and coords.shape == (1, 3 * n)
    assert np.array_equal(coords[0].numpy().reshape(n, 3), ref["coords"])
    assert names(chains[0], n) == list(ref["chain_names"])
    assert names(res[0], n) == list(ref["res_names"])
    assert names(atoms[0], n) == list(ref["atom_names"])
    assert np.array_equal(nums[0].numpy(), ref["res_nums"])


def test_port_matches_fixture_and_live_reference():
    ref = np.load(os.path.join(HERE, "golden", "pdb_ref.npz"))
    c, ch, rn, an, nums = oracle.pdb_read(SAMPLE)
    assert np.array_equal(c, ref["coords"]) and an == list(ref["atom_names"]) and np.array_equal(nums, ref["res_nums"])
    if oracle.ref_available():
        c2, ch2, rn2, an2, nums2 = oracle.pdb_read(SAMPLE, impl="ref")
        assert np.array_equal(c2, ref["coords"]) and rn2 == list(ref["res_names"]) and ch2 == list(ref["chain_names"])


def test_write_read_round_trip_and_sequence(pdb, oracle_lib, tmp_path):
    seqs = ["ACDEFGHIKLMNPQRSTVWY", "GPW"]
    rng = np.random.default_rng(8)
    ang = rng.uniform(-np.pi, np.pi, (2, 8, 20))
    x, rn, an, na = oracle.a2c_forward(ang, seqs)
    # residue numbers from the atom layout: a new residue starts at every N
    resnums = np.zeros((2, x.shape[1] // 3), dtype=np.int32)
    for b in range(2):
        r = 0
        for j in range(na[b]):
            if bytes(an[b, j]).split(b"\0")[0] == b"N" and j > 0:
                r += 1
            resnums[b, j] = r + 1
    chains = np.zeros_like(rn)
    files = []
    for b in range(2):
        f = str(tmp_path / f"chain{b}.pdb")
        pdb.writePDB(f, torch.tensor(x[b:b + 1]), torch.tensor(chains[b:b + 1]), torch.tensor(rn[b:b + 1]),
                     torch.tensor(resnums[b:b + 1]), torch.tensor(an[b:b + 1]), torch.tensor(na[b:b + 1]))
        files.append(f)
    coords, ch, res, nums, atoms, n = pdb.PDB2CoordsUnordered()(files)
    for b in range(2):
        m = int(na[b])
        assert int(n[b]) == m
        assert np.abs(coords[b, :3 * m].numpy() - x[b, :3 * m]).max() <= 5.1e-4
        assert names(atoms[b], m) == names(torch.tensor(an[b]), m)
        assert names(ch[b], m) == ["A"] * m
        assert np.array_equal(nums[b, :m].numpy(), resnums[b, :m])
    assert pdb.pdb2sequence(files) == seqs


def test_missing_file_raises(pdb, tmp_path):
    with pytest.raises(RuntimeError):
        pdb.PDB2CoordsUnordered()([str(tmp_path / "absent.pdb")])


@pytest.mark.gpu
def test_angles2coords_save_matches_reference_writer(built, tmp_path):
    """Angles2Coords_save (GPU forward, then ATOM records) writes the same bytes as
    the reference's cConformation::save (cConformation.cpp:228-262), whose output for
    these inputs is tests/golden/a2c_save_ref.pdb: one chain with mode 'w', then two
    appended as MODEL blocks with mode 'a'."""
    from torchproteinlibrary_gb300 import load_extension
    ext = load_extension("_FullAtomModel")
    d = np.load(os.path.join(HERE, "golden", "a2c_save_ref.npz"))
    out = str(tmp_path / "saved.pdb")
    for i, (seq, mode) in enumerate(zip(d["sequences"], "waa")):
        ext.Angles2Coords_save(str(seq), torch.tensor(d[f"angles{i}"], device="cuda"), out, mode)
    with open(out, "rb") as f, open(os.path.join(HERE, "golden", "a2c_save_ref.pdb"), "rb") as g:
        assert f.read() == g.read()
