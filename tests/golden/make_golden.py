"""Generate the golden fixtures of tests/golden/ from the reference itself.

* Kinematics and the PDB reader: the reference's own CPU sources, compiled
  unmodified by ``make -C oracle ref REF=<reference checkout>``
  (oracle/_ref/libtplref.so).
* CoordsTransform, Coords2TypedCoords and Coords2RMSD: the reference's own CPU
  interfaces compiled unmodified as a torch extension (oracle/build_ref_ext.py),
  driven through the reference's own Python layers
  (TorchProteinLibrary/FullAtomModel/CoordsTransform/CoordsTransform.py,
  .../Coords2TypedCoords/Coords2TypedCoords.py, .../RMSD/Coords2RMSD/Coords2RMSD.py),
  which are loaded from the checkout with that extension standing in for
  ``_FullAtomModel`` / ``_RMSD``; their backwards run through torch autograd.

Inputs are small and seeded; inputs and outputs are stored as .npz.  The
fixtures pin the oracle (tests/test_oracle_pin.py, tests/test_ref_pins.py) and
the GPU kernels on machines where the reference sources are absent.

    python tests/golden/make_golden.py [--ref /path/to/reference] [--which ...]
"""
import argparse
import importlib.util
import os
import sys
import types

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


def save_case():
    """The reference's PDB writer (cConformation::save): one chain written with mode
    'w', then two more appended with mode 'a' (MODEL / ENDMDL blocks)."""
    rng = np.random.default_rng(20261209)
    seqs = [AA, "GP", "".join(rng.choice(list(AA), 17))]
    path = os.path.join(HERE, "a2c_save_ref.pdb")
    out = {"sequences": np.array(seqs)}
    for i, (seq, mode) in enumerate(zip(seqs, "waa")):
        ang = rng.uniform(-np.pi, np.pi, (8, len(seq)))
        ang[2] = np.pi
        out[f"angles{i}"] = ang
        oracle.a2c_save_ref(seq, ang, path, mode)
    return out


# ----------------------------------------------- CoordsTransform, typed, RMSD
def _reference_layers(ref_dir: str):
    """The reference's Python layer modules, loaded from the checkout, with the
    oracle's build of the reference's CPU interfaces as their extensions."""
    from oracle import build_ref_ext

    ext = build_ref_ext.build(ref_dir)
    sys.modules["_FullAtomModel"] = ext
    sys.modules["_RMSD"] = ext

    def load(name, rel):
        spec = importlib.util.spec_from_file_location(name, os.path.join(ref_dir, rel))
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
        return mod

    # the package __init__ files import Biopython-dependent modules: register bare packages
    for pkg in ["TorchProteinLibrary", "TorchProteinLibrary.FullAtomModel", "TorchProteinLibrary.RMSD"]:
        sys.modules.setdefault(pkg, types.ModuleType(pkg))
    ct = load("TorchProteinLibrary.FullAtomModel.CoordsTransform",
              "TorchProteinLibrary/FullAtomModel/CoordsTransform/CoordsTransform.py")
    tc = load("TorchProteinLibrary.FullAtomModel.Coords2TypedCoords",
              "TorchProteinLibrary/FullAtomModel/Coords2TypedCoords/Coords2TypedCoords.py")
    rm = load("TorchProteinLibrary.RMSD.Coords2RMSD", "TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py")
    return ext, ct, tc, rm


def transform_case(ext, ct):
    """CoordsTranslate / CoordsRotate / Coords2Center forward and backward through the
    reference layers, getBBox and getRotation, in float64 and float32."""
    import torch
    rng = np.random.default_rng(20261206)
    out = {}
    B, S = 6, 40
    na = np.array([40, 17, 1, 33, 2, 40], dtype=np.int32)
    u = rng.uniform(0, 1, (B, 3))
    out["u"] = u
    out["rotation"] = ct.getRotation(torch.tensor(u)).numpy()
    for tag, dt in (("f64", torch.float64), ("f32", torch.float32)):
        x = rng.normal(0, 10, (B, 3 * S))
        T = rng.normal(0, 5, (B, 3))
        g = rng.standard_normal((B, 3 * S))
        gc = rng.standard_normal((B, 3))
        num = torch.tensor(na)
        xt = torch.tensor(x, dtype=dt, requires_grad=True)
        Tt = torch.tensor(T, dtype=dt)
        Rt = torch.tensor(out["rotation"], dtype=dt)
        y = ct.CoordsTranslate()(xt, Tt, num)
        y.backward(torch.tensor(g, dtype=dt))
        out[f"{tag}_translate"], out[f"{tag}_translate_grad"] = y.detach().numpy(), xt.grad.numpy().copy()
        xt.grad = None
        y = ct.CoordsRotate()(xt, Rt, num)
        y.backward(torch.tensor(g, dtype=dt))
        out[f"{tag}_rotate"], out[f"{tag}_rotate_grad"] = y.detach().numpy(), xt.grad.numpy().copy()
        xt.grad = None
        c = ct.Coords2Center()(xt, num)
        c.backward(torch.tensor(gc, dtype=dt))
        out[f"{tag}_center"], out[f"{tag}_center_grad"] = c.detach().numpy(), xt.grad.numpy().copy()
        lo, hi = ct.getBBox(xt.detach(), num)
        out[f"{tag}_bbox_lo"], out[f"{tag}_bbox_hi"] = lo.numpy(), hi.numpy()
        out[f"{tag}_x"], out[f"{tag}_T"] = xt.detach().numpy(), Tt.numpy()
        out[f"{tag}_grad_out"] = torch.tensor(g, dtype=dt).numpy()
        out[f"{tag}_grad_center"] = torch.tensor(gc, dtype=dt).numpy()
    out["num_atoms"] = na
    return out


def typed_case(tc):
    """Coords2TypedCoords forward and backward through the reference layer on the
    names and coordinates the reference's Angles2Coords produces."""
    import torch
    rng = np.random.default_rng(20261207)
    seqs = [AA, "G", "GP", "".join(rng.choice(list(AA), 25)), "".join(rng.choice(list(AA), 40)), "WYFHR"]
    L = 40
    ang = rng.uniform(-np.pi, np.pi, (len(seqs), 8, L))
    coords, rn, an, na = oracle.a2c_forward(ang, seqs, impl="ref")
    xt = torch.tensor(coords, requires_grad=True)
    typed, counts, offsets = tc.Coords2TypedCoords()(xt, torch.tensor(rn), torch.tensor(an), torch.tensor(na))
    g = rng.standard_normal(tuple(typed.shape))
    typed.backward(torch.tensor(g))
    return dict(sequences=np.array(seqs), coords=coords, res_names=rn, atom_names=an, num_atoms=na,
                typed=typed.detach().numpy(), num_atoms_of_type=counts.numpy(), offsets=offsets.numpy(),
                grad_typed=g, grad_coords=xt.grad.numpy())


def rmsd_case(rm):
    """Coords2RMSD forward (with its centring) and backward through the reference
    layer: random pairs, rigidly moved noisy copies, ragged atom counts."""
    import torch
    rng = np.random.default_rng(20261208)
    B, S = 6, 30
    na = np.array([30, 12, 30, 5, 21, 3], dtype=np.int32)
    src = rng.normal(0, 8, (B, 3 * S))
    dst = rng.normal(0, 8, (B, 3 * S))
    for b in (2, 3):  # a rotated, translated and slightly perturbed copy
        q = rng.standard_normal(4)
        q /= np.linalg.norm(q)
        a, bq, c, d = q
        R = np.array([[a * a + bq * bq - c * c - d * d, 2 * (bq * c - a * d), 2 * (bq * d + a * c)],
                      [2 * (bq * c + a * d), a * a - bq * bq + c * c - d * d, 2 * (c * d - a * bq)],
                      [2 * (bq * d - a * c), 2 * (c * d + a * bq), a * a - bq * bq - c * c + d * d]])
        pts = src[b].reshape(S, 3) @ R.T + rng.normal(0, 3, 3) + rng.normal(0, 0.1, (S, 3))
        dst[b] = pts.reshape(-1)
    for b, n in enumerate(na):
        src[b, 3 * n:] = 0.0
        dst[b, 3 * n:] = 0.0
    g = rng.uniform(0.5, 2.0, B)
    x = torch.tensor(src, requires_grad=True)
    layer = rm.Coords2RMSD()
    r = layer(x, torch.tensor(dst), torch.tensor(na))
    r.backward(torch.tensor(g))
    return dict(src=src, dst=dst, num_atoms=na, rmsd=r.detach().numpy(), ut=layer.UT.detach().numpy(),
                grad_rmsd=g, grad_src=x.grad.numpy())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=oracle.reference_dir())
    ap.add_argument("--which", default="all",
                    choices=["all", "a2b", "a2c", "pdb", "save", "transform", "typed", "rmsd"])
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(args.ref):
        sys.exit("no reference checkout (set TPL_REFERENCE_DIR or pass --ref); fixtures not regenerated")
    oracle.build(args.ref)
    if not oracle.ref_available():
        sys.exit("reference sources could not be built; fixtures not regenerated")
    if args.which in ("all", "transform", "typed", "rmsd"):
        ext, ct, tc, rm = _reference_layers(args.ref)
        if args.which in ("all", "transform"):
            np.savez_compressed(os.path.join(HERE, "transform_ref.npz"), **transform_case(ext, ct))
        if args.which in ("all", "typed"):
            np.savez_compressed(os.path.join(HERE, "typed_ref.npz"), **typed_case(tc))
        if args.which in ("all", "rmsd"):
            np.savez_compressed(os.path.join(HERE, "rmsd_ref.npz"), **rmsd_case(rm))
    if args.which in ("all", "a2b"):
        np.savez_compressed(os.path.join(HERE, "a2b_ref.npz"), **a2b_case())
    if args.which in ("all", "a2c"):
        np.savez_compressed(os.path.join(HERE, "a2c_ref.npz"), **a2c_case())
    if args.which in ("all", "pdb"):
        np.savez_compressed(os.path.join(HERE, "pdb_ref.npz"), **pdb_case())
    if args.which in ("all", "save"):
        np.savez_compressed(os.path.join(HERE, "a2c_save_ref.npz"), **save_case())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
