"""PDB reading and writing: the on-disk format either side of the path.

Mirrors TorchProteinLibrary/FullAtomModel/PDB2Coords/PDB2Coords.py:
  * ``PDB2CoordsUnordered()(filenames) -> (coords f64 [B, 3N], chain_names u8 [B, N, 4],
    res_names u8 [B, N, 4], res_nums int32 [B, N], atom_names u8 [B, N, 4],
    num_atoms int32 [B])``, CPU tensors, atoms in file order, parsed by the native
    reader of libtpl_gb300 (heavy-atom ATOM records, host threads over the files);
  * ``writePDB(filename, coords, chainnames, resnames, resnums, atomnames, num_atoms,
    bfactors=None, add_model=True, rewrite=True)``, the same record format;
  * ``convertStringList``, ``string2tensor``, ``tensor2string``.

Differences from the reference: ``pdb2sequence`` / ``get_sequence`` read the residue
names with the native reader instead of Biopython (absent here): one letter per
(chain, residue number) in file order, standard amino acids and MSE; anything else
raises, as Biopython's three_to_one does.  ``PDB2CoordsOrdered`` exists by name only
and raises when called: its C++ body is commented out in the reference
(Layers/FullAtomModel/PDB2Coords/pdb2coords_interface.cpp:7, not bound in
Layers/FullAtomModel/main.cpp) and its Python wrapper reads an attribute it never
sets, so it has no behaviour to reproduce.
"""
import os

import numpy as np
import torch

from ... import load_extension

_FullAtomModel = load_extension("_FullAtomModel")

__all__ = ["PDB2CoordsOrdered", "PDB2CoordsUnordered", "writePDB", "pdb2sequence", "get_sequence", "convertStringList",
           "string2tensor", "tensor2string"]

_THREE_TO_ONE = {"ALA": "A", "ARG": "R", "ASN": "N", "ASP": "D", "CYS": "C", "GLN": "Q", "GLU": "E", "GLY": "G",
                 "HIS": "H", "ILE": "I", "LEU": "L", "LYS": "K", "MET": "M", "PHE": "F", "PRO": "P", "SER": "S",
                 "THR": "T", "TRP": "W", "TYR": "Y", "VAL": "V", "MSE": "M"}


def convertStringList(stringList):
    """List of strings -> NUL-terminated uint8 tensor [len, max_len + 1]."""
    maxlen = max([len(s) + 1 for s in stringList] + [1])
    ar = np.zeros((len(stringList), maxlen), dtype=np.uint8)
    for i, s in enumerate(stringList):
        b = s.encode("utf-8")
        ar[i, :len(b)] = np.frombuffer(b, dtype=np.uint8)
    return torch.from_numpy(ar)


def string2tensor(string):
    return torch.from_numpy(np.frombuffer((string + "\0").encode("utf-8"), dtype=np.uint8).copy())


def tensor2string(tensor):
    return bytes(tensor.cpu().numpy().tobytes()).split(b"\x00")[0].decode("utf-8", "strict")


class PDB2CoordsOrdered:
    """Name kept from the reference (PDB2Coords.py:54-70), whose native body is
    commented out; calling it raises.  ``PDB2CoordsUnordered`` reads the same files."""

    def __call__(self, filenames):
        raise NotImplementedError("PDB2CoordsOrdered has no implementation in the reference either; "
                                  "use PDB2CoordsUnordered")


class PDB2CoordsUnordered:
    def __call__(self, filenames):
        filenamesTensor = convertStringList(filenames)
        batch_size = len(filenames)
        num_atoms = torch.zeros(batch_size, dtype=torch.int)
        output_coords_cpu = torch.zeros(batch_size, 1, dtype=torch.double)
        output_chainnames_cpu = torch.zeros(batch_size, 1, 1, dtype=torch.uint8)
        output_resnames_cpu = torch.zeros(batch_size, 1, 1, dtype=torch.uint8)
        output_resnums_cpu = torch.zeros(batch_size, 1, dtype=torch.int)
        output_atomnames_cpu = torch.zeros(batch_size, 1, 1, dtype=torch.uint8)
        _FullAtomModel.PDB2CoordsUnordered(filenamesTensor, output_coords_cpu, output_chainnames_cpu,
                                           output_resnames_cpu, output_resnums_cpu, output_atomnames_cpu, num_atoms)
        return (output_coords_cpu, output_chainnames_cpu, output_resnames_cpu, output_resnums_cpu,
                output_atomnames_cpu, num_atoms)


def get_sequence(filename):
    """One-letter sequence of a PDB file's residues (chain, residue number) in file order."""
    _, chains, res, nums, _, n = PDB2CoordsUnordered()([filename])
    seq, last = [], None
    for j in range(int(n[0])):
        key = (tensor2string(chains[0, j]), int(nums[0, j]))
        if key == last:
            continue
        last = key
        name = tensor2string(res[0, j])
        if name not in _THREE_TO_ONE:
            raise Exception("Can't extract sequence")
        seq.append(_THREE_TO_ONE[name])
    return "".join(seq)


def pdb2sequence(filenames):
    return [get_sequence(f) for f in filenames]


def writePDB(filename, coords, chainnames, resnames, resnums, atomnames, num_atoms, bfactors=None, add_model=True,
             rewrite=True):
    """Write a batch as PDB ATOM records, one MODEL per chain (the reference's format)."""
    batch_size = coords.size(0)
    last_model_num = 0
    last_atom_num = 0
    if os.path.exists(filename):
        if rewrite:
            os.remove(filename)
        else:
            with open(filename, "r") as fin:
                for line in fin:
                    if line.find("MODEL") != -1:
                        last_model_num = max(last_model_num, int(line.split()[1]))
                    if line.find("ATOM") != -1:
                        last_atom_num = max(last_atom_num, int(line[6:11]))
    coords = coords.detach().cpu()
    with open(filename, "a") as fout:
        for i in range(batch_size):
            if add_model:
                fout.write("MODEL %d\n" % (i + last_model_num))
            for j in range(int(num_atoms[i])):
                chain_name = tensor2string(chainnames[i, j, :])
                if len(chain_name) == 0:
                    chain_name = "A"
                atom_name = tensor2string(atomnames[i, j, :])
                res_name = tensor2string(resnames[i, j, :])
                res_num = int(resnums[i, j])
                x, y, z = (float(coords[i, 3 * j + k]) for k in range(3))
                if bfactors is None:
                    fout.write("ATOM  %5d  %-3s %3s %c%4d    %8.3f%8.3f%8.3f\n" % (
                        j + last_atom_num + 1, atom_name, res_name, chain_name[0], res_num, x, y, z))
                else:
                    fout.write("ATOM  %5d  %-3s %3s %c%4d    %8.3f%8.3f%8.3f%6.2f%6.2f\n" % (
                        j + last_atom_num + 1, atom_name, res_name, chain_name[0], res_num, x, y, z, 1.0,
                        float(bfactors[i, j])))
            if add_model:
                fout.write("ENDMDL\n")
