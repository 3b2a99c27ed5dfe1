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
    """Strings -> uint8 tensor [len(stringList), longest + 1], one NUL-terminated row each."""
    raw = [s.encode("utf-8") for s in stringList]
    width = max(map(len, raw), default=0) + 1
    packed = b"".join(r.ljust(width, b"\0") for r in raw)
    return torch.from_numpy(np.frombuffer(packed, dtype=np.uint8).reshape(len(raw), width).copy())


def string2tensor(string):
    """A string -> NUL-terminated uint8 tensor."""
    return torch.tensor(list(string.encode("utf-8")) + [0], dtype=torch.uint8)


def tensor2string(tensor):
    """The bytes of a uint8 tensor up to its first NUL, decoded."""
    return bytes(tensor.cpu().numpy().tobytes()).split(b"\x00")[0].decode("utf-8", "strict")


class PDB2CoordsOrdered:
    """Name kept from the reference (PDB2Coords.py:54-70), whose native body is
    commented out; calling it raises.  ``PDB2CoordsUnordered`` reads the same files."""

    def __call__(self, filenames):
        raise NotImplementedError("PDB2CoordsOrdered has no implementation in the reference either; "
                                  "use PDB2CoordsUnordered")


class PDB2CoordsUnordered:
    """PDB files -> their heavy-atom ATOM records in file order, padded to the
    largest file: (coords f64 [B, 3N], chain_names, res_names u8 [B, N, 4],
    res_nums int32 [B, N], atom_names u8 [B, N, 4], num_atoms int32 [B])."""

    # (dtype, trailing shape) of each output; the native reader resizes them to N atoms
    _OUTPUTS = ((torch.double, (0,)), (torch.uint8, (0, 4)), (torch.uint8, (0, 4)), (torch.int, (0,)),
                (torch.uint8, (0, 4)))

    def __call__(self, filenames):
        n = len(filenames)
        outputs = [torch.empty((n,) + shape, dtype=dtype) for dtype, shape in self._OUTPUTS]
        num_atoms = torch.empty(n, dtype=torch.int)
        _FullAtomModel.PDB2CoordsUnordered(convertStringList(filenames), *outputs, num_atoms)
        return (*outputs, num_atoms)


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


def _last_numbers(filename):
    """The highest MODEL number and ATOM serial already in a PDB file (0 and 0 if none)."""
    model = serial = 0
    with open(filename) as f:
        for record in f:
            if record.startswith("MODEL"):
                model = max(model, int(record[5:].split()[0]))
            elif record.startswith("ATOM"):
                serial = max(serial, int(record[6:11]))
    return model, serial


def _names(t):
    """[B, N, 4] NUL-padded name slots -> lists of strings."""
    raw = t.detach().cpu().numpy()
    return [[bytes(slot).split(b"\x00")[0].decode("utf-8", "strict") for slot in row] for row in raw]


def _atom_record(serial, atom, res, chain, res_num, x, y, z, bfactor=None):
    """One ATOM record: serial in columns 7-11, atom name left-justified from column
    14, residue name 18-20, chain 22, residue number 23-26, x / y / z 31-54 (%8.3f),
    then occupancy 1.00 and the B-factor when one is given."""
    text = "ATOM  %5d  %-3s %3s %c%4d    %8.3f%8.3f%8.3f" % (serial, atom, res, chain, res_num, x, y, z)
    if bfactor is not None:
        text += "%6.2f%6.2f" % (1.0, bfactor)
    return text + "\n"


def writePDB(filename, coords, chainnames, resnames, resnums, atomnames, num_atoms, bfactors=None, add_model=True,
             rewrite=True):
    """Write a batch as PDB ATOM records, chain b as MODEL (first + b) when add_model.

    rewrite=True replaces an existing file.  rewrite=False appends: serials continue
    after the highest ATOM serial in the file, and the model numbers start at the
    highest MODEL number already there, as the reference numbers them.  A chain name
    that is empty is written as "A".  Only MODEL and ATOM records are scanned when
    appending (the reference matches those words anywhere in a line)."""
    first_model = first_serial = 0
    if os.path.exists(filename):
        if rewrite:
            os.remove(filename)
        else:
            first_model, first_serial = _last_numbers(filename)
    xyz = coords.detach().cpu().double().numpy()
    chains, res, atoms = _names(chainnames), _names(resnames), _names(atomnames)
    nums = resnums.detach().cpu().numpy()
    counts = [int(v) for v in num_atoms]
    bf = None if bfactors is None else bfactors.detach().cpu().double().numpy()
    records = []
    for b, count in enumerate(counts):
        if add_model:
            records.append("MODEL %d\n" % (first_model + b))
        records.extend(_atom_record(first_serial + j + 1, atoms[b][j], res[b][j], chains[b][j][:1] or "A",
                                    int(nums[b, j]), *xyz[b, 3 * j:3 * j + 3], None if bf is None else bf[b, j])
                       for j in range(count))
        if add_model:
            records.append("ENDMDL\n")
    with open(filename, "a") as f:
        f.writelines(records)
