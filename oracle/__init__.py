"""ORACLE -- test infrastructure only.

CPU checkers for the internal-coordinate chain kinematics path:

* ``port``: ``oracle/tpl_oracle.c``, a plain-C FP64 restatement of the reference
  algorithms (Angles2Backbone: Layers/ReducedModel/cBackboneProteinCPUKernels.cpp:14-145;
  Angles2Coords: Layers/FullAtomModel/cConformation.cpp:30-211 with the residue
  templates of cConformationAA.cpp and cRigidGroup.cpp).
* ``ref``: the reference's own CPU kinematics sources compiled unmodified into
  ``oracle/_ref/libtplref.so`` (``make -C oracle ref``), when they were built.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline
leg and ``--impl reference``) may import this package.  The product path
(``torchproteinlibrary_gb300``) never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_PORT = None
_REF = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_up = ctypes.POINTER(ctypes.c_ubyte)


def reference_dir() -> str | None:
    """The reference checkout that the oracle's reference builds read: the
    TPL_REFERENCE_DIR environment variable, else the REF default of
    oracle/Makefile (the one place that names the conventional location).
    None when that directory does not exist (e.g. on a machine without it)."""
    d = os.environ.get("TPL_REFERENCE_DIR")
    if not d:
        with open(os.path.join(HERE, "Makefile")) as f:
            for line in f:
                if line.startswith("REF") and "?=" in line:
                    d = line.split("?=", 1)[1].strip()
                    break
    return d if d and os.path.isdir(d) else None


def build(ref_dir: str | None = None) -> None:
    """Compile the C restatement, and the reference sources when ``ref_dir`` exists."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref_dir and os.path.isdir(ref_dir):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_dir}"], check=True)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def port():
    global _PORT
    if _PORT is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.oracle_a2b_forward.argtypes = [_dp, _ip, _dp, _dp, ctypes.c_int, ctypes.c_int]
        lib.oracle_a2b_backward.argtypes = [_dp, _dp, _dp, _ip, _dp, ctypes.c_int, ctypes.c_int]
        lib.oracle_num_atoms.argtypes = [ctypes.c_char_p]
        lib.oracle_a2c_forward.argtypes = [_up, ctypes.c_int, _dp, _dp, _up, _up, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int]
        lib.oracle_a2c_backward.argtypes = [_dp, _dp, _up, ctypes.c_int, _dp, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int]
        _PORT = lib
    return _PORT


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libtplref.so"))


def ref():
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libtplref.so")
        lib = ctypes.CDLL(path)
        i = ctypes.c_int
        lib.ref_a2b_forward.argtypes = [_dp, _ip, _dp, _dp, i, i, i]
        lib.ref_a2b_backward.argtypes = [_dp, _dp, _dp, _ip, _dp, _dp, i, i, i]
        lib.ref_a2c_forward.argtypes = [_up, i, _dp, _dp, _up, _up, i, i, i, i]
        lib.ref_a2c_backward.argtypes = [_dp, _dp, _up, i, _dp, i, i, i, i]
        _REF = lib
    return _REF


# ----------------------------------------------------------------- helpers
def seq_bytes(seqs: list[str]) -> np.ndarray:
    """NUL-terminated byte rows, as TorchProteinLibrary/FullAtomModel/Angles2Coords/Angles2Coords.py:12-26."""
    width = max(len(s) for s in seqs) + 1 if seqs else 1
    out = np.zeros((len(seqs), width), dtype=np.uint8)
    for i, s in enumerate(seqs):
        out[i, : len(s)] = np.frombuffer(s.encode("ascii"), dtype=np.uint8)
    return out


def num_atoms(seq: str) -> int:
    n = port().oracle_num_atoms(seq.encode("ascii"))
    if n < 0:
        raise ValueError(f"unknown residue letter in {seq!r}")
    return n


def a2b_forward(angles: np.ndarray, lengths: np.ndarray, impl: str = "port", threads: int = 1):
    """angles [B,3,L] f64, lengths [B] int32 -> (coords [B,9L], A [B,48L])."""
    angles = np.ascontiguousarray(angles, dtype=np.float64)
    lengths = np.ascontiguousarray(lengths, dtype=np.int32)
    B, _, L = angles.shape
    coords = np.zeros((B, 9 * L))
    A = np.zeros((B, 48 * L))
    if impl == "ref":
        rc = ref().ref_a2b_forward(_ptr(angles, _dp), _ptr(lengths, _ip), _ptr(coords, _dp), _ptr(A, _dp), B, L,
                                   threads)
    else:
        rc = port().oracle_a2b_forward(_ptr(angles, _dp), _ptr(lengths, _ip), _ptr(coords, _dp), _ptr(A, _dp), B, L)
    if rc != 0:
        raise RuntimeError(f"a2b_forward failed ({rc})")
    return coords, A


def a2b_backward(grad_coords: np.ndarray, angles: np.ndarray, lengths: np.ndarray, A: np.ndarray,
                 impl: str = "port", threads: int = 1) -> np.ndarray:
    """Returns dL/dangles [B,3,L].  impl='ref' returns the reference's raw values
    (including its omega[len-1] entry, which reads one matrix past the chain)."""
    angles = np.ascontiguousarray(angles, dtype=np.float64)
    lengths = np.ascontiguousarray(lengths, dtype=np.int32)
    grad_coords = np.ascontiguousarray(grad_coords, dtype=np.float64)
    B, _, L = angles.shape
    out = np.zeros((B, 3, L))
    if impl == "ref":
        dr = np.zeros(27 * L * L * max(1, threads))
        rc = ref().ref_a2b_backward(_ptr(out, _dp), _ptr(grad_coords, _dp), _ptr(angles, _dp), _ptr(lengths, _ip),
                                    _ptr(A, _dp), _ptr(dr, _dp), B, L, threads)
    else:
        rc = port().oracle_a2b_backward(_ptr(out, _dp), _ptr(grad_coords, _dp), _ptr(angles, _dp),
                                        _ptr(lengths, _ip), _ptr(A, _dp), B, L)
    if rc != 0:
        raise RuntimeError(f"a2b_backward failed ({rc})")
    return out


def a2c_forward(angles: np.ndarray, seqs: list[str], impl: str = "port", threads: int = 1):
    """angles [B,8,L] f64 -> (coords [B,3*maxA], res_names u8 [B,maxA,4], atom_names u8 [B,maxA,4], num_atoms)."""
    angles = np.ascontiguousarray(angles, dtype=np.float64)
    B, _, L = angles.shape
    sb = seq_bytes(seqs)
    na = np.array([num_atoms(s) for s in seqs], dtype=np.int32)
    maxA = int(na.max()) if B else 0
    coords = np.zeros((B, 3 * maxA))
    rn = np.zeros((B, maxA, 4), dtype=np.uint8)
    an = np.zeros((B, maxA, 4), dtype=np.uint8)
    if impl == "ref":
        rc = ref().ref_a2c_forward(_ptr(sb, _up), sb.shape[1], _ptr(angles, _dp), _ptr(coords, _dp), _ptr(rn, _up),
                                   _ptr(an, _up), B, L, maxA, threads)
    else:
        rc = port().oracle_a2c_forward(_ptr(sb, _up), sb.shape[1], _ptr(angles, _dp), _ptr(coords, _dp),
                                       _ptr(rn, _up), _ptr(an, _up), B, L, maxA)
    if rc != 0:
        raise RuntimeError(f"a2c_forward failed ({rc})")
    return coords, rn, an, na


def a2c_backward(grad_coords: np.ndarray, angles: np.ndarray, seqs: list[str], impl: str = "port",
                 threads: int = 1) -> np.ndarray:
    angles = np.ascontiguousarray(angles, dtype=np.float64)
    grad_coords = np.ascontiguousarray(grad_coords, dtype=np.float64)
    B, _, L = angles.shape
    sb = seq_bytes(seqs)
    maxA = grad_coords.shape[1] // 3
    out = np.zeros((B, 8, L))
    if impl == "ref":
        rc = ref().ref_a2c_backward(_ptr(grad_coords, _dp), _ptr(out, _dp), _ptr(sb, _up), sb.shape[1],
                                    _ptr(angles, _dp), B, L, maxA, threads)
    else:
        rc = port().oracle_a2c_backward(_ptr(grad_coords, _dp), _ptr(out, _dp), _ptr(sb, _up), sb.shape[1],
                                        _ptr(angles, _dp), B, L, maxA)
    if rc != 0:
        raise RuntimeError(f"a2c_backward failed ({rc})")
    return out


def a2c_save_ref(seq: str, angles: np.ndarray, filename: str, mode: str) -> None:
    """The reference's Angles2Coords_save (angles2coords_interface.cpp:117-137 ->
    cConformation::save, cConformation.cpp:228-262) for one chain, angles [8, len(seq)]."""
    angles = np.ascontiguousarray(angles, dtype=np.float64)
    if angles.shape != (8, len(seq)):
        raise ValueError("the reference reads angles with the sequence length as row stride")
    lib = ref()
    lib.ref_a2c_save.argtypes = [ctypes.c_char_p, _dp, ctypes.c_char_p, ctypes.c_char]
    if lib.ref_a2c_save(seq.encode(), _ptr(angles, _dp), filename.encode(), mode.encode()) != 0:
        raise RuntimeError("reference save failed")


# ------------------------------------------------------------------ Coords2RMSD
def rmsd(src: np.ndarray, dst: np.ndarray, num_atoms, center: bool = True):
    """Least RMSD per chain after optimal superposition, restating the reference's
    CPU path (Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp:113-183: FP64
    correlation R, 4x4 quaternion matrix, largest eigenpair, rmsd =
    sqrt((R2 - 2|lambda| + 1e-10)/N), UT = U^T) with the centring of
    TorchProteinLibrary/RMSD/Coords2RMSD/Coords2RMSD.py:71-78.  The reference solves
    the eigen problem with torch's eig; this uses numpy.linalg.eigh (symmetric).
    Returns (rmsd [B], UT [B,3,3], grad_factor) where dL/dsrc = g * grad_factor[b]."""
    src = np.asarray(src, dtype=np.float64)
    dst = np.asarray(dst, dtype=np.float64)
    B = src.shape[0]
    out = np.zeros(B)
    UT = np.zeros((B, 3, 3))
    grads = np.zeros_like(src)
    for b in range(B):
        n = int(num_atoms[b])
        x = src[b, :3 * n].reshape(n, 3)
        y = dst[b, :3 * n].reshape(n, 3)
        if center and n:
            x = x - x.mean(0)
            y = y - y.mean(0)
        R = x.T @ y
        F = np.array([
            [R[0, 0] + R[1, 1] + R[2, 2], R[1, 2] - R[2, 1], R[2, 0] - R[0, 2], R[0, 1] - R[1, 0]],
            [R[1, 2] - R[2, 1], R[0, 0] - R[1, 1] - R[2, 2], R[0, 1] + R[1, 0], R[0, 2] + R[2, 0]],
            [R[2, 0] - R[0, 2], R[0, 1] + R[1, 0], -R[0, 0] + R[1, 1] - R[2, 2], R[1, 2] + R[2, 1]],
            [R[0, 1] - R[1, 0], R[0, 2] + R[2, 0], R[1, 2] + R[2, 1], -R[0, 0] - R[1, 1] + R[2, 2]]])
        w, v = np.linalg.eigh(F)
        lam, q = w[-1], v[:, -1]
        U = np.array([
            [q[0] ** 2 + q[1] ** 2 - q[2] ** 2 - q[3] ** 2, 2 * (q[1] * q[2] - q[0] * q[3]), 2 * (q[1] * q[3] + q[0] * q[2])],
            [2 * (q[1] * q[2] + q[0] * q[3]), q[0] ** 2 - q[1] ** 2 + q[2] ** 2 - q[3] ** 2, 2 * (q[2] * q[3] - q[0] * q[1])],
            [2 * (q[1] * q[3] - q[0] * q[2]), 2 * (q[2] * q[3] + q[0] * q[1]), q[0] ** 2 - q[1] ** 2 - q[2] ** 2 + q[3] ** 2]])
        UT[b] = U.T
        R2 = (x ** 2).sum() + (y ** 2).sum()
        out[b] = np.sqrt(max((R2 - 2 * abs(lam) + 1e-10) / max(n, 1), 0.0)) if n else 0.0
        if n and out[b] > 0:
            # Coords2RMSD.py:48-56: (x - UT y) / (rmsd N), UT applied as out = UT @ y
            grads[b, :3 * n] = ((x - y @ UT[b].T) / (out[b] * n)).reshape(-1)
    return out, UT, grads


# -------------------------------------------------------------- CoordsTransform
# Restatements of Layers/FullAtomModel/TransformCUDAKernels.cu:4-107 and
# Math/nUtil.cpp:27-79 on [B, 3 * atoms_stride] rows; atoms past num_atoms[b] are 0.
def coords_translate(x: np.ndarray, T, num_atoms) -> np.ndarray:
    """out = x + T[b] for the first num_atoms[b] atoms (T None: the masked copy, the backward)."""
    x = np.asarray(x)
    out = np.zeros_like(x)
    for b, n in enumerate(num_atoms):
        n = int(min(max(n, 0), x.shape[1] // 3))
        v = x[b, :3 * n].reshape(n, 3)
        out[b, :3 * n] = (v + (0 if T is None else np.asarray(T)[b])).reshape(-1)
    return out


def coords_rotate(x: np.ndarray, R, num_atoms, transpose: bool = False) -> np.ndarray:
    """out = R[b] x (transpose: R[b]^T x) per atom, mat33Vec3Mul of the reference."""
    x = np.asarray(x)
    out = np.zeros_like(x)
    for b, n in enumerate(num_atoms):
        n = int(min(max(n, 0), x.shape[1] // 3))
        M = np.asarray(R)[b].T if transpose else np.asarray(R)[b]
        out[b, :3 * n] = (x[b, :3 * n].reshape(n, 3) @ M.T).reshape(-1)
    return out


def coords_center(x: np.ndarray, num_atoms) -> np.ndarray:
    """Mean of the first num_atoms[b] atoms (0 for an empty chain)."""
    x = np.asarray(x)
    out = np.zeros((x.shape[0], 3), dtype=x.dtype)
    for b, n in enumerate(num_atoms):
        n = int(min(max(n, 0), x.shape[1] // 3))
        if n:
            out[b] = x[b, :3 * n].reshape(n, 3).astype(np.float64).mean(0)
    return out


def coords_center_backward(grad_center, num_atoms, atoms_stride: int) -> np.ndarray:
    g = np.asarray(grad_center)
    out = np.zeros((g.shape[0], 3 * atoms_stride), dtype=g.dtype)
    for b, n in enumerate(num_atoms):
        n = int(min(max(n, 0), atoms_stride))
        if n:
            out[b, :3 * n] = np.tile(g[b] / n, n)
    return out


def coords_bbox(x: np.ndarray, num_atoms):
    """Per-coordinate min / max of the first num_atoms[b] atoms (+inf / -inf when empty)."""
    x = np.asarray(x)
    lo = np.full((x.shape[0], 3), np.inf, dtype=x.dtype)
    hi = np.full((x.shape[0], 3), -np.inf, dtype=x.dtype)
    for b, n in enumerate(num_atoms):
        n = int(min(max(n, 0), x.shape[1] // 3))
        if n:
            v = x[b, :3 * n].reshape(n, 3)
            lo[b], hi[b] = v.min(0), v.max(0)
    return lo, hi


def rotation_from_u(u: np.ndarray) -> np.ndarray:
    """Math/nUtil.cpp:60-79: rotation matrix of the quaternion built from u in [0,1)^3."""
    u = np.asarray(u, dtype=np.float64)
    out = np.zeros((u.shape[0], 3, 3))
    for b, (u1, u2, u3) in enumerate(u):
        q = [np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
             np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)]
        out[b] = [[q[0] ** 2 + q[1] ** 2 - q[2] ** 2 - q[3] ** 2, 2 * (q[1] * q[2] - q[0] * q[3]),
                   2 * (q[1] * q[3] + q[0] * q[2])],
                  [2 * (q[1] * q[2] + q[0] * q[3]), q[0] ** 2 - q[1] ** 2 + q[2] ** 2 - q[3] ** 2,
                   2 * (q[2] * q[3] - q[0] * q[1])],
                  [2 * (q[1] * q[3] - q[0] * q[2]), 2 * (q[2] * q[3] + q[0] * q[1]),
                   q[0] ** 2 - q[1] ** 2 - q[2] ** 2 + q[3] ** 2]]
    return out


# ----------------------------------------------------------- Coords2TypedCoords
# Restatement of ProtUtil::get11AtomType (Math/nUtil.cpp:567-703, terminal = false,
# 0-based as it returns) and of Coords2TypedCoords_forward / _backward
# (Layers/FullAtomModel/Coords2TypedCoords/coords2typedcoords_interface.cpp).
_TYPE_GROUPS = {
    0: ["CYSSG", "METSD", "MSESE"],
    1: ["ASNND2", "GLNNE2"],
    2: ["HISND1", "HISNE2", "TRPNE1"],
    3: ["ARGNH1", "ARGNH2", "ARGNE"],
    4: ["LYSNZ"],
    5: ["ACEO", "ASNOD1", "GLNOE1"],
    6: ["SEROG", "THROG1", "TYROH"],
    7: ["ASPOD1", "ASPOD2", "GLUOE1", "GLUOE2"],
    8: ["ARGCZ", "ASPCG", "GLUCD", "ACEC", "ASNCG", "GLNCD"],
    9: ["HISCD2", "HISCE1", "HISCG", "PHECD1", "PHECD2", "PHECE1", "PHECE2", "PHECG", "PHECZ",
        "TRPCD1", "TRPCD2", "TRPCE2", "TRPCE3", "TRPCG", "TRPCH2", "TRPCZ2", "TRPCZ3",
        "TYRCD1", "TYRCD2", "TYRCE1", "TYRCE2", "TYRCG", "TYRCZ"],
    10: ["ALACB", "ARGCB", "ARGCG", "ARGCD", "ASNCB", "ASPCB", "GLNCB", "GLNCG", "GLUCB", "GLUCG", "HISCB",
         "ILECB", "ILECD1", "ILECG1", "ILECG2", "LEUCB", "LEUCD1", "LEUCD2", "LEUCG",
         "LYSCB", "LYSCD", "LYSCG", "LYSCE", "METCB", "METCE", "METCG", "MSECB", "MSECE", "MSECG",
         "PHECB", "PROCB", "PROCG", "PROCD", "SERCB", "THRCG2", "TRPCB", "TYRCB",
         "VALCB", "VALCG1", "VALCG2", "ACECH3", "THRCB", "CYSCB"],
}
_FULL_NAME_TYPE = {name: t for t, names in _TYPE_GROUPS.items() for name in names}


def atom_type_11(res: str, atom: str) -> int:
    """0-based atom type, or -1 where the reference throws."""
    atom = "".join(atom.split())
    if atom == "O":
        return 5
    if atom in ("OXT", "OT2"):
        return 7
    if atom == "N":
        return 1
    if atom == "C":
        return 8
    if atom == "CA":
        return 10
    return _FULL_NAME_TYPE.get(res + atom, -1)


def _name(slot) -> str:
    b = bytes(slot)
    return b.split(b"\0", 1)[0].decode("ascii")


def typed_coords(coords: np.ndarray, res_names: np.ndarray, atom_names: np.ndarray, num_atoms, out_stride=None):
    """(typed [B, 3 out_stride], num_atoms_of_type [B, 11], offsets [B, 11], atom_indexes [B, out_stride])."""
    coords = np.asarray(coords)
    B = coords.shape[0]
    S = out_stride if out_stride is not None else int(max(num_atoms)) if B else 0
    typed = np.zeros((B, 3 * S), dtype=coords.dtype)
    counts = np.zeros((B, 11), dtype=np.int32)
    offsets = np.zeros((B, 11), dtype=np.int32)
    index = np.zeros((B, S), dtype=np.int32)
    for b in range(B):
        n = int(num_atoms[b])
        types = [atom_type_11(_name(res_names[b, j]), _name(atom_names[b, j])) for j in range(n)]
        for t in types:
            counts[b, t] += 1
        offsets[b, 1:] = np.cumsum(counts[b])[:-1]
        added = np.zeros(11, dtype=np.int64)
        for j, t in enumerate(types):
            slot = offsets[b, t] + added[t]
            typed[b, 3 * slot:3 * slot + 3] = coords[b, 3 * j:3 * j + 3]
            index[b, slot] = j
            added[t] += 1
    return typed, counts, offsets, index


def typed_coords_backward(grad_typed: np.ndarray, counts, index, in_stride: int) -> np.ndarray:
    grad_typed = np.asarray(grad_typed)
    B = grad_typed.shape[0]
    out = np.zeros((B, 3 * in_stride), dtype=grad_typed.dtype)
    for b in range(B):
        for s in range(int(np.sum(counts[b]))):
            j = index[b, s]
            out[b, 3 * j:3 * j + 3] = grad_typed[b, 3 * s:3 * s + 3]
    return out


# ------------------------------------------------------------------ PDB reading
def pdb_read(filename: str, impl: str = "port"):
    """Heavy-atom ATOM records of a PDB file as the reference's cPDBLoader reads them
    (Layers/FullAtomModel/cPDBLoader.cpp:25-55): (coords [n, 3] f64, chain_names,
    res_names, atom_names as lists of str, res_nums int32 [n]).  impl="ref" runs the
    reference's own reader (oracle/_ref); "port" restates it: a line whose first four
    characters are "ATOM", atom name = columns 13-16 trimmed and starting with
    C/N/O/S, x/y/z = columns 31-38/39-46/47-54 read as float32, residue name =
    columns 18-20, chain = column 22, residue number = columns 23-26."""
    if impl == "ref":
        lib = ref()
        lib.ref_pdb_read.restype = ctypes.c_int
        lib.ref_pdb_read.argtypes = [ctypes.c_char_p, ctypes.c_int, _dp, ctypes.c_char_p, ctypes.c_char_p, _ip,
                                     ctypes.c_char_p]
        n = lib.ref_pdb_read(filename.encode(), 0, None, None, None, None, None)
        if n < 0:
            raise RuntimeError(f"reference PDB reader failed on {filename}")
        coords = np.zeros((max(n, 1), 3))
        names = [ctypes.create_string_buffer(4 * max(n, 1)) for _ in range(3)]
        nums = np.zeros(max(n, 1), dtype=np.int32)
        lib.ref_pdb_read(filename.encode(), n, _ptr(coords, _dp), names[0], names[1], _ptr(nums, _ip), names[2])
        dec = [[buf.raw[4 * j:4 * j + 4].split(b"\0", 1)[0].decode() for j in range(n)] for buf in names]
        return coords[:n], dec[0], dec[1], dec[2], nums[:n]
    coords, chains, res, atoms, nums = [], [], [], [], []
    with open(filename) as f:
        for line in f:
            line = line.rstrip("\n")
            if not line.startswith("ATOM"):
                continue
            name = line[12:16].strip()
            if not name or name[0] not in "CNOS":
                continue
            coords.append([float(np.float32(line[k:k + 8])) for k in (30, 38, 46)])
            res.append(line[17:20].strip())
            chains.append(line[21:22].strip())
            nums.append(int(line[22:26]))
            atoms.append(name)
    return np.array(coords, dtype=np.float64).reshape(-1, 3), chains, res, atoms, np.array(nums, dtype=np.int32)
