"""ctypes binding of libtpl_gb300.so (the C ABI of include/tpl_gb300.h).

This is the binding a non-torch host would write; the tests use it to drive the
kernels through the C ABI directly, with tensors standing in for device buffers.
"""
from __future__ import annotations

import ctypes
import os
import re

from . import native_library_path

_LIB = None

_vp = ctypes.c_void_p
_i = ctypes.c_int
_sz = ctypes.c_size_t


class tpl_options(ctypes.Structure):
    _fields_ = [("residues_per_thread", _i), ("threads_per_cta", _i), ("fp64_carry_min_len", _i),
                ("renormalize", _i), ("max_ctas", _i), ("copy_buffers", _i)]


_SIGNATURES = {
    "tpl_status_string": (ctypes.c_char_p, [_i]),
    "tpl_version": (_i, []),
    "tpl_a2b_workspace_bytes": (_sz, [_i, _i, _vp]),
    "tpl_workspace_init": (_i, [_vp, _sz, _vp]),
    "tpl_workspace_status": (_i, [_vp, _vp, ctypes.POINTER(_i)]),
    "tpl_a2b_forward_f32": (_i, [_vp, _vp, _vp, _vp, _sz, _i, _i, _vp, _vp]),
    "tpl_a2b_backward_f32": (_i, [_vp, _vp, _vp, _vp, _vp, _sz, _i, _i, _vp, _vp]),
    "tpl_a2b_backward_coords_f32": (_i, [_vp, _vp, _vp, _vp, _vp, _sz, _i, _i, _vp, _vp]),
    "tpl_a2b_forward_f64": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "tpl_a2b_backward_f64": (_i, [_vp, _vp, _vp, _vp, _vp, _sz, _i, _i, _vp]),
    "tpl_num_atoms": (_i, [ctypes.c_char_p]),
    "tpl_a2c_workspace_bytes": (_sz, [_i, _i, _i, _vp]),
    "tpl_a2c_forward_f32": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _sz, _i, _i, _i, _vp, _vp]),
    "tpl_a2c_backward_f32": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _i, _i, _i, _vp, _vp]),
    "tpl_a2c_forward_f64": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _sz, _i, _i, _i, _vp, _vp]),
    "tpl_a2c_backward_f64": (_i, [_vp, _vp, _vp, _i, _vp, _vp, _sz, _i, _i, _i, _vp, _vp]),
    "tpl_a2c_backward_coords_f32": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _sz, _i, _i, _i, _vp]),
    "tpl_a2b_forward_f32_noalloc": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp]),
    "tpl_a2b_noalloc_status": (_i, [_vp, ctypes.POINTER(_i)]),
    "tpl_sincos_f32": (_i, [_vp, _vp, _vp, _i, _vp]),
    "tpl_coords_translate_f32": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_translate_f64": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_rotate_f32": (_i, [_vp, _vp, _vp, _i, _vp, _i, _i, _vp]),
    "tpl_coords_rotate_f64": (_i, [_vp, _vp, _vp, _i, _vp, _i, _i, _vp]),
    "tpl_coords_center_f32": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_center_f64": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_center_backward_f32": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_center_backward_f64": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_bbox_f32": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp]),
    "tpl_coords_bbox_f64": (_i, [_vp, _vp, _vp, _vp, _i, _i, _vp]),
    "tpl_typed_coords_forward_f32": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "tpl_typed_coords_forward_f64": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
    "tpl_typed_coords_backward_f32": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _vp]),
    "tpl_typed_coords_backward_f64": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _vp]),
    "tpl_pdb_count_atoms": (_i, [ctypes.c_char_p, _vp]),
    "tpl_pdb_read_batch": (_i, [ctypes.POINTER(ctypes.c_char_p), _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i]),
    "tpl_rmsd_forward_f32": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _sz, _vp]),
    "tpl_rmsd_forward_f64": (_i, [_vp, _vp, _vp, _i, _i, _i, _vp, _vp, _vp, _vp, _sz, _vp]),
    "tpl_rmsd_backward_f32": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp]),
    "tpl_rmsd_backward_f64": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp]),
}


def lib():
    """Load libtpl_gb300.so (raises OSError when it is not built)."""
    global _LIB
    if _LIB is None:
        l = ctypes.CDLL(native_library_path())
        for name, (res, args) in _SIGNATURES.items():
            if hasattr(l, name):
                f = getattr(l, name)
                f.restype = res
                f.argtypes = args
        _LIB = l
    return _LIB


def declared_symbols(header: str | None = None) -> list[str]:
    """Function names declared in include/tpl_gb300.h."""
    if header is None:
        header = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "tpl_gb300.h")
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tpl_[a-z0-9_]+)\s*\(", text)))


def check(status: int, what: str = "call") -> None:
    if status != 0:
        msg = lib().tpl_status_string(status).decode()
        raise RuntimeError(f"{what}: {msg} ({status})")


def options(**kw) -> tpl_options:
    o = tpl_options()
    for k, v in kw.items():
        setattr(o, k, int(v))
    return o


def ptr(t) -> int:
    return t.data_ptr() if t is not None else None


def stream_ptr(device=None) -> int:
    import torch

    return torch.cuda.current_stream(device).cuda_stream
