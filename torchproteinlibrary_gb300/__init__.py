"""GB300 (sm_103a) implementation of TorchProteinLibrary's internal-coordinate
chain kinematics: ``ReducedModel.Angles2Backbone`` and
``FullAtomModel.Angles2Coords``, with the reference's module paths, class names,
argument order and output layouts.

The compute runs in ``lib/libtpl_gb300.so`` (hand-written CUDA behind the C ABI
of ``include/tpl_gb300.h``); the ``_ReducedModel`` / ``_FullAtomModel`` extension
modules keep the reference's entry-point names.  There is no CPU path: CPU
tensors raise.  ``install_alias()`` registers this package under the reference's
import name ``TorchProteinLibrary``.
"""
from __future__ import annotations

import importlib
import os
import sys

__version__ = "0.1.0"

_PKG = os.path.dirname(os.path.abspath(__file__))


def native_library_path() -> str:
    return os.path.join(_PKG, "lib", "libtpl_gb300.so")


def load_extension(name: str):
    """Import one of the in-tree extension modules (``_ReducedModel``, ``_FullAtomModel``).

    Raises ImportError with the build command when the module has not been
    built: the layers have no fallback."""
    full = f"{__name__}.{name}"
    try:
        return importlib.import_module(full)
    except ImportError as e:  # pragma: no cover - exercised on unbuilt trees
        raise ImportError(
            f"{full} is not built ({e}); run `python -c \"import __graft_entry__ as g; g.build()\"` "
            f"or `python -m torchproteinlibrary_gb300._build`") from e


def install_alias() -> None:
    """Make ``import TorchProteinLibrary`` (and its ReducedModel / FullAtomModel
    sub-packages) resolve to this package."""
    from . import RMSD, FullAtomModel, ReducedModel  # noqa: F401

    sys.modules.setdefault("TorchProteinLibrary", sys.modules[__name__])
    for sub in ("ReducedModel", "FullAtomModel", "RMSD"):
        sys.modules.setdefault(f"TorchProteinLibrary.{sub}", sys.modules[f"{__name__}.{sub}"])
    for ext in ("_ReducedModel", "_FullAtomModel", "_RMSD"):
        sys.modules.setdefault(ext, load_extension(ext))
