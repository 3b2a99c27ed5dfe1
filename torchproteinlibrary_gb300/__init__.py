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


_ALIAS = "TorchProteinLibrary"
_ALIASED_PACKAGES = ("ReducedModel", "FullAtomModel", "RMSD")


def install_alias() -> None:
    """Make ``import TorchProteinLibrary`` and every module below its ReducedModel,
    FullAtomModel and RMSD packages (``TorchProteinLibrary.FullAtomModel.CoordsTransform``
    and so on), as well as the bare extension names ``_ReducedModel``,
    ``_FullAtomModel`` and ``_RMSD``, resolve to this package's modules.

    Each alias is the same module object as the original, so classes compare
    identical whichever name imported them.  Names already present in
    ``sys.modules`` (an installed reference, say) are left alone."""
    import pkgutil

    sys.modules.setdefault(_ALIAS, sys.modules[__name__])
    for sub in _ALIASED_PACKAGES:
        pkg = importlib.import_module(f"{__name__}.{sub}")
        for info in pkgutil.walk_packages(pkg.__path__, prefix=f"{pkg.__name__}."):
            importlib.import_module(info.name)
    prefix = f"{__name__}."
    for name, module in list(sys.modules.items()):
        if name.startswith(prefix) and name[len(prefix):].split(".")[0] in _ALIASED_PACKAGES:
            sys.modules.setdefault(_ALIAS + name[len(__name__):], module)
    for ext in ("_ReducedModel", "_FullAtomModel", "_RMSD"):
        sys.modules.setdefault(ext, load_extension(ext))
