"""Build the reference's own CPU interfaces of CoordsTransform,
Coords2TypedCoords and Coords2RMSD as one torch extension (test infrastructure).

The sources are compiled unmodified where they lie in the reference checkout:

* Layers/FullAtomModel/CoordsTransform/coordsTransform_interface.cpp
* Layers/FullAtomModel/Coords2TypedCoords/coords2typedcoords_interface.cpp
* Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp
* Math/nUtil.cpp, Math/cVector3.cpp, Math/cMatrix33.cpp, Math/cMatrix44.cpp

``oracle/ref_shim_torch/nUtil.h`` stands in for Math/nUtil.h (it bridges the
torch 2.x API changes, including the removed Tensor::eig) and
``oracle/ref_ext_main.cpp`` binds the entry points.  The module is written to
``oracle/_ref/`` (git-ignored) and imported as ``_tplref``.

    python oracle/build_ref_ext.py [reference checkout]
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref", "ext_build")


def build(ref: str, verbose: bool = False):
    """Compile (if stale) and import the extension; returns the module."""
    from torch.utils.cpp_extension import load

    ref = os.path.abspath(ref)
    srcs = [
        os.path.join(HERE, "ref_ext_main.cpp"),
        os.path.join(ref, "Layers/FullAtomModel/CoordsTransform/coordsTransform_interface.cpp"),
        os.path.join(ref, "Layers/FullAtomModel/Coords2TypedCoords/coords2typedcoords_interface.cpp"),
        os.path.join(ref, "Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp"),
        os.path.join(ref, "Math/nUtil.cpp"),
        os.path.join(ref, "Math/cVector3.cpp"),
        os.path.join(ref, "Math/cMatrix33.cpp"),
        os.path.join(ref, "Math/cMatrix44.cpp"),
    ]
    for s in srcs:
        if not os.path.exists(s):
            raise FileNotFoundError(s)
    incs = [os.path.join(HERE, "ref_shim_torch"), os.path.join(ref, "Math"), os.path.join(ref, "Layers/FullAtomModel"),
            os.path.join(ref, "Layers/RMSD"), os.path.join(ref, "Layers/ReducedModel")]
    os.makedirs(OUT, exist_ok=True)
    return load(name="_tplref", sources=srcs, extra_include_paths=incs, build_directory=OUT,
                extra_cflags=["-O2", "-w", "-fopenmp"], extra_ldflags=["-fopenmp"], verbose=verbose)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    import oracle

    m = build(sys.argv[1] if len(sys.argv) > 1 else oracle.reference_dir(), verbose=True)
    print("built", m.__file__)
