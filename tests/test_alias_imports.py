"""The reference's own import forms, after ``install_alias()``, reach this package.

Runs in a fresh interpreter so that the aliases do not leak into the rest of the
session.  No GPU: only imports, module identity and the extension entry-point
names are checked (the names the reference's layer files call, e.g.
Layers/ReducedModel/main.cpp:4-9, Layers/FullAtomModel/main.cpp:13-42).
"""
import subprocess
import sys
import textwrap

from conftest import ROOT

SCRIPT = textwrap.dedent("""
    import sys
    import torchproteinlibrary_gb300 as t
    t.install_alias()

    from TorchProteinLibrary import ReducedModel, FullAtomModel, RMSD
    from TorchProteinLibrary.ReducedModel.Angles2Backbone import (
        Angles2Backbone, Angles2BackboneCPUFunction, Angles2BackboneGPUFunction)
    from TorchProteinLibrary.FullAtomModel import (
        Angles2Coords, Coords2TypedCoords, CoordsTranslate, CoordsRotate, Coords2Center,
        getBBox, getRandomRotation, getRandomTranslation, PDB2CoordsUnordered, writePDB)
    from TorchProteinLibrary.FullAtomModel.CoordsTransform import (
        CoordsTranslate as CT2, getBBox as gb2, CoordsRotate as CR2, getRandomRotation as grr2,
        Coords2Center as CC2)
    from TorchProteinLibrary.FullAtomModel.PDB2Coords import PDB2CoordsOrdered, PDB2CoordsUnordered as PU2
    from TorchProteinLibrary.RMSD import Coords2RMSD
    import TorchProteinLibrary.FullAtomModel.CoordsTransform.CoordsTransform
    import _ReducedModel, _FullAtomModel, _RMSD
    ctm = sys.modules["TorchProteinLibrary.FullAtomModel.CoordsTransform.CoordsTransform"]

    # one module object per file, whichever name imported it
    assert ctm is sys.modules["torchproteinlibrary_gb300.FullAtomModel.CoordsTransform.CoordsTransform"]
    assert Angles2Backbone is t.ReducedModel.Angles2Backbone
    assert CT2 is CoordsTranslate and CC2 is Coords2Center and PU2 is PDB2CoordsUnordered
    assert _ReducedModel is t.load_extension("_ReducedModel")
    dup = [n for n, m in sys.modules.items()
           if n.startswith("TorchProteinLibrary.") and m.__name__.startswith("TorchProteinLibrary")]
    assert not dup, dup

    for name in ("Angles2BackboneGPU_forward", "Angles2BackboneGPU_backward",
                 "Angles2BackboneCPU_forward", "Angles2BackboneCPU_backward", "angles2backbone_autograd"):
        assert hasattr(_ReducedModel, name), name
    # the C++ autograd functions the modules run
    assert hasattr(_FullAtomModel, "angles2coords_autograd") and hasattr(_RMSD, "coords2rmsd_autograd")
    for name in ("Angles2Coords_forward", "Angles2Coords_backward", "Angles2Coords_save", "getSeqNumAtoms",
                 "PDB2CoordsUnordered", "Coords2TypedCoords_forward", "Coords2TypedCoords_backward",
                 "CoordsTranslate_forward", "CoordsTranslateGPU_forward", "CoordsTranslate_backward",
                 "CoordsTranslateGPU_backward", "CoordsRotate_forward", "CoordsRotateGPU_forward",
                 "CoordsRotate_backward", "CoordsRotateGPU_backward", "Coords2Center_forward",
                 "Coords2CenterGPU_forward", "Coords2Center_backward", "Coords2CenterGPU_backward",
                 "getBBox", "getRandomRotation", "getRotation", "getRandomTranslation"):
        assert hasattr(_FullAtomModel, name), name

    # the names kept for import compatibility raise instead of computing on the CPU
    import torch
    try:
        Angles2BackboneCPUFunction.apply(torch.zeros(1, 3, 2, dtype=torch.double), torch.ones(1, dtype=torch.int))
    except RuntimeError as e:
        assert "no CPU path" in str(e)
    else:
        raise AssertionError("Angles2BackboneCPUFunction computed on the CPU")
    try:
        PDB2CoordsOrdered()(["x.pdb"])
    except NotImplementedError:
        pass
    else:
        raise AssertionError("PDB2CoordsOrdered returned")
    print("aliases ok")
""")


def test_reference_import_forms_resolve_to_this_package(built):
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "aliases ok" in r.stdout
