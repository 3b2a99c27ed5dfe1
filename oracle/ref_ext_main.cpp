// Python bindings of the reference's own CPU interfaces for CoordsTransform,
// Coords2TypedCoords and Coords2RMSD, compiled unmodified from the reference's
// sources by oracle/build_ref_ext.py (with ref_shim_torch/nUtil.h).  Test
// infrastructure only: tests/golden/make_golden.py calls them to write the golden
// fixtures that pin the oracle's numpy restatements.  Entry names follow the
// reference's Layers/FullAtomModel/main.cpp and Layers/RMSD/main.cpp.
#include <torch/extension.h>

#include <stdexcept>

#include "Coords2RMSD/coords2rmsd_interface.h"
#include "Coords2TypedCoords/coords2typedcoords_interface.h"
#include "CoordsTransform/coordsTransform_interface.h"
#include "RMSDKernels.h"

// coords2rmsd_interface.cpp also holds the GPU forward, which calls these CUDA
// launchers; the CPU-only oracle build links these stand-ins, which refuse to run.
template <typename T>
void gpu_correlationMatrix(T *, T *, double *, int *, int, int) {
    throw std::runtime_error("the oracle's reference build has no GPU path");
}
template <typename T>
void gpu_computeR2(T *, int, double *) {
    throw std::runtime_error("the oracle's reference build has no GPU path");
}
template void gpu_correlationMatrix<float>(float *, float *, double *, int *, int, int);
template void gpu_correlationMatrix<double>(double *, double *, double *, int *, int, int);
template void gpu_computeR2<float>(float *, int, double *);
template void gpu_computeR2<double>(double *, int, double *);

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("CoordsTranslate_forward", &CoordsTranslate_forward);
    m.def("CoordsTranslate_backward", &CoordsTranslate_backward);
    m.def("CoordsRotate_forward", &CoordsRotate_forward);
    m.def("CoordsRotate_backward", &CoordsRotate_backward);
    m.def("Coords2Center_forward", &Coords2Center_forward);
    m.def("Coords2Center_backward", &Coords2Center_backward);
    m.def("getBBox", &getBBox);
    m.def("getRotation", &getRotation);
    m.def("Coords2TypedCoords_forward", &Coords2TypedCoords_forward);
    m.def("Coords2TypedCoords_backward", &Coords2TypedCoords_backward);
    m.def("Coords2RMSD_forward", &Coords2RMSD_forward);
}
