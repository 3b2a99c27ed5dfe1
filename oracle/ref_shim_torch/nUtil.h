// Stand-in for the reference's Math/nUtil.h when its torch interfaces
// (CoordsTransform, Coords2TypedCoords, Coords2RMSD CPU paths) are compiled
// unmodified against the torch of this machine.  Test infrastructure only
// (oracle/build_ref_ext.py); nothing in the product includes it.
//
// It declares the same helpers as Math/nUtil.h (their definitions come from the
// reference's own Math/nUtil.cpp) and bridges three things that torch 2.x
// removed or changed:
//   1. AT_DISPATCH_* on `x.type()`: an overload of ::detail::scalar_type for the
//      deprecated type object, so the dispatch macros accept it again;
//   2. the device checks use x.is_cuda() (Math/nUtil.h:49,55 go through
//      x.type().is_cuda());
//   3. Tensor::eig (coords2rmsd_interface.cpp:14), removed from torch: the member
//      call `m.eig(true)` is rewritten by a macro into a call of eig_request()
//      below, which returns the old (eigenvalues [n, 2] real / imaginary,
//      eigenvectors as columns [n, n]) pair from at::linalg_eigh.  The 4x4
//      matrix it is used on is symmetric, so the eigenvalues are real.
#ifndef NUTIL_H_
#define NUTIL_H_
#include <torch/extension.h>

#include <algorithm>
#include <memory>
#include <string>
#include <tuple>

#include <cMatrix33.h>
#include <cVector3.h>

namespace detail {
inline at::ScalarType scalar_type(const at::DeprecatedTypeProperties &t) { return t.scalarType(); }
}  // namespace detail

namespace tpl_ref_shim {
struct EigRequest {};
inline std::tuple<at::Tensor, at::Tensor> operator|(const at::Tensor &m, EigRequest) {
    auto vals_vecs = at::linalg_eigh(m.to(at::kDouble));
    at::Tensor vals = std::get<0>(vals_vecs);
    at::Tensor pairs = at::stack({vals, at::zeros_like(vals)}, 1);
    return std::make_tuple(pairs, std::get<1>(vals_vecs));
}
}  // namespace tpl_ref_shim
#define eig(eigenvectors) alias() | tpl_ref_shim::EigRequest {}

namespace StringUtil {
std::string trim(const std::string &s);
std::string string_format(const std::string fmt, ...);
torch::Tensor string2Tensor(std::string s);
void string2Tensor(std::string s, torch::Tensor T);
std::string tensor2String(torch::Tensor T);
}  // namespace StringUtil

namespace ProtUtil {
uint getAtomIndex(std::string &res_name, std::string &atom_name);
uint getNumAtoms(std::string &sequence, bool add_terminal);
bool isHeavyAtom(std::string &atom_name);
std::string convertRes1to3(char resName);
uint get11AtomType(std::string res_name, std::string atom_name, bool terminal);
}  // namespace ProtUtil

template <typename T>
void rotate(torch::Tensor &input_coords, cMatrix33<T> &R, torch::Tensor &output_coords, int num_atoms);
template <typename T>
void translate(torch::Tensor &input_coords, cVector3<T> &Tr, torch::Tensor &output_coords, int num_atoms);
template <typename T>
void computeBoundingBox(torch::Tensor &input_coords, int num_atoms, cVector3<T> &b0, cVector3<T> &b1);
template <typename T>
cMatrix33<T> getRotation(T u1, T u2, T u3);
template <typename T>
cMatrix33<T> getRandomRotation();
template <typename T>
cVector3<T> getRandomTranslation(float spatial_dim, cVector3<T> &b0, cVector3<T> &b1);
template <typename T>
cMatrix33<T> tensor2Matrix33(torch::Tensor Ten);
template <typename T>
void matrix2Tensor(cMatrix33<T> &mat, torch::Tensor &Ten);

#define ERROR(x) AT_ASSERTM(true, #x)
#define CHECK_CPU(x) AT_ASSERTM(!(x).is_cuda(), #x " must be a CPU tensor")
#define CHECK_CONTIGUOUS(x) AT_ASSERTM((x).is_contiguous(), #x " must be contiguous")
#define CHECK_TYPE(x, y) AT_ASSERTM((x).dtype() == y, #x " wrong tensor type")
#define CHECK_CPU_INPUT(x) \
    CHECK_CPU(x);          \
    CHECK_CONTIGUOUS(x)
#define CHECK_CPU_INPUT_TYPE(x, y) \
    CHECK_CPU(x);                  \
    CHECK_CONTIGUOUS(x);           \
    CHECK_TYPE(x, y)
#define CHECK_GPU(x) AT_ASSERTM((x).is_cuda(), #x " must be a GPU tensor")
#define CHECK_GPU_INPUT(x) \
    CHECK_GPU(x);          \
    CHECK_CONTIGUOUS(x)
#define CHECK_GPU_INPUT_TYPE(x, y) \
    CHECK_GPU(x);                  \
    CHECK_CONTIGUOUS(x);           \
    CHECK_TYPE(x, y)

#endif
