// _FullAtomModel extension module: the reference's Angles2Coords, CoordsTransform
// and Coords2TypedCoords entry points (Layers/FullAtomModel/main.cpp,
// Angles2Coords/angles2coords_interface.cpp, CoordsTransform/
// coordsTransformGPU_interface.cpp, Coords2TypedCoords/
// coords2typedcoords_interface.cpp) over the libtpl_gb300 C ABI.
//
// Differences from the reference, all deliberate:
//  * The compute runs on CUDA tensors (float32: batched kernels, float64: FP64
//    kernels); the reference runs on the CPU only.  A CPU `sequences` tensor is
//    copied to the angles' device; CPU angles raise.
//  * Unknown residue letters raise RuntimeError (the reference's getNumAtoms
//    throws, its tree builder silently skips them, nUtil.cpp:515-516 /
//    cConformation.cpp:60-121).
//  * res_names / atom_names may be empty tensors to skip writing them.
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/extension.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>
#include <map>
#include <mutex>
#include <string>

#include "../../../include/tpl_gb300.h"

namespace {

// Tuning knobs of the Angles2Coords kernels (threads_per_cta 0, 4, 8, 128, 256 or 512).
tpl_options g_a2c_opt = {};
bool g_a2c_tree_backward = false;  // float32 Angles2Coords_backward: rebuild the tree per joint

void check_status(int s, const char *what) {
    TORCH_CHECK(s == TPL_OK, what, ": ", tpl_status_string(s), " (", s, ")");
}

void *stream_of(const torch::Tensor &t) {
    return (void *)c10::cuda::getCurrentCUDAStream(t.device().index()).stream();
}

// One small status workspace per device (the reference entry points carry none).
torch::Tensor status_ws(const torch::Device &dev) {
    static std::mutex mu;
    static std::map<int, torch::Tensor> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(dev.index());
    if (it != cache.end()) return it->second;
    auto t = torch::zeros({(int64_t)tpl_a2c_workspace_bytes(0, 0, 0, nullptr)},
                          torch::TensorOptions().dtype(torch::kUInt8).device(dev));
    cache[dev.index()] = t;
    return t;
}

torch::Tensor seq_on(const torch::Tensor &sequences, const torch::Device &dev) {
    TORCH_CHECK(sequences.scalar_type() == torch::kByte, "sequences must be uint8");
    TORCH_CHECK(sequences.dim() == 2, "sequences must be [batch, max_len + 1]");
    auto s = sequences.is_cuda() ? sequences : sequences.to(dev, /*non_blocking=*/false);
    return s.contiguous();
}

void Angles2Coords_forward(torch::Tensor sequences, torch::Tensor input_angles, torch::Tensor output_coords,
                           torch::Tensor res_names, torch::Tensor atom_names) {
    TORCH_CHECK(input_angles.is_cuda(), "input_angles must be a CUDA tensor (this build has no CPU path)");
    TORCH_CHECK(input_angles.is_contiguous() && output_coords.is_contiguous(), "tensors must be contiguous");
    TORCH_CHECK(input_angles.dim() == 3 && input_angles.size(1) >= 8, "input_angles must be [batch, 8, max_len]");
    TORCH_CHECK(input_angles.size(1) == 8, "input_angles must have 8 rows (phi, psi, omega, chi1..chi5)");
    TORCH_CHECK(output_coords.is_cuda() && output_coords.scalar_type() == input_angles.scalar_type(),
                "output_coords must be a CUDA tensor of the angles' dtype");
    const at::cuda::CUDAGuard guard(input_angles.device());
    const int64_t B = input_angles.size(0), L = input_angles.size(2);
    TORCH_CHECK(output_coords.dim() == 2 && output_coords.size(0) == B && output_coords.size(1) % 3 == 0,
                "output_coords must be [batch, 3 * max_atoms]");
    const int64_t maxA = output_coords.size(1) / 3;
    auto seq = seq_on(sequences, input_angles.device());
    TORCH_CHECK(seq.size(0) == B, "one sequence per chain");
    uint8_t *rn = nullptr, *an = nullptr;
    if (res_names.numel() > 0 || atom_names.numel() > 0) {
        TORCH_CHECK(res_names.is_cuda() && atom_names.is_cuda(), "names must be CUDA tensors");
        TORCH_CHECK(res_names.scalar_type() == torch::kByte && atom_names.scalar_type() == torch::kByte,
                    "names must be uint8");
        TORCH_CHECK(res_names.numel() == B * maxA * 4 && atom_names.numel() == B * maxA * 4,
                    "names must be [batch, max_atoms, 4]");
        TORCH_CHECK(res_names.is_contiguous() && atom_names.is_contiguous(), "names must be contiguous");
        rn = res_names.data_ptr<uint8_t>();
        an = atom_names.data_ptr<uint8_t>();
    }
    auto ws = status_ws(input_angles.device());
    void *st = stream_of(input_angles);
    int s;
    if (input_angles.scalar_type() == torch::kFloat) {
        s = tpl_a2c_forward_f32(seq.data_ptr<uint8_t>(), (int)seq.size(1), input_angles.data_ptr<float>(),
                                output_coords.data_ptr<float>(), rn, an, ws.data_ptr(), ws.nbytes(), (int)B, (int)L,
                                (int)maxA, &g_a2c_opt, st);
    } else if (input_angles.scalar_type() == torch::kDouble) {
        s = tpl_a2c_forward_f64(seq.data_ptr<uint8_t>(), (int)seq.size(1), input_angles.data_ptr<double>(),
                                output_coords.data_ptr<double>(), rn, an, ws.data_ptr(), ws.nbytes(), (int)B, (int)L,
                                (int)maxA, &g_a2c_opt, st);
    } else {
        TORCH_CHECK(false, "input_angles must be float32 or float64");
    }
    check_status(s, "Angles2Coords_forward");
}

void Angles2Coords_backward(torch::Tensor grad_atoms, torch::Tensor grad_angles, torch::Tensor sequences,
                            torch::Tensor input_angles) {
    TORCH_CHECK(input_angles.is_cuda() && grad_atoms.is_cuda() && grad_angles.is_cuda(),
                "tensors must be CUDA tensors (this build has no CPU path)");
    TORCH_CHECK(input_angles.is_contiguous() && grad_atoms.is_contiguous() && grad_angles.is_contiguous(),
                "tensors must be contiguous");
    TORCH_CHECK(input_angles.dim() == 3 && input_angles.size(1) == 8, "input_angles must be [batch, 8, max_len]");
    TORCH_CHECK(grad_angles.sizes() == input_angles.sizes(), "grad_angles must have the angles' shape");
    TORCH_CHECK(grad_atoms.scalar_type() == input_angles.scalar_type() &&
                    grad_angles.scalar_type() == input_angles.scalar_type(),
                "gradient dtypes must match the angles");
    const at::cuda::CUDAGuard guard(input_angles.device());
    const int64_t B = input_angles.size(0), L = input_angles.size(2);
    TORCH_CHECK(grad_atoms.dim() == 2 && grad_atoms.size(0) == B && grad_atoms.size(1) % 3 == 0,
                "grad_atoms must be [batch, 3 * max_atoms]");
    const int64_t maxA = grad_atoms.size(1) / 3;
    auto seq = seq_on(sequences, input_angles.device());
    auto ws = status_ws(input_angles.device());
    void *st = stream_of(input_angles);
    int s;
    if (input_angles.scalar_type() == torch::kFloat && !g_a2c_tree_backward) {
        // the chunked forward into a temporary, then the backward from those coordinates:
        // 2.2x faster than rebuilding the tree per joint at 4096 x 500 residues
        auto coords = torch::empty({B, 3 * maxA}, input_angles.options());
        s = tpl_a2c_forward_f32(seq.data_ptr<uint8_t>(), (int)seq.size(1), input_angles.data_ptr<float>(),
                                coords.data_ptr<float>(), nullptr, nullptr, ws.data_ptr(), ws.nbytes(), (int)B, (int)L,
                                (int)maxA, &g_a2c_opt, st);
        if (s == TPL_OK)
            s = tpl_a2c_backward_coords_f32(grad_angles.data_ptr<float>(), grad_atoms.data_ptr<float>(),
                                            coords.data_ptr<float>(), seq.data_ptr<uint8_t>(), (int)seq.size(1),
                                            ws.data_ptr(), ws.nbytes(), (int)B, (int)L, (int)maxA, st);
    } else if (input_angles.scalar_type() == torch::kFloat) {
        s = tpl_a2c_backward_f32(grad_angles.data_ptr<float>(), grad_atoms.data_ptr<float>(), seq.data_ptr<uint8_t>(),
                                 (int)seq.size(1), input_angles.data_ptr<float>(), ws.data_ptr(), ws.nbytes(), (int)B,
                                 (int)L, (int)maxA, &g_a2c_opt, st);
    } else if (input_angles.scalar_type() == torch::kDouble) {
        s = tpl_a2c_backward_f64(grad_angles.data_ptr<double>(), grad_atoms.data_ptr<double>(),
                                 seq.data_ptr<uint8_t>(), (int)seq.size(1), input_angles.data_ptr<double>(),
                                 ws.data_ptr(), ws.nbytes(), (int)B, (int)L, (int)maxA, &g_a2c_opt, st);
    } else {
        TORCH_CHECK(false, "input_angles must be float32 or float64");
    }
    check_status(s, "Angles2Coords_backward");
}

// Backward of the float32 path from the forward's output coordinates (no tree
// rebuild).  Not a reference entry point: the Python layer calls it with the
// coordinates it saved; Angles2Coords_backward above keeps the reference's signature.
void Angles2Coords_backward_coords(torch::Tensor grad_atoms, torch::Tensor grad_angles, torch::Tensor sequences,
                                   torch::Tensor coords) {
    TORCH_CHECK(coords.is_cuda() && grad_atoms.is_cuda() && grad_angles.is_cuda(),
                "tensors must be CUDA tensors (this build has no CPU path)");
    TORCH_CHECK(coords.is_contiguous() && grad_atoms.is_contiguous() && grad_angles.is_contiguous(),
                "tensors must be contiguous");
    TORCH_CHECK(grad_angles.dim() == 3 && grad_angles.size(1) == 8, "grad_angles must be [batch, 8, max_len]");
    TORCH_CHECK(coords.scalar_type() == torch::kFloat && grad_atoms.scalar_type() == torch::kFloat &&
                    grad_angles.scalar_type() == torch::kFloat,
                "the coordinate backward is float32");
    const int64_t B = grad_angles.size(0), L = grad_angles.size(2);
    TORCH_CHECK(grad_atoms.dim() == 2 && grad_atoms.size(0) == B && grad_atoms.size(1) % 3 == 0 &&
                    coords.sizes() == grad_atoms.sizes(),
                "grad_atoms and coords must be [batch, 3 * max_atoms]");
    const int64_t maxA = grad_atoms.size(1) / 3;
    const at::cuda::CUDAGuard guard(coords.device());
    auto seq = seq_on(sequences, coords.device());
    auto ws = status_ws(coords.device());
    const int s = tpl_a2c_backward_coords_f32(grad_angles.data_ptr<float>(), grad_atoms.data_ptr<float>(),
                                              coords.data_ptr<float>(), seq.data_ptr<uint8_t>(), (int)seq.size(1),
                                              ws.data_ptr(), ws.nbytes(), (int)B, (int)L, (int)maxA,
                                              stream_of(coords));
    check_status(s, "Angles2Coords_backward_coords");
}

// The Angles2Coords autograd function in C++: the same forward and backward entries
// as the Python Angles2CoordsFunction, with the autograd engine calling the backward
// without a Python frame.  The float32 path saves its output coordinates and its
// backward reads every joint from them; float64 rebuilds the tree.
struct Angles2CoordsAutograd : public torch::autograd::Function<Angles2CoordsAutograd> {
    static torch::autograd::variable_list forward(torch::autograd::AutogradContext *ctx, torch::Tensor angles,
                                                  torch::Tensor sequences, int64_t max_atoms, bool names) {
        auto x = angles.contiguous();
        const int64_t B = x.size(0);
        auto coords = torch::empty({B, 3 * max_atoms}, x.options());
        auto byte = x.options().dtype(torch::kByte);
        auto rn = names ? torch::empty({B, max_atoms, 4}, byte) : torch::empty({0}, byte);
        auto an = names ? torch::empty({B, max_atoms, 4}, byte) : torch::empty({0}, byte);
        Angles2Coords_forward(sequences, x, coords, rn, an);
        const bool from_coords = x.scalar_type() == torch::kFloat;
        ctx->saved_data["from_coords"] = from_coords;
        ctx->save_for_backward({x, sequences, from_coords ? coords : torch::Tensor()});
        ctx->mark_non_differentiable({rn, an});
        // no zero-filled gradients for the name outputs (two fill kernels per call)
        ctx->set_materialize_grads(false);
        return {coords, rn, an};
    }
    static torch::autograd::variable_list backward(torch::autograd::AutogradContext *ctx,
                                                   torch::autograd::variable_list grads) {
        if (!grads[0].defined()) return {torch::Tensor(), torch::Tensor(), torch::Tensor(), torch::Tensor()};
        auto saved = ctx->get_saved_variables();
        auto g = grads[0].contiguous();
        auto grad_angles = torch::empty_like(saved[0]);
        if (ctx->saved_data["from_coords"].toBool())
            Angles2Coords_backward_coords(g, grad_angles, saved[1], saved[2]);
        else
            Angles2Coords_backward(g, grad_angles, saved[1], saved[0]);
        return {grad_angles, torch::Tensor(), torch::Tensor(), torch::Tensor()};
    }
};

std::vector<torch::Tensor> angles2coords_autograd(torch::Tensor angles, torch::Tensor sequences, int64_t max_atoms,
                                                  bool names) {
    TORCH_CHECK(angles.is_cuda(), "Angles2Coords: this build has no CPU path; move the angles to a CUDA device");
    return Angles2CoordsAutograd::apply(angles, sequences, max_atoms, names);
}

int64_t getSeqNumAtoms(const std::string &sequence) {
    int n = tpl_num_atoms(sequence.c_str());
    TORCH_CHECK(n >= 0, "Unknown atom/res names in sequence '", sequence, "'");
    return n;
}

// Angles2Coords_save (angles2coords_interface.cpp:117-137 -> cConformation::save,
// cConformation.cpp:228-262): PDB ATOM records of one chain, mode 'w' (overwrite)
// or 'a' (append as a MODEL).  The coordinates come from the GPU forward.
void Angles2Coords_save(const std::string &sequence, torch::Tensor input_angles, const std::string &output_filename,
                        const std::string &mode) {
    TORCH_CHECK(input_angles.dim() == 2 && input_angles.size(0) == 8, "input_angles must be [8, length]");
    TORCH_CHECK(mode == "w" || mode == "a", "mode must be 'w' or 'a'");
    const int64_t na = getSeqNumAtoms(sequence);
    torch::Device dev = input_angles.is_cuda() ? input_angles.device() : torch::Device(torch::kCUDA, 0);
    auto ang = input_angles.to(dev, torch::kDouble).contiguous().unsqueeze(0);
    auto opts = torch::TensorOptions().device(dev);
    auto coords = torch::empty({1, 3 * na}, opts.dtype(torch::kDouble));
    auto rn = torch::empty({1, na, 4}, opts.dtype(torch::kByte));
    auto an = torch::empty({1, na, 4}, opts.dtype(torch::kByte));
    std::vector<uint8_t> sbytes(sequence.begin(), sequence.end());
    sbytes.push_back(0);
    auto seq = torch::from_blob(sbytes.data(), {1, (int64_t)sbytes.size()}, torch::kByte).clone();
    Angles2Coords_forward(seq, ang, coords, rn, an);
    auto c = coords.cpu();
    auto r = rn.cpu();
    auto a = an.cpu();
    FILE *f = std::fopen(output_filename.c_str(), mode == "w" ? "w" : "a");
    TORCH_CHECK(f != nullptr, "cannot open ", output_filename);
    if (mode == "a") std::fprintf(f, "MODEL\n");
    const double *x = c.data_ptr<double>();
    const char *rnp = (const char *)r.data_ptr<uint8_t>();
    const char *anp = (const char *)a.data_ptr<uint8_t>();
    int res_index = -1, first_atom = 0;
    for (int64_t i = 0; i < na; i++) {
        std::string aname(anp + 4 * i, strnlen(anp + 4 * i, 4));
        std::string rname(rnp + 4 * i, strnlen(rnp + 4 * i, 4));
        if (aname == "N") {
            res_index++;
            first_atom = (int)i;
        }
        (void)first_atom;
        std::fprintf(f, "ATOM  %5d %4s %3s A%4d    %8.3f%8.3f%8.3f\n", (int)i, aname.c_str(), rname.c_str(),
                     res_index, x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    }
    if (mode == "a") std::fprintf(f, "ENDMDL\n");
    std::fclose(f);
}

int64_t workspace_status(int64_t device) {
    auto dev = torch::Device(torch::kCUDA, (int)device);
    const at::cuda::CUDAGuard guard(dev);
    auto ws = status_ws(dev);
    int st = 0;
    check_status(tpl_workspace_status(ws.data_ptr(), stream_of(ws), &st), "workspace_status");
    return st;
}

// ------------------------------------------------------------- CoordsTransform
// The reference's entry points (Layers/FullAtomModel/CoordsTransform/
// coordsTransformGPU_interface.cpp, coordsTransform_interface.cpp), CUDA tensors
// only; the CPU variants raise.  Coordinates [batch, 3 * atoms_stride], num_atoms
// int32 [batch] on the same device.
void check_coords(const torch::Tensor &x, const char *name) {
    TORCH_CHECK(x.is_cuda(), name, " must be a CUDA tensor (this build has no CPU path)");
    TORCH_CHECK(x.is_contiguous(), name, " must be contiguous");
    TORCH_CHECK(x.scalar_type() == torch::kFloat || x.scalar_type() == torch::kDouble, name,
                " must be float32 or float64");
}
void check_num_atoms(const torch::Tensor &na, const torch::Tensor &x) {
    TORCH_CHECK(na.is_cuda() && na.device() == x.device(), "num_atoms must be on the coordinates' device");
    TORCH_CHECK(na.scalar_type() == torch::kInt && na.is_contiguous() && na.numel() == x.size(0),
                "num_atoms must be contiguous int32 [batch]");
}
void check_same(const torch::Tensor &a, const torch::Tensor &b, const char *name) {
    TORCH_CHECK(a.is_cuda() && a.device() == b.device() && a.scalar_type() == b.scalar_type() && a.is_contiguous(),
                name, " must be a contiguous CUDA tensor of the coordinates' dtype and device");
}

void coords_translate(torch::Tensor in, torch::Tensor out, torch::Tensor T, torch::Tensor num_atoms, bool with_T,
                      const char *what) {
    check_coords(in, "input");
    TORCH_CHECK(in.dim() == 2 && in.size(1) % 3 == 0, what, ": coordinates must be [batch, 3 * atoms]");
    check_same(out, in, "output");
    TORCH_CHECK(out.sizes() == in.sizes(), what, ": output shape must match the input");
    check_num_atoms(num_atoms, in);
    if (with_T) {
        check_same(T, in, "T");
        TORCH_CHECK(T.numel() == in.size(0) * 3, what, ": T must be [batch, 3]");
    }
    const at::cuda::CUDAGuard guard(in.device());
    const int B = (int)in.size(0), S = (int)(in.size(1) / 3);
    int s;
    if (in.scalar_type() == torch::kFloat)
        s = tpl_coords_translate_f32(in.data_ptr<float>(), out.data_ptr<float>(), with_T ? T.data_ptr<float>() : nullptr,
                                     num_atoms.data_ptr<int32_t>(), B, S, stream_of(in));
    else
        s = tpl_coords_translate_f64(in.data_ptr<double>(), out.data_ptr<double>(),
                                     with_T ? T.data_ptr<double>() : nullptr, num_atoms.data_ptr<int32_t>(), B, S,
                                     stream_of(in));
    check_status(s, what);
}
void CoordsTranslateGPU_forward(torch::Tensor input_coords, torch::Tensor output_coords, torch::Tensor T,
                                torch::Tensor num_atoms) {
    coords_translate(input_coords, output_coords, T, num_atoms, true, "CoordsTranslateGPU_forward");
}
void CoordsTranslateGPU_backward(torch::Tensor grad_output_coords, torch::Tensor grad_input_coords, torch::Tensor T,
                                 torch::Tensor num_atoms) {
    coords_translate(grad_output_coords, grad_input_coords, T, num_atoms, false, "CoordsTranslateGPU_backward");
}

void coords_rotate(torch::Tensor in, torch::Tensor out, torch::Tensor R, torch::Tensor num_atoms, int transpose,
                   const char *what) {
    check_coords(in, "input");
    TORCH_CHECK(in.dim() == 2 && in.size(1) % 3 == 0, what, ": coordinates must be [batch, 3 * atoms]");
    check_same(out, in, "output");
    TORCH_CHECK(out.sizes() == in.sizes(), what, ": output shape must match the input");
    check_same(R, in, "R");
    TORCH_CHECK(R.numel() == in.size(0) * 9, what, ": R must be [batch, 3, 3]");
    check_num_atoms(num_atoms, in);
    const at::cuda::CUDAGuard guard(in.device());
    const int B = (int)in.size(0), S = (int)(in.size(1) / 3);
    int s;
    if (in.scalar_type() == torch::kFloat)
        s = tpl_coords_rotate_f32(in.data_ptr<float>(), out.data_ptr<float>(), R.data_ptr<float>(), transpose,
                                  num_atoms.data_ptr<int32_t>(), B, S, stream_of(in));
    else
        s = tpl_coords_rotate_f64(in.data_ptr<double>(), out.data_ptr<double>(), R.data_ptr<double>(), transpose,
                                  num_atoms.data_ptr<int32_t>(), B, S, stream_of(in));
    check_status(s, what);
}
void CoordsRotateGPU_forward(torch::Tensor input_coords, torch::Tensor output_coords, torch::Tensor R,
                             torch::Tensor num_atoms) {
    coords_rotate(input_coords, output_coords, R, num_atoms, 0, "CoordsRotateGPU_forward");
}
void CoordsRotateGPU_backward(torch::Tensor grad_output_coords, torch::Tensor grad_input_coords, torch::Tensor R,
                              torch::Tensor num_atoms) {
    coords_rotate(grad_output_coords, grad_input_coords, R, num_atoms, 1, "CoordsRotateGPU_backward");
}

void Coords2CenterGPU_forward(torch::Tensor input_coords, torch::Tensor output_T, torch::Tensor num_atoms) {
    check_coords(input_coords, "input_coords");
    TORCH_CHECK(input_coords.dim() == 2 && input_coords.size(1) % 3 == 0, "coordinates must be [batch, 3 * atoms]");
    check_same(output_T, input_coords, "output_T");
    TORCH_CHECK(output_T.numel() == input_coords.size(0) * 3, "output_T must be [batch, 3]");
    check_num_atoms(num_atoms, input_coords);
    const at::cuda::CUDAGuard guard(input_coords.device());
    const int B = (int)input_coords.size(0), S = (int)(input_coords.size(1) / 3);
    int s;
    if (input_coords.scalar_type() == torch::kFloat)
        s = tpl_coords_center_f32(input_coords.data_ptr<float>(), output_T.data_ptr<float>(),
                                  num_atoms.data_ptr<int32_t>(), B, S, stream_of(input_coords));
    else
        s = tpl_coords_center_f64(input_coords.data_ptr<double>(), output_T.data_ptr<double>(),
                                  num_atoms.data_ptr<int32_t>(), B, S, stream_of(input_coords));
    check_status(s, "Coords2CenterGPU_forward");
}
void Coords2CenterGPU_backward(torch::Tensor grad_output_T, torch::Tensor grad_input_coords,
                               torch::Tensor num_atoms) {
    check_coords(grad_input_coords, "grad_input_coords");
    TORCH_CHECK(grad_input_coords.dim() == 2 && grad_input_coords.size(1) % 3 == 0,
                "gradients must be [batch, 3 * atoms]");
    check_same(grad_output_T, grad_input_coords, "grad_output_T");
    TORCH_CHECK(grad_output_T.numel() == grad_input_coords.size(0) * 3, "grad_output_T must be [batch, 3]");
    check_num_atoms(num_atoms, grad_input_coords);
    const at::cuda::CUDAGuard guard(grad_input_coords.device());
    const int B = (int)grad_input_coords.size(0), S = (int)(grad_input_coords.size(1) / 3);
    int s;
    if (grad_input_coords.scalar_type() == torch::kFloat)
        s = tpl_coords_center_backward_f32(grad_output_T.data_ptr<float>(), grad_input_coords.data_ptr<float>(),
                                           num_atoms.data_ptr<int32_t>(), B, S, stream_of(grad_input_coords));
    else
        s = tpl_coords_center_backward_f64(grad_output_T.data_ptr<double>(), grad_input_coords.data_ptr<double>(),
                                           num_atoms.data_ptr<int32_t>(), B, S, stream_of(grad_input_coords));
    check_status(s, "Coords2CenterGPU_backward");
}

void getBBox(torch::Tensor input_coords, torch::Tensor a, torch::Tensor b, torch::Tensor num_atoms) {
    check_coords(input_coords, "input_coords");
    TORCH_CHECK(input_coords.dim() == 2 && input_coords.size(1) % 3 == 0, "coordinates must be [batch, 3 * atoms]");
    check_same(a, input_coords, "a");
    check_same(b, input_coords, "b");
    TORCH_CHECK(a.numel() == input_coords.size(0) * 3 && b.numel() == a.numel(), "a and b must be [batch, 3]");
    check_num_atoms(num_atoms, input_coords);
    const at::cuda::CUDAGuard guard(input_coords.device());
    const int B = (int)input_coords.size(0), S = (int)(input_coords.size(1) / 3);
    int s;
    if (input_coords.scalar_type() == torch::kFloat)
        s = tpl_coords_bbox_f32(input_coords.data_ptr<float>(), a.data_ptr<float>(), b.data_ptr<float>(),
                                num_atoms.data_ptr<int32_t>(), B, S, stream_of(input_coords));
    else
        s = tpl_coords_bbox_f64(input_coords.data_ptr<double>(), a.data_ptr<double>(), b.data_ptr<double>(),
                                num_atoms.data_ptr<int32_t>(), B, S, stream_of(input_coords));
    check_status(s, "getBBox");
}

// ------------------------------------------------------------ random poses
// Host helpers of the reference (coordsTransform_interface.cpp:201-259 over
// Math/nUtil.cpp:60-100), which fill small [B, 3, 3] / [B, 3] tensors for a
// training loop's data augmentation.  They are tensor arithmetic here, so they
// accept tensors on any device; the draws come from torch.rand (torch.manual_seed
// applies, as it does for the reference's draws).

// Rotation from u in [0, 1)^3 through the unit quaternion
// q = (sqrt(1-u1) sin 2 pi u2, sqrt(1-u1) cos 2 pi u2, sqrt(u1) sin 2 pi u3, sqrt(u1) cos 2 pi u3).
torch::Tensor rotation_from_uniform(const torch::Tensor &u) {
    const torch::Tensor ud = u.to(torch::kDouble);
    const double two_pi = 6.283185307179586;
    const torch::Tensor u1 = ud.select(1, 0), w2 = ud.select(1, 1) * two_pi, w3 = ud.select(1, 2) * two_pi;
    const torch::Tensor s1 = torch::sqrt(1.0 - u1), s2 = torch::sqrt(u1);
    const torch::Tensor q0 = s1 * torch::sin(w2), q1 = s1 * torch::cos(w2), q2 = s2 * torch::sin(w3),
                        q3 = s2 * torch::cos(w3);
    return torch::stack({q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3, 2.0 * (q1 * q2 - q0 * q3), 2.0 * (q1 * q3 + q0 * q2),
                         2.0 * (q1 * q2 + q0 * q3), q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3, 2.0 * (q2 * q3 - q0 * q1),
                         2.0 * (q1 * q3 - q0 * q2), 2.0 * (q2 * q3 + q0 * q1), q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3},
                        1)
        .view({-1, 3, 3});
}

void getRotation(torch::Tensor R, torch::Tensor u) {
    TORCH_CHECK(R.dim() == 3 && R.size(1) == 3 && R.size(2) == 3, "getRotation: R must be [batch, 3, 3]");
    TORCH_CHECK(u.dim() == 2 && u.size(0) == R.size(0) && u.size(1) >= 3, "getRotation: u must be [batch, 3]");
    R.copy_(rotation_from_uniform(u.to(R.device())));
}

void getRandomRotation(torch::Tensor R) {
    TORCH_CHECK(R.dim() == 3 && R.size(1) == 3 && R.size(2) == 3, "getRandomRotation: R must be [batch, 3, 3]");
    R.copy_(rotation_from_uniform(torch::rand({R.size(0), 3}, R.options().dtype(torch::kDouble))));
}

// T_k ~ U[-d_k, d_k], d_k = max(0, volume_size / 2 - (b_k - a_k) / 2) / 2: the box [a, b]
// stays inside a cube of side volume_size centred on the origin.
void getRandomTranslation(torch::Tensor T, torch::Tensor a, torch::Tensor b, double volume_size) {
    TORCH_CHECK(T.dim() == 2 && T.size(1) == 3, "getRandomTranslation: T must be [batch, 3]");
    TORCH_CHECK(a.sizes() == T.sizes() && b.sizes() == T.sizes(), "getRandomTranslation: a and b must be [batch, 3]");
    const torch::Tensor ad = a.to(T.device(), torch::kDouble), bd = b.to(T.device(), torch::kDouble);
    const torch::Tensor d = torch::clamp_min(volume_size / 2.0 - (bd - ad) / 2.0, 0.0) * 0.5;
    T.copy_(torch::rand(T.sizes(), T.options().dtype(torch::kDouble)) * (2.0 * d) - d);
}

// ---------------------------------------------------------- Coords2TypedCoords
// Reference entry points (Layers/FullAtomModel/Coords2TypedCoords/
// coords2typedcoords_interface.cpp), on CUDA tensors.  Typed rows hold
// output_coords.size(1) / 3 slots (the reference sizes them by max(num_atoms)).
void Coords2TypedCoords_forward(torch::Tensor input_coords, torch::Tensor res_names, torch::Tensor atom_names,
                                torch::Tensor num_atoms, torch::Tensor output_coords, torch::Tensor num_atoms_of_type,
                                torch::Tensor offsets, torch::Tensor atom_indexes) {
    check_coords(input_coords, "input_coords");
    TORCH_CHECK(input_coords.dim() == 2 && input_coords.size(1) % 3 == 0, "coordinates must be [batch, 3 * atoms]");
    const int64_t B = input_coords.size(0), S_in = input_coords.size(1) / 3;
    for (auto *t : {&res_names, &atom_names}) {
        TORCH_CHECK(t->is_cuda() && t->device() == input_coords.device() && t->scalar_type() == torch::kByte &&
                        t->is_contiguous() && t->numel() == B * S_in * 4,
                    "res_names / atom_names must be contiguous uint8 [batch, atoms, 4] on the coordinates' device");
    }
    check_num_atoms(num_atoms, input_coords);
    check_same(output_coords, input_coords, "output_coords");
    TORCH_CHECK(output_coords.dim() == 2 && output_coords.size(0) == B && output_coords.size(1) % 3 == 0,
                "output_coords must be [batch, 3 * max_atoms]");
    const int64_t S_out = output_coords.size(1) / 3;
    for (auto *t : {&num_atoms_of_type, &offsets})
        TORCH_CHECK(t->is_cuda() && t->scalar_type() == torch::kInt && t->is_contiguous() && t->numel() == B * 11,
                    "num_atoms_of_type / offsets must be contiguous int32 [batch, 11] on the device");
    TORCH_CHECK(atom_indexes.is_cuda() && atom_indexes.scalar_type() == torch::kInt && atom_indexes.is_contiguous() &&
                    atom_indexes.numel() == B * S_out,
                "atom_indexes must be contiguous int32 [batch, max_atoms] on the device");
    const at::cuda::CUDAGuard guard(input_coords.device());
    auto ws = status_ws(input_coords.device());
    const bool f64 = input_coords.scalar_type() == torch::kDouble;
    int s;
    if (f64)
        s = tpl_typed_coords_forward_f64(input_coords.data_ptr<double>(), res_names.data_ptr<uint8_t>(),
                                         atom_names.data_ptr<uint8_t>(), num_atoms.data_ptr<int32_t>(), (int)B,
                                         (int)S_in, (int)S_out, output_coords.data_ptr<double>(),
                                         num_atoms_of_type.data_ptr<int32_t>(), offsets.data_ptr<int32_t>(),
                                         atom_indexes.data_ptr<int32_t>(), ws.data_ptr(), ws.nbytes(),
                                         stream_of(input_coords));
    else
        s = tpl_typed_coords_forward_f32(input_coords.data_ptr<float>(), res_names.data_ptr<uint8_t>(),
                                         atom_names.data_ptr<uint8_t>(), num_atoms.data_ptr<int32_t>(), (int)B,
                                         (int)S_in, (int)S_out, output_coords.data_ptr<float>(),
                                         num_atoms_of_type.data_ptr<int32_t>(), offsets.data_ptr<int32_t>(),
                                         atom_indexes.data_ptr<int32_t>(), ws.data_ptr(), ws.nbytes(),
                                         stream_of(input_coords));
    check_status(s, "Coords2TypedCoords_forward");
}

void Coords2TypedCoords_backward(torch::Tensor grad_typed_coords, torch::Tensor grad_flat_coords,
                                 torch::Tensor num_atoms_of_type, torch::Tensor offsets, torch::Tensor atom_indexes) {
    (void)offsets;  // the typed slots are addressed through atom_indexes
    check_coords(grad_typed_coords, "grad_typed_coords");
    check_same(grad_flat_coords, grad_typed_coords, "grad_flat_coords");
    TORCH_CHECK(grad_typed_coords.dim() == 2 && grad_flat_coords.dim() == 2 &&
                    grad_typed_coords.size(0) == grad_flat_coords.size(0) && grad_typed_coords.size(1) % 3 == 0 &&
                    grad_flat_coords.size(1) % 3 == 0,
                "gradients must be [batch, 3 * atoms]");
    const int64_t B = grad_typed_coords.size(0), S_out = grad_typed_coords.size(1) / 3,
                  S_in = grad_flat_coords.size(1) / 3;
    TORCH_CHECK(num_atoms_of_type.is_cuda() && num_atoms_of_type.scalar_type() == torch::kInt &&
                    num_atoms_of_type.is_contiguous() && num_atoms_of_type.numel() == B * 11,
                "num_atoms_of_type must be contiguous int32 [batch, 11] on the device");
    TORCH_CHECK(atom_indexes.is_cuda() && atom_indexes.scalar_type() == torch::kInt && atom_indexes.is_contiguous() &&
                    atom_indexes.numel() == B * S_out,
                "atom_indexes must be contiguous int32 [batch, max_atoms] on the device");
    const at::cuda::CUDAGuard guard(grad_typed_coords.device());
    int s;
    if (grad_typed_coords.scalar_type() == torch::kDouble)
        s = tpl_typed_coords_backward_f64(grad_typed_coords.data_ptr<double>(), grad_flat_coords.data_ptr<double>(),
                                          num_atoms_of_type.data_ptr<int32_t>(), atom_indexes.data_ptr<int32_t>(),
                                          (int)B, (int)S_in, (int)S_out, stream_of(grad_typed_coords));
    else
        s = tpl_typed_coords_backward_f32(grad_typed_coords.data_ptr<float>(), grad_flat_coords.data_ptr<float>(),
                                          num_atoms_of_type.data_ptr<int32_t>(), atom_indexes.data_ptr<int32_t>(),
                                          (int)B, (int)S_in, (int)S_out, stream_of(grad_typed_coords));
    check_status(s, "Coords2TypedCoords_backward");
}

// ------------------------------------------------------------------ PDB reading
// PDB2CoordsUnordered (Layers/FullAtomModel/PDB2Coords/pdb2coords_interface.cpp:
// 75-127): host tensors, resized in place to the largest file's atom count, as the
// reference does.  The parsing is the C ABI's tpl_pdb_read_batch (host threads).
void PDB2CoordsUnordered(torch::Tensor filenames, torch::Tensor coords, torch::Tensor chain_names,
                         torch::Tensor res_names, torch::Tensor res_nums, torch::Tensor atom_names,
                         torch::Tensor num_atoms) {
    TORCH_CHECK(!filenames.is_cuda() && filenames.scalar_type() == torch::kByte && filenames.dim() == 2,
                "filenames must be a CPU uint8 [batch, max_len] tensor of NUL-terminated paths");
    TORCH_CHECK(!coords.is_cuda() && coords.scalar_type() == torch::kDouble, "coords must be a CPU float64 tensor");
    for (auto *t : {&chain_names, &res_names, &atom_names})
        TORCH_CHECK(!t->is_cuda() && t->scalar_type() == torch::kByte, "names must be CPU uint8 tensors");
    TORCH_CHECK(!res_nums.is_cuda() && res_nums.scalar_type() == torch::kInt, "res_nums must be a CPU int32 tensor");
    TORCH_CHECK(!num_atoms.is_cuda() && num_atoms.scalar_type() == torch::kInt && num_atoms.is_contiguous(),
                "num_atoms must be a contiguous CPU int32 tensor");
    const int64_t B = filenames.size(0);
    TORCH_CHECK(num_atoms.numel() == B, "num_atoms must hold one count per file");
    auto fn = filenames.contiguous();
    std::vector<std::string> names(B);
    std::vector<const char *> ptrs(B);
    int32_t max_atoms = 0;
    for (int64_t b = 0; b < B; b++) {
        const char *row = reinterpret_cast<const char *>(fn.data_ptr<uint8_t>()) + b * fn.size(1);
        names[b] = std::string(row, strnlen(row, (size_t)fn.size(1)));
        ptrs[b] = names[b].c_str();
        int32_t n = 0;
        check_status(tpl_pdb_count_atoms(ptrs[b], &n), ("PDB2CoordsUnordered: " + names[b]).c_str());
        max_atoms = std::max(max_atoms, n);
    }
    coords.resize_({B, 3 * (int64_t)max_atoms});
    chain_names.resize_({B, max_atoms, 4});
    res_names.resize_({B, max_atoms, 4});
    res_nums.resize_({B, max_atoms});
    atom_names.resize_({B, max_atoms, 4});
    const int s = tpl_pdb_read_batch(ptrs.data(), (int)B, max_atoms, coords.data_ptr<double>(),
                                     chain_names.data_ptr<uint8_t>(), res_names.data_ptr<uint8_t>(),
                                     res_nums.data_ptr<int32_t>(), atom_names.data_ptr<uint8_t>(),
                                     num_atoms.data_ptr<int32_t>(), 0);
    check_status(s, "PDB2CoordsUnordered");
}

void no_cpu_transform(torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor) {
    TORCH_CHECK(false, "CoordsTransform: this build has no CPU path; move the tensors to a CUDA device");
}
void no_cpu_center(torch::Tensor, torch::Tensor, torch::Tensor) {
    TORCH_CHECK(false, "Coords2Center: this build has no CPU path; move the tensors to a CUDA device");
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("CoordsTranslateGPU_forward", &CoordsTranslateGPU_forward, "CoordsTranslate gpu forward");
    m.def("CoordsTranslateGPU_backward", &CoordsTranslateGPU_backward, "CoordsTranslate gpu backward");
    m.def("CoordsRotateGPU_forward", &CoordsRotateGPU_forward, "CoordsRotate gpu forward");
    m.def("CoordsRotateGPU_backward", &CoordsRotateGPU_backward, "CoordsRotate gpu backward");
    m.def("Coords2CenterGPU_forward", &Coords2CenterGPU_forward, "Coords2Center gpu forward");
    m.def("Coords2CenterGPU_backward", &Coords2CenterGPU_backward, "Coords2Center gpu backward");
    m.def("CoordsTranslate_forward", &no_cpu_transform, "not available: no CPU path");
    m.def("CoordsTranslate_backward", &no_cpu_transform, "not available: no CPU path");
    m.def("CoordsRotate_forward", &no_cpu_transform, "not available: no CPU path");
    m.def("CoordsRotate_backward", &no_cpu_transform, "not available: no CPU path");
    m.def("Coords2Center_forward", &no_cpu_center, "not available: no CPU path");
    m.def("Coords2Center_backward", &no_cpu_center, "not available: no CPU path");
    m.def("getBBox", &getBBox, "per-chain bounding box (GPU)");
    m.def("getRotation", &getRotation, "rotation matrices from uniform parameters");
    m.def("getRandomRotation", &getRandomRotation, "uniformly random rotations");
    m.def("getRandomTranslation", &getRandomTranslation, "random translation keeping a box inside a cube");
    m.def("PDB2CoordsUnordered", &PDB2CoordsUnordered, "Convert PDB to coordinates in the PDB order");
    m.def(
        "set_options",
        [](int64_t threads_per_cta) {
            TORCH_CHECK(threads_per_cta == 0 || threads_per_cta == 4 || threads_per_cta == 8 ||
                            threads_per_cta == 128 || threads_per_cta == 256 || threads_per_cta == 512,
                        "threads_per_cta of Angles2Coords must be 0, 4, 8, 128, 256 or 512");
            g_a2c_opt.threads_per_cta = (int)threads_per_cta;
        },
        "Angles2Coords float32 forward: threads per chain (0 = 256; 256 or 512 = 1 residue each; 128 = 2 each; "
        "4 or 8 = four or eight warps per chain, chunks of 32 residues)",
        py::arg("threads_per_cta") = 0);
    m.def("get_options", []() { return (int64_t)g_a2c_opt.threads_per_cta; }, "Angles2Coords threads per chain");
    m.def(
        "set_backward_tree", [](bool tree) { g_a2c_tree_backward = tree; },
        "float32 Angles2Coords_backward: false (default) = forward into a temporary, then the backward from "
        "those coordinates; true = rebuild the tree per joint (tpl_a2c_backward_f32)",
        py::arg("tree") = false);
    m.def("Coords2TypedCoords_forward", &Coords2TypedCoords_forward, "Coords2TypedCoords forward (GPU)");
    m.def("Coords2TypedCoords_backward", &Coords2TypedCoords_backward, "Coords2TypedCoords backward (GPU)");
    m.def("Angles2Coords_forward", &Angles2Coords_forward, "Angles2Coords forward");
    m.def("Angles2Coords_backward", &Angles2Coords_backward, "Angles2Coords backward");
    m.def("Angles2Coords_backward_coords", &Angles2Coords_backward_coords,
          "float32 Angles2Coords backward from the forward's output coordinates");
    m.def("Angles2Coords_save", &Angles2Coords_save, "Angles2Coords save");
    m.def("getSeqNumAtoms", &getSeqNumAtoms, "Get number of atoms in a sequence");
    m.def("angles2coords_autograd", &angles2coords_autograd,
          "Angles2Coords forward as a C++ autograd function: (coords, res_names, atom_names)");
    m.def("workspace_status", &workspace_status, "synchronise and read the first device-detected error");
}
