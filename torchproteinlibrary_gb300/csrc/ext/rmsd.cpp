// _RMSD extension module: the reference's Coords2RMSD entry points
// (Layers/RMSD/main.cpp, Layers/RMSD/Coords2RMSD/coords2rmsd_interface.cpp) over the
// libtpl_gb300 C ABI, plus a backward entry and a fused-centring variant.
// CUDA tensors only; the CPU entry point raises.
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/extension.h>

#include "../../../include/tpl_gb300.h"

namespace {

void check_status(int s, const char *what) {
    TORCH_CHECK(s == TPL_OK, what, ": ", tpl_status_string(s), " (", s, ")");
}

void *stream_of(const torch::Tensor &t) {
    return (void *)c10::cuda::getCurrentCUDAStream(t.device().index()).stream();
}

void check(const torch::Tensor &src, const torch::Tensor &dst, const torch::Tensor &num_atoms) {
    TORCH_CHECK(src.is_cuda() && dst.is_cuda() && num_atoms.is_cuda(), "tensors must be CUDA tensors");
    TORCH_CHECK(src.is_contiguous() && dst.is_contiguous() && num_atoms.is_contiguous(), "tensors must be contiguous");
    TORCH_CHECK(src.dim() == 2 && src.sizes() == dst.sizes() && src.size(1) % 3 == 0,
                "coordinates must be [batch, 3 * atoms]");
    TORCH_CHECK(num_atoms.scalar_type() == torch::kInt && num_atoms.numel() == src.size(0),
                "num_atoms must be int32 [batch]");
    TORCH_CHECK(src.scalar_type() == dst.scalar_type(), "dtypes must match");
}

void forward_impl(torch::Tensor src, torch::Tensor dst, torch::Tensor output, torch::Tensor num_atoms,
                  torch::Tensor UT, torch::Tensor centroids, int center) {
    check(src, dst, num_atoms);
    const at::cuda::CUDAGuard guard(src.device());
    const int B = (int)src.size(0), stride = (int)(src.size(1) / 3);
    TORCH_CHECK(output.numel() == B && UT.numel() == 9 * B && output.is_cuda() && UT.is_cuda(),
                "output [batch] and UT [batch, 3, 3] must be CUDA tensors");
    TORCH_CHECK(output.scalar_type() == src.scalar_type() && UT.scalar_type() == src.scalar_type(),
                "output and UT dtypes must match the coordinates");
    double *cent = nullptr;
    if (center) {
        TORCH_CHECK(centroids.is_cuda() && centroids.scalar_type() == torch::kDouble && centroids.numel() == 6 * B,
                    "centroids must be CUDA float64 [batch, 6]");
        cent = centroids.data_ptr<double>();
    }
    int s;
    if (src.scalar_type() == torch::kFloat)
        s = tpl_rmsd_forward_f32(src.data_ptr<float>(), dst.data_ptr<float>(), num_atoms.data_ptr<int32_t>(), B,
                                 stride, center, output.data_ptr<float>(), UT.data_ptr<float>(), cent, nullptr, 0,
                                 stream_of(src));
    else if (src.scalar_type() == torch::kDouble)
        s = tpl_rmsd_forward_f64(src.data_ptr<double>(), dst.data_ptr<double>(), num_atoms.data_ptr<int32_t>(), B,
                                 stride, center, output.data_ptr<double>(), UT.data_ptr<double>(), cent, nullptr, 0,
                                 stream_of(src));
    else
        TORCH_CHECK(false, "coordinates must be float32 or float64");
    check_status(s, "Coords2RMSD forward");
}

void Coords2RMSDGPU_forward(torch::Tensor centered_src, torch::Tensor centered_dst, torch::Tensor output,
                            torch::Tensor num_atoms, torch::Tensor UT) {
    forward_impl(centered_src, centered_dst, output, num_atoms, UT, torch::Tensor(), 0);
}

void Coords2RMSDGPU_forward_centering(torch::Tensor src, torch::Tensor dst, torch::Tensor output,
                                      torch::Tensor num_atoms, torch::Tensor UT, torch::Tensor centroids) {
    forward_impl(src, dst, output, num_atoms, UT, centroids, 1);
}

void Coords2RMSDGPU_backward(torch::Tensor grad_rmsd, torch::Tensor src, torch::Tensor dst, torch::Tensor num_atoms,
                             torch::Tensor output, torch::Tensor UT, torch::Tensor centroids, torch::Tensor grad_src,
                             int64_t center) {
    check(src, dst, num_atoms);
    const at::cuda::CUDAGuard guard(src.device());
    const int B = (int)src.size(0), stride = (int)(src.size(1) / 3);
    TORCH_CHECK(grad_src.sizes() == src.sizes() && grad_src.scalar_type() == src.scalar_type() && grad_src.is_cuda(),
                "grad_src must match the coordinates");
    auto g = grad_rmsd.contiguous();
    const double *cent = center ? centroids.data_ptr<double>() : nullptr;
    int s;
    if (src.scalar_type() == torch::kFloat)
        s = tpl_rmsd_backward_f32(g.data_ptr<float>(), src.data_ptr<float>(), dst.data_ptr<float>(),
                                  num_atoms.data_ptr<int32_t>(), output.data_ptr<float>(), UT.data_ptr<float>(), cent,
                                  B, stride, (int)center, grad_src.data_ptr<float>(), stream_of(src));
    else
        s = tpl_rmsd_backward_f64(g.data_ptr<double>(), src.data_ptr<double>(), dst.data_ptr<double>(),
                                  num_atoms.data_ptr<int32_t>(), output.data_ptr<double>(), UT.data_ptr<double>(),
                                  cent, B, stride, (int)center, grad_src.data_ptr<double>(), stream_of(src));
    check_status(s, "Coords2RMSD backward");
}

// Coords2RMSD with the centring folded in, as a C++ autograd function (the same
// entries as the Python _Coords2RMSDCentering, without a Python frame in the
// backward).  num_atoms: int32 on the coordinates' device.
struct Coords2RMSDAutograd : public torch::autograd::Function<Coords2RMSDAutograd> {
    static torch::autograd::variable_list forward(torch::autograd::AutogradContext *ctx, torch::Tensor input,
                                                  torch::Tensor target, torch::Tensor num_atoms) {
        auto x = input.contiguous(), y = target.contiguous();
        const int64_t B = x.size(0);
        auto output = torch::empty({B}, x.options());
        auto UT = torch::empty({B, 3, 3}, x.options());
        auto cent = torch::empty({B, 6}, x.options().dtype(torch::kDouble));
        forward_impl(x, y, output, num_atoms, UT, cent, 1);
        ctx->save_for_backward({output, num_atoms, UT, x, y, cent});
        ctx->mark_non_differentiable({UT});
        // no zero-filled gradient for the unused UT output (one fill kernel per call)
        ctx->set_materialize_grads(false);
        return {output, UT};
    }
    static torch::autograd::variable_list backward(torch::autograd::AutogradContext *ctx,
                                                   torch::autograd::variable_list grads) {
        if (!grads[0].defined()) return {torch::Tensor(), torch::Tensor(), torch::Tensor()};
        auto s = ctx->get_saved_variables();
        auto grad = torch::empty_like(s[3]);
        Coords2RMSDGPU_backward(grads[0], s[3], s[4], s[1], s[0], s[2], s[5], grad, 1);
        return {grad, torch::Tensor(), torch::Tensor()};
    }
};

std::vector<torch::Tensor> coords2rmsd_autograd(torch::Tensor input, torch::Tensor target, torch::Tensor num_atoms) {
    TORCH_CHECK(input.is_cuda(), "Coords2RMSD: this build has no CPU path; move the tensors to a CUDA device");
    return Coords2RMSDAutograd::apply(input, target, num_atoms);
}

void no_cpu_path(torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor) {
    TORCH_CHECK(false, "Coords2RMSD: this build has no CPU path; move the tensors to a CUDA device");
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("Coords2RMSDGPU_forward", &Coords2RMSDGPU_forward, "Coords2RMSD gpu forward (centred inputs)");
    m.def("Coords2RMSD_forward", &no_cpu_path, "not available: no CPU path");
    m.def("Coords2RMSDGPU_forward_centering", &Coords2RMSDGPU_forward_centering,
          "Coords2RMSD gpu forward with the centring folded in");
    m.def("Coords2RMSDGPU_backward", &Coords2RMSDGPU_backward, "Coords2RMSD gpu backward");
    m.def("coords2rmsd_autograd", &coords2rmsd_autograd,
          "Coords2RMSD with centring as a C++ autograd function: (rmsd, UT)");
}
