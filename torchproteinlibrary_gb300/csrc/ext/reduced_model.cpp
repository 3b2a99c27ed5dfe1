// _ReducedModel extension module: the reference's entry points
// (Layers/ReducedModel/main.cpp:4-9, Layers/ReducedModel/Angles2Backbone/
// angles2backbone_interface.cpp) over the libtpl_gb300 C ABI.
//
// Differences from the reference, all deliberate:
//  * CUDA tensors of float32 run the batched FP32 kernels, float64 the plain FP64
//    form; the CPU entry points raise (this build has no CPU path).
//  * `A` is the caller-owned workspace (any dtype, at least
//    workspace_bytes(batch, max_len) bytes, zeroed before its first use).  It
//    carries per-tile transforms from the forward to the backward.
//  * `dr_dangle` is accepted and ignored: the adjoint forms no Jacobian.
//  * Errors raise RuntimeError instead of passing silently (the reference's
//    ERROR() is a no-op, Math/nUtil.h:48).
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/extension.h>

#include "../../../include/tpl_gb300.h"

namespace {

tpl_options g_opt = {0, 0, 0, 0, 0};

void check_status(int s, const char *what) {
    TORCH_CHECK(s == TPL_OK, what, ": ", tpl_status_string(s), " (", s, ")");
}

void check_cuda(const torch::Tensor &t, const char *name) {
    TORCH_CHECK(t.is_cuda(), name, " must be a CUDA tensor (this build has no CPU path)");
    TORCH_CHECK(t.is_contiguous(), name, " must be contiguous");
}

void *stream_of(const torch::Tensor &t) {
    return (void *)c10::cuda::getCurrentCUDAStream(t.device().index()).stream();
}

// The options of one call: the module-wide ones (set_options), with the scheme and
// residues per thread replaced where the caller passes them (>= 0), as the layer
// does with the autotuner's choice for the batch's shape.
tpl_options call_options(int64_t residues_per_thread, int64_t threads_per_cta) {
    tpl_options o = g_opt;
    if (residues_per_thread >= 0) o.residues_per_thread = (int)residues_per_thread;
    if (threads_per_cta >= 0) o.threads_per_cta = (int)threads_per_cta;
    return o;
}

size_t ws_bytes(int64_t B, int64_t L, const tpl_options &o) { return tpl_a2b_workspace_bytes((int)B, (int)L, &o); }

void Angles2BackboneGPU_forward(torch::Tensor input_angles, torch::Tensor output_coords,
                                torch::Tensor angles_length, torch::Tensor A, int64_t residues_per_thread,
                                int64_t threads_per_cta) {
    check_cuda(input_angles, "input_angles");
    check_cuda(output_coords, "output_coords");
    check_cuda(angles_length, "angles_length");
    check_cuda(A, "A");
    TORCH_CHECK(input_angles.dim() == 3 && input_angles.size(1) == 3, "input_angles must be [batch, 3, max_len]");
    TORCH_CHECK(angles_length.scalar_type() == torch::kInt, "angles_length must be int32");
    const int64_t B = input_angles.size(0), L = input_angles.size(2);
    TORCH_CHECK(angles_length.numel() == B, "angles_length must have one entry per chain");
    TORCH_CHECK(output_coords.numel() == B * 9 * L, "output_coords must hold batch * 9 * max_len values");
    TORCH_CHECK(output_coords.scalar_type() == input_angles.scalar_type(), "output_coords dtype must match angles");
    const at::cuda::CUDAGuard guard(input_angles.device());
    void *st = stream_of(input_angles);
    int s;
    if (input_angles.scalar_type() == torch::kFloat) {
        const tpl_options o = call_options(residues_per_thread, threads_per_cta);
        s = tpl_a2b_forward_f32(input_angles.data_ptr<float>(), angles_length.data_ptr<int32_t>(),
                                output_coords.data_ptr<float>(), A.data_ptr(), A.nbytes(), (int)B, (int)L, &o, st);
    } else if (input_angles.scalar_type() == torch::kDouble) {
        s = tpl_a2b_forward_f64(input_angles.data_ptr<double>(), angles_length.data_ptr<int32_t>(),
                                output_coords.data_ptr<double>(), (int)B, (int)L, st);
    } else {
        TORCH_CHECK(false, "input_angles must be float32 or float64");
    }
    check_status(s, "Angles2BackboneGPU_forward");
}

void Angles2BackboneGPU_backward(torch::Tensor gradInput, torch::Tensor gradOutput, torch::Tensor input_angles,
                                 torch::Tensor angles_length, torch::Tensor A, torch::Tensor dr_dangle,
                                 int64_t residues_per_thread, int64_t threads_per_cta) {
    (void)dr_dangle;
    check_cuda(gradInput, "gradInput");
    check_cuda(gradOutput, "gradOutput");
    check_cuda(input_angles, "input_angles");
    check_cuda(angles_length, "angles_length");
    check_cuda(A, "A");
    TORCH_CHECK(input_angles.dim() == 3 && input_angles.size(1) == 3, "input_angles must be [batch, 3, max_len]");
    TORCH_CHECK(angles_length.scalar_type() == torch::kInt, "angles_length must be int32");
    const int64_t B = input_angles.size(0), L = input_angles.size(2);
    TORCH_CHECK(gradOutput.numel() == B * 9 * L, "gradOutput must hold batch * 9 * max_len values");
    TORCH_CHECK(gradInput.numel() == B * 3 * L, "gradInput must hold batch * 3 * max_len values");
    TORCH_CHECK(gradInput.scalar_type() == input_angles.scalar_type() &&
                    gradOutput.scalar_type() == input_angles.scalar_type(),
                "gradient dtypes must match angles");
    const at::cuda::CUDAGuard guard(input_angles.device());
    void *st = stream_of(input_angles);
    int s;
    if (input_angles.scalar_type() == torch::kFloat) {
        const tpl_options o = call_options(residues_per_thread, threads_per_cta);  // the forward's options
        s = tpl_a2b_backward_f32(gradInput.data_ptr<float>(), gradOutput.data_ptr<float>(),
                                 input_angles.data_ptr<float>(), angles_length.data_ptr<int32_t>(), A.data_ptr(),
                                 A.nbytes(), (int)B, (int)L, &o, st);
    } else if (input_angles.scalar_type() == torch::kDouble) {
        s = tpl_a2b_backward_f64(gradInput.data_ptr<double>(), gradOutput.data_ptr<double>(),
                                 input_angles.data_ptr<double>(), angles_length.data_ptr<int32_t>(), A.data_ptr(),
                                 A.nbytes(), (int)B, (int)L, st);
    } else {
        TORCH_CHECK(false, "input_angles must be float32 or float64");
    }
    check_status(s, "Angles2BackboneGPU_backward");
}

// Backward of the FP32 path from the forward's output coordinates (no re-walk).
// Not a reference entry point: the Python layer calls it with the coordinates it
// saved; Angles2BackboneGPU_backward above keeps the reference's signature.
int g_bwd_rpt = 0;  // residues per lane of the coordinate backward: 0 (= 4), 4 or 8
int g_bwd_buffers = 0;  // chunk buffers of the coordinate backward: 0 (= 1), 1 or 2
int g_bwd_scheme = 0;   // 0 (automatic) or 32 = one warp per chain, 4 = one CTA of four warps per chain

void Angles2BackboneGPU_backward_coords(torch::Tensor gradInput, torch::Tensor gradOutput, torch::Tensor output_coords,
                                        torch::Tensor angles_length, torch::Tensor A, int64_t residues_per_thread,
                                        int64_t copy_buffers, int64_t threads_per_cta) {
    check_cuda(gradInput, "gradInput");
    check_cuda(gradOutput, "gradOutput");
    check_cuda(output_coords, "output_coords");
    check_cuda(angles_length, "angles_length");
    check_cuda(A, "A");
    TORCH_CHECK(gradInput.dim() == 3 && gradInput.size(1) == 3, "gradInput must be [batch, 3, max_len]");
    TORCH_CHECK(angles_length.scalar_type() == torch::kInt, "angles_length must be int32");
    TORCH_CHECK(gradInput.scalar_type() == torch::kFloat && gradOutput.scalar_type() == torch::kFloat &&
                    output_coords.scalar_type() == torch::kFloat,
                "the coordinate backward is float32");
    const int64_t B = gradInput.size(0), L = gradInput.size(2);
    TORCH_CHECK(gradOutput.numel() == B * 9 * L && output_coords.numel() == B * 9 * L,
                "gradOutput and output_coords must hold batch * 9 * max_len values");
    const at::cuda::CUDAGuard guard(gradInput.device());
    tpl_options o = g_opt;
    o.residues_per_thread = residues_per_thread >= 0 ? (int)residues_per_thread : g_bwd_rpt;
    o.copy_buffers = copy_buffers >= 0 ? (int)copy_buffers : g_bwd_buffers;
    o.threads_per_cta = threads_per_cta >= 0 ? (int)threads_per_cta : g_bwd_scheme;
    const int s = tpl_a2b_backward_coords_f32(gradInput.data_ptr<float>(), gradOutput.data_ptr<float>(),
                                              output_coords.data_ptr<float>(), angles_length.data_ptr<int32_t>(),
                                              A.data_ptr(), A.nbytes(), (int)B, (int)L, &o, stream_of(gradInput));
    check_status(s, "Angles2BackboneGPU_backward_coords");
}

// The float32 Angles2Backbone autograd function in C++ (forward, then the backward
// from the coordinates it returned), so that the autograd engine calls the backward
// without a Python frame.  The caller passes the workspace and the per-call options
// (the layer's autotuned choice; -1 = the module-wide ones).
struct Angles2BackboneAutograd : public torch::autograd::Function<Angles2BackboneAutograd> {
    static torch::Tensor forward(torch::autograd::AutogradContext *ctx, torch::Tensor angles, torch::Tensor lengths,
                                 torch::Tensor A, std::vector<int64_t> fwd_opts, std::vector<int64_t> bwd_opts) {
        TORCH_CHECK(fwd_opts.size() == 2 && bwd_opts.size() == 3,
                    "fwd_opts = (residues_per_thread, threads_per_cta), bwd_opts = (residues_per_thread, "
                    "copy_buffers, threads_per_cta)");
        TORCH_CHECK(angles.scalar_type() == torch::kFloat, "the C++ Angles2Backbone function is float32");
        auto x = angles.contiguous();
        TORCH_CHECK(x.dim() == 3, "input_angles must be [batch, 3, max_len]");
        auto coords = torch::empty({x.size(0), 9 * x.size(2)}, x.options());
        Angles2BackboneGPU_forward(x, coords, lengths, A, fwd_opts[0], fwd_opts[1]);
        ctx->saved_data["bwd_opts"] = c10::IValue(bwd_opts);
        ctx->saved_data["angles_shape"] = c10::IValue(x.sizes().vec());
        ctx->save_for_backward({lengths, coords, A});
        return coords;
    }
    static torch::autograd::variable_list backward(torch::autograd::AutogradContext *ctx,
                                                   torch::autograd::variable_list grads) {
        auto s = ctx->get_saved_variables();
        const auto o = ctx->saved_data["bwd_opts"].toIntVector();
        auto g = grads[0].contiguous();
        auto grad = torch::empty(ctx->saved_data["angles_shape"].toIntVector(), g.options());
        Angles2BackboneGPU_backward_coords(grad, g, s[1], s[0], s[2], o[0], o[1], o[2]);
        return {grad, torch::Tensor(), torch::Tensor(), torch::Tensor(), torch::Tensor()};
    }
};

torch::Tensor angles2backbone_autograd(torch::Tensor angles, torch::Tensor lengths, torch::Tensor A,
                                       std::vector<int64_t> fwd_opts, std::vector<int64_t> bwd_opts) {
    return Angles2BackboneAutograd::apply(angles, lengths, A, fwd_opts, bwd_opts);
}

void set_backward_options(int64_t residues_per_thread, int64_t copy_buffers, int64_t threads_per_cta) {
    TORCH_CHECK(residues_per_thread == 0 || residues_per_thread == 4 || residues_per_thread == 8,
                "residues_per_thread of the coordinate backward must be 0, 4 or 8");
    TORCH_CHECK(copy_buffers >= 0 && copy_buffers <= 2 && !(copy_buffers == 2 && residues_per_thread == 8),
                "copy_buffers of the coordinate backward must be 0, 1 or 2 (2 with 4 residues per lane)");
    TORCH_CHECK(threads_per_cta == 0 || threads_per_cta == 32 || threads_per_cta == 4,
                "threads_per_cta of the coordinate backward must be 0 (automatic), 32 (one warp per chain) or 4 "
                "(one CTA of four warps per chain)");
    g_bwd_rpt = (int)residues_per_thread;
    g_bwd_buffers = (int)copy_buffers;
    g_bwd_scheme = (int)threads_per_cta;
}

void no_cpu_path(torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor) {
    TORCH_CHECK(false, "Angles2Backbone: this build has no CPU path; move the tensors to a CUDA device");
}
void no_cpu_path_bwd(torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor, torch::Tensor) {
    TORCH_CHECK(false, "Angles2Backbone: this build has no CPU path; move the tensors to a CUDA device");
}

int64_t workspace_bytes(int64_t B, int64_t L, int64_t residues_per_thread, int64_t threads_per_cta) {
    return (int64_t)ws_bytes(B, L, call_options(residues_per_thread, threads_per_cta));
}

int64_t workspace_status(torch::Tensor A) {
    check_cuda(A, "A");
    const at::cuda::CUDAGuard guard(A.device());
    int st = 0;
    check_status(tpl_workspace_status(A.data_ptr(), stream_of(A), &st), "workspace_status");
    return st;
}

void set_options(int64_t residues_per_thread, int64_t fp64_carry_min_len, int64_t renormalize, int64_t max_ctas,
                 int64_t threads_per_cta) {
    tpl_options o = {(int)residues_per_thread, (int)threads_per_cta, (int)fp64_carry_min_len, (int)renormalize,
                     (int)max_ctas, g_opt.copy_buffers};
    TORCH_CHECK(o.threads_per_cta == 0 || o.threads_per_cta == 1 || o.threads_per_cta == 128 ||
                    o.threads_per_cta == 32 || o.threads_per_cta == 4,
                "threads_per_cta must be 0 (automatic), 1 (warp tiles), 128 (CTA tiles), 32 (one warp per chain) "
                "or 4 (one CTA of four warps per chain)");
    TORCH_CHECK((o.threads_per_cta != 32 && o.threads_per_cta != 4) || o.residues_per_thread == 0 ||
                    o.residues_per_thread == 4 || o.residues_per_thread == 8,
                "one warp or one CTA per chain takes residues_per_thread 4 or 8");
    TORCH_CHECK(o.residues_per_thread == 0 || o.residues_per_thread == 1 || o.residues_per_thread == 2 ||
                    o.residues_per_thread == 4 || o.residues_per_thread == 8,
                "residues_per_thread must be 0, 1, 2, 4 or 8");
    g_opt = o;
}

std::vector<int64_t> get_options() {
    return {g_opt.residues_per_thread, g_opt.fp64_carry_min_len, g_opt.renormalize, g_opt.max_ctas,
            g_opt.threads_per_cta};
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("Angles2BackboneGPU_forward", &Angles2BackboneGPU_forward, "Angles2Backbone gpu forward",
          py::arg("input_angles"), py::arg("output_coords"), py::arg("angles_length"), py::arg("A"),
          py::arg("residues_per_thread") = -1, py::arg("threads_per_cta") = -1);
    m.def("Angles2BackboneGPU_backward", &Angles2BackboneGPU_backward, "Angles2Backbone gpu backward",
          py::arg("gradInput"), py::arg("gradOutput"), py::arg("input_angles"), py::arg("angles_length"), py::arg("A"),
          py::arg("dr_dangle"), py::arg("residues_per_thread") = -1, py::arg("threads_per_cta") = -1);
    m.def("Angles2BackboneCPU_forward", &no_cpu_path, "not available: no CPU path");
    m.def("Angles2BackboneCPU_backward", &no_cpu_path_bwd, "not available: no CPU path");
    m.def("workspace_bytes", &workspace_bytes, "bytes of the A workspace for (batch, max_len)", py::arg("batch"),
          py::arg("max_len"), py::arg("residues_per_thread") = -1, py::arg("threads_per_cta") = -1);
    m.def("workspace_status", &workspace_status, "synchronise and read the first device-detected error");
    m.def("set_options", &set_options, "tuning knobs", py::arg("residues_per_thread") = 0,
          py::arg("fp64_carry_min_len") = 0, py::arg("renormalize") = 0, py::arg("max_ctas") = 0,
          py::arg("threads_per_cta") = 0);
    m.def("get_options", &get_options, "current tuning knobs");
    m.def("Angles2BackboneGPU_backward_coords", &Angles2BackboneGPU_backward_coords,
          "float32 backward from the forward's output coordinates", py::arg("gradInput"), py::arg("gradOutput"),
          py::arg("output_coords"), py::arg("angles_length"), py::arg("A"), py::arg("residues_per_thread") = -1,
          py::arg("copy_buffers") = -1, py::arg("threads_per_cta") = -1);
    m.def("set_backward_options", &set_backward_options,
          "residues per lane, chunk buffers and scheme of the coordinate backward",
          py::arg("residues_per_thread") = 0, py::arg("copy_buffers") = 0, py::arg("threads_per_cta") = 0);
    m.def("get_backward_options", []() { return std::vector<int64_t>{g_bwd_rpt, g_bwd_buffers, g_bwd_scheme}; },
          "residues per lane, chunk buffers and scheme of the coordinate backward");
    m.def("angles2backbone_autograd", &angles2backbone_autograd,
          "float32 Angles2Backbone as a C++ autograd function (backward from the coordinates)", py::arg("angles"),
          py::arg("lengths"), py::arg("A"), py::arg("fwd_opts"), py::arg("bwd_opts"));
}
