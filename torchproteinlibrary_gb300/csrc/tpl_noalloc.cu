// tpl_a2b_forward_f32_noalloc: the Angles2Backbone FP32 forward for callers that
// cannot allocate device memory (see include/tpl_gb300.h).  Its scratch, the
// tile scan's look-back records, lives in a fixed array declared here in device
// memory instead of a caller-provided workspace.
#include <cstdint>
#include <mutex>

#include "tpl_internal.h"

namespace tpl {

// Maximum scratch of the no-allocation entry point.  Every GPU that loads the
// library holds this array until the process exits.
constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// In host code `g_noalloc_scratch` names a host-side stand-in, not a device
// address; the device address is looked up once per device, with that device
// current, and cached.  A cudaDeviceReset (or a release and re-creation of the
// primary context) reloads the module and leaves the cached address stale, so
// the entry points below must not be used across a device reset.
static void *noalloc_scratch_ptr(int *status) {
    static std::mutex mu;
    static void *ptrs[256] = {nullptr};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
        *status = TPL_ERR_LAUNCH;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (!ptrs[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
            *status = TPL_ERR_LAUNCH;
            return nullptr;
        }
        ptrs[dev] = p;
    }
    *status = TPL_OK;
    return ptrs[dev];
}

}  // namespace tpl

using namespace tpl;

extern "C" int tpl_a2b_forward_f32_noalloc(const float *angles, const int32_t *lengths, float *coords, int batch,
                                           int max_len, const tpl_options *opt, void *stream) {
    if (batch < 0 || max_len < 0) return TPL_ERR_ARGUMENT;
    const tpl_options o = resolve(opt);
    if (!options_ok(o)) return TPL_ERR_ARGUMENT;
    if (batch == 0 || max_len == 0) return TPL_OK;
    if (!angles || !lengths || !coords) return TPL_ERR_ARGUMENT;
    const size_t need = a2b_ws(batch, max_len, o);
    if (need > kNoAllocScratchBytes) return TPL_ERR_TOO_LARGE;
    int status = TPL_OK;
    void *scratch = noalloc_scratch_ptr(&status);
    if (status != TPL_OK) return status;
    // the look-back flags, tickets and epochs must start at zero
    if (cudaMemsetAsync(scratch, 0, need, (cudaStream_t)stream) != cudaSuccess) return TPL_ERR_LAUNCH;
    return a2b_forward_f32(angles, lengths, coords, scratch, batch, max_len, o, (cudaStream_t)stream);
}

// The status word sits at the start of the scratch (the workspace header that the
// kernels write their first error into).  The next no-allocation call clears it.
extern "C" int tpl_a2b_noalloc_status(void *stream, int *status_out) {
    if (!status_out) return TPL_ERR_ARGUMENT;
    int status = TPL_OK;
    void *scratch = noalloc_scratch_ptr(&status);
    if (status != TPL_OK) return status;
    return tpl_workspace_status(scratch, stream, status_out);
}
