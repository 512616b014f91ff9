// Allocation-free K*u with the p.Kp dot product.
//
// Some callers cannot allocate device memory at the moment they need the
// operator: a real-time solver loop in a host application that fixes its
// device memory budget at start-up, or a plugin whose process hands all
// device memory to another framework's caching allocator.  sgld_kbyu_dot_noalloc serves them: its only
// scratch (one partial sum per CTA of the K*u grid) lives in the file-scope
// device array below, which every GPU that loads this library holds until the
// process exits.  The call itself allocates nothing.
#include <atomic>

#include "../../include/sgld_gpu.h"
#include "sgld_internal.cuh"

namespace sgld {
int kbyu_num_blocks(const Level &l0);
}

using namespace sgld;

// Scratch for the per-CTA partial sums of u . (K u): SGLD_NOALLOC_MAX_CTAS
// doubles (256 KiB).  Every slot a launch uses is written by that launch
// before it is read, so nothing needs clearing between calls.
static __device__ __align__(256) double g_noalloc_partial[SGLD_NOALLOC_MAX_CTAS];

namespace {
std::atomic<double *> g_partial_addr[kMaxDevices];   // device address of the array, per device
}  // namespace

void sgld::forget_noalloc_scratch(int dev) { g_partial_addr[dev] = nullptr; }

extern "C" int sgld_kbyu_dot_noalloc(sgld_ctx *ctx, const double *d_u, double *d_y, double *d_dot, void *stream) {
    if (!ctx || !d_u || !d_y || !d_dot) return SGLD_ERR_ARG;
    Ctx &c = ctx->c;
    if (!c.have_fixed || !c.have_E) {
        c.err = "sgld_kbyu_dot_noalloc: fixed DOFs and moduli must be set first";
        return SGLD_ERR_STATE;
    }
    const Level &l0 = c.lv[0];
    const int nb = kbyu_num_blocks(l0);
    if (nb > SGLD_NOALLOC_MAX_CTAS) {
        c.err = "sgld_kbyu_dot_noalloc: grid of " + std::to_string(nb) + " CTAs exceeds the scratch limit of " +
                std::to_string(SGLD_NOALLOC_MAX_CTAS) + " (use sgld_kbyu_device for larger grids)";
        return SGLD_ERR_ARG;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != c.device || dev < 0 || dev >= kMaxDevices) {
        c.err = "sgld_kbyu_dot_noalloc: the context's device must be current";
        return SGLD_ERR_STATE;
    }
    if (!kh_bound(c)) {   // the call changes no device state besides its outputs and scratch
        c.err = "sgld_kbyu_dot_noalloc: the device holds another context's element matrix; call any other "
                "entry point of this context (e.g. sgld_kbyu_device) first";
        return SGLD_ERR_STATE;
    }
    if (!g_partial_addr[dev]) {   // once per device: host code needs the array's device address
        double *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_partial);
        if (e != cudaSuccess || !ptr) {
            c.err = std::string("sgld_kbyu_dot_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return SGLD_ERR_CUDA;
        }
        g_partial_addr[dev] = ptr;
    }
    double *partial = g_partial_addr[dev];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int used = 0;
    launch_kbyu_f64(l0, c.E, d_u, d_y, partial, &used, st);
    launch_finalize_sum(partial, used, d_dot, st);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        c.err = std::string("sgld_kbyu_dot_noalloc: ") + cudaGetErrorString(e);
        return SGLD_ERR_CUDA;
    }
    return SGLD_OK;
}
