// mce_batch_step_noalloc: the batched step for callers that may not allocate
// device memory while they estimate.
//
// Who cannot allocate: a process whose device memory is already handed out
// (a PyTorch job whose caching allocator holds the GPU, a real-time or
// embedded loop that sizes all of its memory at start-up and treats an
// allocation failure mid-run as unacceptable), and any caller for which the
// device-wide synchronisation of cudaMalloc/cudaFree would stall work on
// other streams.  mce_batch_step grows the handle's buffers, and its g-table
// kernel's per-warp scratch, with cudaMalloc whenever a step needs more room.
//
// This entry point runs the same step with two differences:
//  * the g-table kernel (k_gtable) takes its per-warp scratch from the
//    file-scope array below instead of a buffer of the handle, launching only
//    as many warps as the array has slots for; the warps stride over the
//    roots, so the tables are the same;
//  * no device buffer of the handle may grow: one that would have to fails
//    the call with MCE_ERR_NOMEM instead of calling cudaMalloc.
// It calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array is shared by every call in the process on a device and keeps the
// last call's contents.  k_gtable writes each scratch slot before it reads it
// within the same call, so nothing needs clearing between calls.  Calls that
// overlap on the GPU (two handles stepped from two threads, or on streams
// that are not ordered) race on the array: serialise them.
#include "../../include/mce_c_api.h"

#include <cuda_runtime.h>

#include <mutex>
#include <string>

struct mce_handle;

namespace mce {
void report_error(const std::string& s);
int batch_step_in_fixed_scratch(mce_handle* h, void* scratch, size_t bytes, const double* msmt, const double* Phi,
                                const double* Gamma, const double* beta, const double* H, const double* gamma,
                                const double* B, const double* u, int shared_model, int* err_out);
}  // namespace mce

// 32 MiB: 2 Mi complex doubles.  One warp needs half the cells of a
// full-shape term; the call is refused when 4 warps (one block) do not fit,
// i.e. above 524,288 half-cells, which no handle of this build reaches (16
// hyperplanes in 8 states is 16,384).  The grid matches mce_batch_step's
// (152 SMs x 64 warps) up to 215 half-cells per term and shrinks above that.
static constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_gtable_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the array on the current device, looked up once per
// device (the first call on a device does this set-up).
int scratch_on_current_device(void** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        mce::report_error(std::string("mce_batch_step_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return MCE_ERR_DEVICE;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        mce::report_error("mce_batch_step_noalloc: device ordinal " + std::to_string(dev) + " out of range");
        return MCE_ERR_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_gtable_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            mce::report_error(std::string("mce_batch_step_noalloc: cudaGetSymbolAddress of the static scratch: ") +
                              cudaGetErrorString(e));
            return MCE_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return MCE_OK;
}

}  // namespace

extern "C" int mce_batch_step_noalloc(mce_handle* h, const double* msmt, const double* Phi, const double* Gamma,
                                      const double* beta, const double* H, const double* gamma, const double* B,
                                      const double* u, int shared_model, int* err_out)
{
    if (!h) return MCE_ERR_ARG;
    void* scratch = nullptr;
    const int s = scratch_on_current_device(&scratch);
    if (s != MCE_OK) return s;
    return mce::batch_step_in_fixed_scratch(h, scratch, kNoAllocScratchBytes, msmt, Phi, Gamma, beta, H, gamma, B, u,
                                            shared_model, err_out);
}
