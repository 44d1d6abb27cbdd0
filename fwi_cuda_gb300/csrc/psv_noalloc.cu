// psv_noalloc.cu -- psv_misfit_noalloc: the misfit reduction for callers that
// must not allocate device memory.
//
// Who needs it: code that calls this library from inside another runtime's
// memory discipline -- a host application whose GPU memory is all owned by a
// framework allocator or a pre-sized pool (its own cudaMalloc would bypass
// that accounting, and fail once the pool holds the device), or a real-time
// loop that must not hit cudaMalloc/cudaFree latency or fragmentation.  Those callers own their input and output buffers already;
// what psv_misfit would allocate beyond them is only scratch: the per-block
// partial sums of the deterministic two-stage L2 reduction.  Here that
// scratch is a fixed file-scope device array instead.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "fwi_psv.h"
#include "psv_fwi.cuh"
#include "psv_internal.h"

namespace {

// Partial sums per shot: the first-stage grid of launch_adjsrc, whose
// partial-sum buffer this array stands in for.
constexpr int kPartialPerShot = psv::kRedBlocks;
static_assert(kPartialPerShot * PSV_MISFIT_NOALLOC_MAX_SHOTS * sizeof(double) == (2u << 20),
              "the scratch array's stated size (2 MiB) follows from the reduction's grid");

// Scratch of every psv_misfit_noalloc call on a device: 256 partial sums per
// shot for up to PSV_MISFIT_NOALLOC_MAX_SHOTS shots (2 MiB).  Each GPU that
// loads the library holds it until the process exits.
static __device__ __align__(256) double g_misfit_scratch[kPartialPerShot * PSV_MISFIT_NOALLOC_MAX_SHOTS];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so its device address is
// looked up once per device, with that device current.
int scratch_for_current_device(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return psv::fail(PSV_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return psv::fail(PSV_ERR_UNSUPPORTED, "device index above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_misfit_scratch);
        if (e != cudaSuccess || !p)
            return psv::fail(PSV_ERR_CUDA, std::string("cudaGetSymbolAddress(misfit scratch): ") +
                                               cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_ptr[dev];
    return PSV_OK;
}

}  // namespace

extern "C" int psv_misfit_noalloc(const double *d_mod_z, const double *d_mod_x,
                                  const double *d_true_z, const double *d_true_x, double *d_res_z,
                                  double *d_res_x, int nshot, int nrec, int nt, double dt,
                                  double *d_L2, void *stream)
{
    if (!d_mod_z || !d_mod_x || !d_true_z || !d_true_x || !d_L2)
        return psv::fail(PSV_ERR_ARG, "misfit_noalloc: null device pointer");
    if ((d_res_z == nullptr) != (d_res_x == nullptr))
        return psv::fail(PSV_ERR_ARG, "misfit_noalloc: give both residual outputs or neither");
    if (nshot <= 0 || nrec < 0 || nt < 0)
        return psv::fail(PSV_ERR_ARG, "misfit_noalloc: nshot must be > 0, nrec and nt >= 0");
    if (nshot > PSV_MISFIT_NOALLOC_MAX_SHOTS)
        return psv::fail(PSV_ERR_ARG, "misfit_noalloc: nshot " + std::to_string(nshot) +
                                          " exceeds the fixed scratch size (PSV_MISFIT_NOALLOC_MAX_SHOTS = " +
                                          std::to_string(PSV_MISFIT_NOALLOC_MAX_SHOTS) + ")");
    double *scratch = nullptr;
    const int s = scratch_for_current_device(&scratch);
    if (s != PSV_OK) return s;
    // Every partial sum is written by the first kernel before the second
    // reads it, so the scratch left by an earlier call needs no clearing.
    const cudaError_t e = psv::launch_adjsrc(d_mod_z, d_mod_x, d_true_z, d_true_x, d_res_z,
                                             d_res_x, (long long)nrec * nt, nshot, dt, scratch,
                                             d_L2, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return psv::fail(PSV_ERR_CUDA, std::string("misfit_noalloc launch: ") + cudaGetErrorString(e));
    return PSV_OK;
}
