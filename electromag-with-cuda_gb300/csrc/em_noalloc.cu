// em_calc_field_noalloc_f32: the device-pointer tracer for callers that
// cannot let this library allocate device memory.
//
// Who needs it: an application that hands the whole GPU to its own memory
// pool (so a cudaMalloc from a library would fail or fragment the arena),
// and code that cannot afford the device-wide synchronisation a cudaMalloc or
// cudaFree may imply in the middle of its stream work.  Such a caller passes
// its inputs and outputs as device pointers; this entry point's only scratch
// (the staged, padded charge copy and the kernel's error word) lives in the
// file-scope __device__ array below, which every GPU that loads the library
// holds until the process exits.
//
// Rules of use:
// - Limit: at most EM_NOALLOC_MAX_CHARGES charges; larger sets are refused
//   with EM_ERR_TOO_LARGE before any device work.
// - The first call on a device does a one-time set-up (it looks up the
//   array's device address with cudaGetSymbolAddress, which may load this
//   module onto the device); make that first call before any stream capture.
// - Every call waits for its own work: it reads the kernel's error word back
//   and synchronises `stream` before it returns.
// - Every call on a device shares the one array and leaves its contents
//   behind.  The error word is cleared at the start of each call; the staged
//   charges are rewritten.  Calls whose work overlaps on the GPU (different
//   streams or threads without ordering) race on the array: order them.
#include <climits>
#include <mutex>

#include "em_internal.h"
#include "em_plan.h"
#include "emgb300.h"

namespace em {
namespace {

// Staged charges (padding granule at most 128 records) + a 256-B error slot.
constexpr size_t kNoallocChargeBytes = (size_t)(EM_NOALLOC_MAX_CHARGES + 128) * 16;
constexpr size_t kNoallocBytes = kNoallocChargeBytes + 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

struct NoallocDev {
    bool ready = false;
    void *scratch = nullptr; // device address of g_noalloc_scratch on this device
    int nsm = 0;
    size_t smem_optin = 0;
};

std::mutex g_noalloc_mu;
NoallocDev g_noalloc_dev[kMaxDevices];

// Once per device, with that device current: the array's device address and
// the device shape the planner needs.
int noalloc_setup(int dev, NoallocDev **out)
{
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    NoallocDev &d = g_noalloc_dev[dev];
    if (!d.ready) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return EM_ERR_CUDA;
        }
        int nsm = 0, smem = 0;
        if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
                cudaSuccess) {
            cudaGetLastError();
            return EM_ERR_NO_DEVICE;
        }
        d.scratch = ptr;
        d.nsm = nsm;
        d.smem_optin = (size_t)smem;
        d.ready = true;
    }
    *out = &d;
    return EM_OK;
}

} // namespace
} // namespace em

extern "C" int em_calc_field_noalloc_f32(float *x, float *y, float *z, size_t n,
                                         size_t total_steps, const float *charges, size_t p,
                                         float resolution, int use_curvature, void *stream)
{
    using namespace em;
    // the reference's checks and order (CPU_Implement.cpp:213-230), any n
    if (!n)
        return EM_ERR_N_ZERO;
    if (resolution == 0)
        return EM_ERR_RESOLUTION;
    if (total_steps < 2)
        return EM_ERR_STEPS;
    if (!x || !y || !z || (p && !charges) || ((uintptr_t)charges & 15))
        return EM_ERR_ARG;
    if (p > (size_t)EM_NOALLOC_MAX_CHARGES)
        return EM_ERR_TOO_LARGE;
    if (total_steps > (size_t)INT_MAX || n > (size_t)(LLONG_MAX / 64) / total_steps)
        return EM_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    NoallocDev *d = nullptr;
    int code = noalloc_setup(dev, &d);
    if (code)
        return code;

    // plan exactly as the allocating entry point does (default options)
    em_options o{};
    DevCtx shape;
    shape.nsm = d->nsm;
    shape.smem_optin = d->smem_optin;
    Plan pl;
    code = make_plan<float>(shape, n, p, o, &pl);
    if (code)
        return code;
    if ((size_t)pl.p_pad * 16 > kNoallocChargeBytes)
        return EM_ERR_TOO_LARGE;

    unsigned char *base = static_cast<unsigned char *>(d->scratch);
    void *staged = base;
    int *err = reinterpret_cast<int *>(base + kNoallocChargeBytes);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e == cudaSuccess)
        e = launch_stage_charges<float>(charges, (int)p, staged, pl.p_pad,
                                        stage_layout(pl.arith), pl.cfg.tile_recs, s);
    RefTraceParams<float> prm{};
    prm.x = x;
    prm.y = y;
    prm.z = z;
    prm.charges = staged;
    prm.n = (long long)n;
    prm.n_groups = pl.n_groups;
    prm.total_steps = (int)total_steps;
    prm.p_pad = pl.p_pad;
    prm.n_tiles = pl.n_tiles;
    prm.tile_recs = pl.cfg.tile_recs;
    prm.stages = pl.cfg.stages;
    prm.resident = pl.cfg.resident;
    prm.rule = use_curvature ? RULE_SSE : RULE_FIXED;
    prm.resolution = resolution;
    prm.err = err;
    if (pl.arith == ARITH_EXACT)
        prm.exact_nb = exact_nb_verified(s) ? 1 : 0;
    if (e == cudaSuccess)
        e = launch_ref_trace<float>(prm, pl.cfg, pl.arith, s);
    int dev_err = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&dev_err, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return map_cuda(e);
    return dev_err == EM_DEVERR_TIMEOUT ? EM_ERR_TIMEOUT : (dev_err ? EM_ERR_CUDA : EM_OK);
}
