// Device diagnostics: the FP32 FFMA throughput of the current device (the
// denominator of the tracer's FP32 roofline) and the count of kernels this
// library has launched in the process.
#include <atomic>

#include "em_device.cuh"
#include "em_internal.h"
#include "emgb300.h"

namespace em {

std::atomic<unsigned long long> g_launches{0};

void count_launch(unsigned long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

namespace {

// 8 independent FFMA chains per thread; every result feeds the output so
// nothing is dead code.  a <- a*b + c with |b| < 1 keeps values bounded.
__global__ void __launch_bounds__(512) ffma_peak_kernel(float *out, int iters, float b, float c)
{
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        a[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int k = 0; k < 8; ++k)
                a[k] = fmaf(a[k], b, c);
        }
    }
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// One warp waits on an mbarrier that nothing completes, with a short limit:
// the bounded-wait path every tracer kernel relies on, exercised on purpose.
__global__ void wait_selftest_kernel(int *err, unsigned long long limit_ns)
{
    __shared__ __align__(8) uint64_t bar;
    const uint32_t b = smem_addr(&bar);
    if (threadIdx.x == 0) {
        mbar_init(b, 1);
        fence_mbar_init();
    }
    __syncwarp();
    mbar_wait_limit(b, 0, err, limit_ns);
}

} // namespace
} // namespace em

extern "C" {

int em_selftest_wait_timeout(int limit_ms, double *elapsed_ms)
{
    if (limit_ms < 1 || limit_ms > 5000)
        return EM_ERR_ARG;
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_NOMEM;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemset(err, 0, sizeof(int));
    cudaEventRecord(e0);
    em::wait_selftest_kernel<<<1, 32>>>(err, (unsigned long long)limit_ms * 1000000ull);
    cudaEventRecord(e1);
    em::count_launch(1);
    int v = 0;
    cudaError_t e = cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost);
    float ms = 0;
    if (e == cudaSuccess)
        cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(err);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_CUDA;
    }
    if (elapsed_ms)
        *elapsed_ms = ms;
    return v == em::EM_DEVERR_TIMEOUT ? EM_ERR_TIMEOUT : (v ? EM_ERR_CUDA : EM_OK);
}

int em_fp32_peak_tflops(double *tflops, double *seconds)
{
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    const int blocks = prop.multiProcessorCount * 4, threads = 512, iters = 4096;
    float *out = nullptr;
    cudaEvent_t e0, e1;
    if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_NOMEM;
    }
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        em::ffma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-4f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best)
            best = ms;
    }
    em::count_launch(4);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess)
        return EM_ERR_CUDA;
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    if (tflops)
        *tflops = flops / (best * 1e-3) / 1e12;
    if (seconds)
        *seconds = best * 1e-3;
    return EM_OK;
}

unsigned long long em_launch_count(void) { return em::g_launches.load(); }

} // extern "C"
