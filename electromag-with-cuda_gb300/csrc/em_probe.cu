// Device diagnostics: the FP32 FFMA throughput of the current device (the
// denominator of the tracer's FP32 roofline), the count of kernels this
// library has launched in the process, and self-checks (the bounded device
// wait; the branch-free rounded operations of the exact arithmetic against
// the compiler's rounded operations).
#include <atomic>
#include <mutex>

#include "em_device.cuh"
#include "em_internal.h"
#include "em_math.cuh"
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

// The exact arithmetic's branch-free root, reciprocal and quotient against
// __fsqrt_rn, __frcp_rn and __fdiv_rn over the operand ranges it admits:
// every float in [2^-40, 2^40] (roots), every float in [2^-60, 2^60]
// (divisors), and n quotients of a numerator and divisor with seeded random
// significands, exponents in [-60, 60] and signs.  bad[0..2]: mismatches.
__device__ __forceinline__ unsigned long long selftest_mix(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void rounded_ops_kernel(unsigned long long n, unsigned long long *bad)
{
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long i0 = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    unsigned long long b0 = 0, b1 = 0, b2 = 0;
    // bit patterns: 2^-40 .. 2^40 and 2^-60 .. 2^60 (positive, normal)
    const unsigned r_lo = (127u - 40u) << 23, r_hi = (127u + 40u) << 23;
    const unsigned d_lo = (127u - 60u) << 23, d_hi = (127u + 60u) << 23;
    for (unsigned long long u = d_lo + i0; u <= d_hi; u += stride) {
        const float x = __uint_as_float((unsigned)u);
        if (u >= r_lo && u <= r_hi)
            b0 += __float_as_uint(sqrt_rn_nb(x)) != __float_as_uint(__fsqrt_rn(x));
        b1 += __float_as_uint(rcp_rn_nb(x)) != __float_as_uint(__frcp_rn(x));
    }
    for (unsigned long long i = i0; i < n; i += stride) {
        const unsigned long long h = selftest_mix(i ^ 0x5eed5eed5eedull);
        const unsigned ma = (unsigned)(h & 0x7fffff), mb = (unsigned)((h >> 23) & 0x7fffff);
        const unsigned ea = (unsigned)((h >> 46) % 121) + 67u, eb = (unsigned)((h >> 54) % 121) + 67u;
        const unsigned sa = (unsigned)(h >> 62) & 1u, sb = (unsigned)(h >> 63) & 1u;
        const float a = __uint_as_float((sa << 31) | (ea << 23) | ma);
        const float b = __uint_as_float((sb << 31) | (eb << 23) | mb);
        b2 += __float_as_uint(div_rn_nb(a, b, rcp_rn_nb(b))) != __float_as_uint(__fdiv_rn(a, b));
    }
    if (b0)
        atomicAdd(&bad[0], b0);
    if (b1)
        atomicAdd(&bad[1], b1);
    if (b2)
        atomicAdd(&bad[2], b2);
}

// the check's counters: a static array, so the check allocates nothing
__device__ unsigned long long g_rounded_bad[3];
std::mutex g_rounded_mu;

// Runs the check on stream s (serialised: one set of counters per device).
cudaError_t run_rounded_check(unsigned long long n_quotients, unsigned long long *out,
                              cudaStream_t s)
{
    std::lock_guard<std::mutex> guard(g_rounded_mu);
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    void *bad = nullptr;
    if (e == cudaSuccess)
        e = cudaGetSymbolAddress(&bad, g_rounded_bad);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(bad, 0, 3 * sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        rounded_ops_kernel<<<nsm * 8, 256, 0, s>>>(n_quotients,
                                                   static_cast<unsigned long long *>(bad));
        count_launch(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, bad, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    return e;
}

} // namespace

bool exact_nb_verified(cudaStream_t s)
{
    constexpr int kMaxDev = 64;
    static std::atomic<int> state[kMaxDev]; // 0 unknown, 1 verified, 2 not
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) {
        cudaGetLastError();
        return false;
    }
    const int v = state[dev].load();
    if (v)
        return v == 1;
    unsigned long long bad[3] = {1, 1, 1};
    const cudaError_t e = run_rounded_check(1ull << 24, bad, s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false; // not verified: the compiler's rounded operations
    }
    const bool ok = bad[0] == 0 && bad[1] == 0 && bad[2] == 0;
    state[dev].store(ok ? 1 : 2);
    return ok;
}

} // namespace em

extern "C" {

int em_selftest_rounded_ops(unsigned long long n_quotients, unsigned long long *mismatches)
{
    if (!mismatches)
        return EM_ERR_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    if (em::run_rounded_check(n_quotients, mismatches, 0) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_CUDA;
    }
    return EM_OK;
}


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
