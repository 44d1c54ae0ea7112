// The --autoregress check of ElectroMag.cpp:400-453 on the GPU: for every
// line, the first row where the two runs' vertices lie more than a threshold
// apart, then the reference's regression.txt report for those lines.
//
// The scan is memory-bound (24 bytes per vertex pair).  A work item is 32
// consecutive lines (one per lane, so every row load is coalesced) times a
// chunk of 64 rows; items are dealt chunk-major so early chunks finish first
// and later chunks of an already-diverged line are skipped.  The distance is
// the reference's vec3Len(vec3(a, b)) in FP32 with one rounding per
// operation, so the decision at the threshold matches its x86 build.
#include <climits>
#include <cstdio>
#include <mutex>
#include <vector>

#include "em_internal.h"
#include "em_plan.h"
#include "emgb300.h"

namespace em {
namespace {

constexpr int kRegressChunk = 64;   // rows per work item
constexpr int kRecFloats = 16;      // report record per line

__device__ __forceinline__ float offset3(float ax, float ay, float az, float bx, float by,
                                         float bz)
{
    const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    return __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}

struct RegressArgs {
    const float *ax, *ay, *az, *bx, *by, *bz;
    long long n;
    int rows;
    float thr;
    unsigned long long *first; // ULLONG_MAX: no divergence found
    float *rec;                // n * kRecFloats
};

__global__ void __launch_bounds__(256) diverge_kernel(const RegressArgs A)
{
    const long long groups = (A.n + 31) / 32;
    const long long chunks = (A.rows + kRegressChunk - 1) / kRegressChunk;
    const long long items = groups * chunks;
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long it = w0; it < items; it += nw) {
        const long long g = it % groups, c = it / groups;
        const long long line = g * 32 + lane;
        if (line >= A.n)
            continue;
        const int s0 = (int)(c * kRegressChunk);
        const int s1 = min(A.rows, s0 + kRegressChunk);
        if (*(volatile unsigned long long *)(A.first + line) <= (unsigned long long)s0)
            continue; // an earlier chunk already found this line's row
        // four rows' loads in flight before their offsets are tested
        constexpr int U = 4;
        bool found = false;
        for (int s = s0; s < s1 && !found; s += U) {
            float v[U][6];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const size_t i = (size_t)min(s + u, s1 - 1) * (size_t)A.n + (size_t)line;
                v[u][0] = A.ax[i];
                v[u][1] = A.ay[i];
                v[u][2] = A.az[i];
                v[u][3] = A.bx[i];
                v[u][4] = A.by[i];
                v[u][5] = A.bz[i];
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (!found && s + u < s1 &&
                    offset3(v[u][0], v[u][1], v[u][2], v[u][3], v[u][4], v[u][5]) > A.thr) {
                    atomicMin(A.first + line, (unsigned long long)(s + u));
                    found = true;
                }
            }
        }
    }
}

// Report record of a diverged line: rows s-1 (absent for s = 0) and s of
// both runs with their offsets.
__global__ void diverge_gather_kernel(const RegressArgs A)
{
    const long long line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (line >= A.n)
        return;
    const unsigned long long s = A.first[line];
    if (s >= (unsigned long long)A.rows)
        return;
    float *r = A.rec + (size_t)line * kRecFloats;
    for (int k = 0; k < 2; ++k) {
        if (k == 0 && s == 0)
            continue;
        const size_t i = (size_t)(s - 1 + k) * (size_t)A.n + (size_t)line;
        float *o = r + 7 * k;
        o[0] = A.ax[i];
        o[1] = A.ay[i];
        o[2] = A.az[i];
        o[3] = A.bx[i];
        o[4] = A.by[i];
        o[5] = A.bz[i];
        o[6] = offset3(o[0], o[1], o[2], o[3], o[4], o[5]);
    }
}

void put_pair(std::FILE *f, unsigned long long line, long long row, const float *o)
{
    std::fprintf(f, " CPUL [%llu][%lld] x: %g y: %g z: %g\n", line, row, (double)o[0],
                 (double)o[1], (double)o[2]);
    std::fprintf(f, " GPUL [%llu][%lld] x: %g y: %g z: %g\n", line, row, (double)o[3],
                 (double)o[4], (double)o[5]);
    std::fprintf(f, " 3D offset: %g\n", (double)o[6]);
}

int autoregress(const char *path, size_t n, size_t rows, const float *ax, const float *ay,
                const float *az, const float *bx, const float *by, const float *bz, float thr,
                long long *first_out, size_t *ndiv, const em_options *opt)
{
    if (!n)
        return EM_ERR_N_ZERO;
    if (!rows)
        return EM_ERR_STEPS;
    if (!ax || !ay || !az || !bx || !by || !bz)
        return EM_ERR_ARG;
    if (rows > (size_t)INT_MAX || n > (size_t)(LLONG_MAX / 64) / rows)
        return EM_ERR_TOO_LARGE;
    em_options o{};
    if (opt)
        o = *opt;
    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);
    cudaStream_t s = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;
    const size_t elems = n * rows;

    RegressArgs A{};
    A.n = (long long)n;
    A.rows = (int)rows;
    A.thr = thr;
    cudaError_t e = cudaSuccess;
    if (o.device_ptrs) {
        A.ax = ax, A.ay = ay, A.az = az, A.bx = bx, A.by = by, A.bz = bz;
    } else {
        if ((code = grow(&c.lines, &c.lines_cap, 3 * elems * 4)) ||
            (code = grow(&c.scratch, &c.scratch_cap, 3 * elems * 4)))
            return code;
        float *da = static_cast<float *>(c.lines), *db = static_cast<float *>(c.scratch);
        const float *src[6] = {ax, ay, az, bx, by, bz};
        float *dst[6] = {da, da + elems, da + 2 * elems, db, db + elems, db + 2 * elems};
        for (int k = 0; k < 6 && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(dst[k], src[k], elems * 4, cudaMemcpyHostToDevice, s);
        A.ax = dst[0], A.ay = dst[1], A.az = dst[2], A.bx = dst[3], A.by = dst[4], A.bz = dst[5];
    }
    const size_t off_rec = (n * 8 + 255) / 256 * 256;
    if ((code = grow(&c.adj, &c.adj_cap, off_rec + n * kRecFloats * 4)))
        return code;
    A.first = static_cast<unsigned long long *>(c.adj);
    A.rec = reinterpret_cast<float *>(static_cast<unsigned char *>(c.adj) + off_rec);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(A.first, 0xff, n * 8, s);
    if (e == cudaSuccess) {
        diverge_kernel<<<c.nsm * 8, 256, 0, s>>>(A);
        diverge_gather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(A);
        count_launch(2);
        e = cudaGetLastError();
    }
    std::vector<unsigned long long> first(n);
    std::vector<float> rec(n * kRecFloats);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(first.data(), A.first, n * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rec.data(), A.rec, n * kRecFloats * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return map_cuda(e);

    size_t count = 0;
    for (size_t l = 0; l < n; ++l) {
        const bool hit = first[l] < (unsigned long long)rows;
        count += hit;
        if (first_out)
            first_out[l] = hit ? (long long)first[l] : -1;
    }
    if (ndiv)
        *ndiv = count;
    if (path) {
        std::FILE *f = std::fopen(path, "w");
        if (!f)
            return EM_ERR_IO;
        for (size_t l = 0; l < n; ++l) {
            const unsigned long long row = first[l];
            if (row >= (unsigned long long)rows)
                continue;
            const float *r = rec.data() + l * kRecFloats;
            if (row > 0)
                put_pair(f, l, (long long)row - 1, r);
            put_pair(f, l, (long long)row, r + 7);
            std::fputc('\n', f);
        }
        if (std::fclose(f) != 0)
            return EM_ERR_IO;
    }
    return EM_OK;
}

} // namespace
} // namespace em

extern "C" int em_autoregress_f32(const char *path, size_t n, size_t rows, const float *ax,
                                  const float *ay, const float *az, const float *bx,
                                  const float *by, const float *bz, float threshold,
                                  long long *first, size_t *ndiverged, const em_options *opt)
{
    return em::autoregress(path, n, rows, ax, ay, az, bx, by, bz, threshold, first, ndiverged,
                           opt);
}
