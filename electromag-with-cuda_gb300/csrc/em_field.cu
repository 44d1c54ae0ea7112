// Field at arbitrary points: E(p_i) = sum_j PartField(charge_j, p_i) in
// charge order, one thread per point (include/Electrostatics.h:38-60 summed
// as CPU_Implement.cpp:274-320 does).  Not the tracer's hot loop: it exists
// to evaluate the field where a caller (or a parity check) needs it.
#include "em_device.cuh"
#include "em_internal.h"

namespace em {
namespace {

__device__ __forceinline__ float f_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float f_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float f_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float f_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float f_sqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double f_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double f_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double f_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double f_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double f_sqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float f_rsqrt(float a) { return rsqrtf(a); }
__device__ __forceinline__ double f_rsqrt(double a) { return rsqrt(a); }

constexpr int kFieldTile = 256;

template <class T, int ARITH>
__global__ void __launch_bounds__(256) field_kernel(const T *px, const T *py, const T *pz,
                                                    long long m, const T *charges, int p,
                                                    int three_arg, T *ex, T *ey, T *ez)
{
    __shared__ T sc[kFieldTile * 4];
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool own = i < m;
    const T x = own ? px[i] : T(0), y = own ? py[i] : T(0), z = own ? pz[i] : T(0);
    const T K = (T)kElectroK;
    T ax = 0, ay = 0, az = 0;
    for (int base = 0; base < p; base += kFieldTile) {
        const int cnt = min(kFieldTile, p - base);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt * 4; k += blockDim.x)
            sc[k] = charges[(size_t)base * 4 + k];
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const T cx = sc[4 * j], cy = sc[4 * j + 1], cz = sc[4 * j + 2], q = sc[4 * j + 3];
            if (ARITH == ARITH_FAST) {
                const T dx = x - cx, dy = y - cy, dz = z - cz;
                const T r2 = fma(dz, dz, fma(dy, dy, dx * dx));
                const T inv = f_rsqrt(r2);
                const T s = (q * inv) * (inv * inv);
                ax = fma(s, dx, ax);
                ay = fma(s, dy, ay);
                az = fma(s, dz, az);
            } else {
                const T rx = f_sub(x, cx), ry = f_sub(y, cy), rz = f_sub(z, cz);
                const T l2 = f_add(f_add(f_mul(rx, rx), f_mul(ry, ry)), f_mul(rz, rz));
                const T d = f_mul(l2, f_sqrt(l2));
                if (three_arg) {
                    ax = f_add(ax, f_div(f_mul(f_mul(rx, K), q), d));
                    ay = f_add(ay, f_div(f_mul(f_mul(ry, K), q), d));
                    az = f_add(az, f_div(f_mul(f_mul(rz, K), q), d));
                } else {
                    const T s = f_div(f_mul(K, q), d);
                    ax = f_add(ax, f_mul(rx, s));
                    ay = f_add(ay, f_mul(ry, s));
                    az = f_add(az, f_mul(rz, s));
                }
            }
        }
    }
    if (own) {
        if (ARITH == ARITH_FAST) {
            ax = f_mul(ax, K);
            ay = f_mul(ay, K);
            az = f_mul(az, K);
        }
        ex[i] = ax;
        ey[i] = ay;
        ez[i] = az;
    }
}

} // namespace

template <class T>
cudaError_t launch_field(const T *px, const T *py, const T *pz, long long m, const T *charges,
                         int p, int arith, int three_arg, T *ex, T *ey, T *ez,
                         cudaStream_t stream)
{
    if (m <= 0)
        return cudaSuccess;
    const unsigned grid = (unsigned)((m + 255) / 256);
    if (arith == ARITH_EXACT)
        field_kernel<T, ARITH_EXACT>
            <<<grid, 256, 0, stream>>>(px, py, pz, m, charges, p, three_arg, ex, ey, ez);
    else
        field_kernel<T, ARITH_FAST>
            <<<grid, 256, 0, stream>>>(px, py, pz, m, charges, p, three_arg, ex, ey, ez);
    count_launch(1);
    return cudaGetLastError();
}

template cudaError_t launch_field<float>(const float *, const float *, const float *,
                                         long long, const float *, int, int, int, float *,
                                         float *, float *, cudaStream_t);
template cudaError_t launch_field<double>(const double *, const double *, const double *,
                                          long long, const double *, int, int, int,
                                          double *, double *, double *, cudaStream_t);

} // namespace em
