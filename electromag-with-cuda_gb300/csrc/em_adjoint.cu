// Adjoint of the discrete stepping map with frozen step lengths.
//
// Forward map (the reference rule, CPU_Implement.cpp:322-338, curvature
// against the seed): v_{s+1} = v_s + lam_s u_s, u_s = E_s/|E_s|,
// lam_s = 1/((k_s+1) res) held constant.  Loss L = sum |v_s - t_s|^2 over all
// vertices.  With E' = E/K = sum_j q_j r/|r|^3 and r = v - c_j:
//   a_{S-1} = 2 (v_{S-1} - t_{S-1})
//   mu_s    = lam_s (a_{s+1} - u_s (u_s . a_{s+1})) / |E'_s|
//   a_s     = 2 (v_s - t_s) + a_{s+1} + sum_j q_j G(r) mu_s
//   dL/dc_j = -q_j sum_s G(r_sj) mu_s,   dL/dq_j = sum_s r_sj . mu_s / |r_sj|^3
//   G(r) mu = mu/|r|^3 - 3 r (r . mu)/|r|^5            (K cancels throughout)
//
// Schedule: the forward writes every vertex (the caller's output).  The
// backward walks segments of P.seg rows (64: the line-state checkpoint
// interval) from the end.  Per segment,
// adj_line_kernel (TPL lanes per line, charges resident in shared memory)
// recomputes E at each stored vertex (the same lane order as the forward, so
// the same bits and the same lam), forms mu, runs the Jacobian-vector pair
// loop and writes (v_s, mu_s) records; adj_charge_kernel then keeps a few
// charges per thread in registers and streams the segment's records
// (L2-resident) to accumulate the charge gradients into FP64 partial sums,
// one per (slice of records, charge), summed at the end.
#include "em_device.cuh"
#include "em_internal.h"
#include "em_math.cuh"

#include <algorithm>

namespace em {
namespace {

constexpr int kAdjTpl = 8;      // lanes per line (matches the forward's order)
constexpr int kChargesPerThread = 2;
constexpr int kChargeThreads = 256;
constexpr int kRecChunk = 256;  // records staged per chunk in the charge pass

template <int TPL>
__device__ __forceinline__ float lane_sum(float v)
{
#pragma unroll
    for (int o = TPL / 2; o >= 1; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Loss sum (v - t)^2 over all vertices, FP64 partials, one atomic per CTA.
__global__ void __launch_bounds__(256) adj_loss_kernel(const float *x, const float *y,
                                                       const float *z, const float *tx,
                                                       const float *ty, const float *tz,
                                                       size_t elems, double *loss)
{
    double acc = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < elems;
         i += (size_t)gridDim.x * blockDim.x) {
        const double dx = (double)x[i] - tx[i], dy = (double)y[i] - ty[i],
                     dz = (double)z[i] - tz[i];
        acc += dx * dx + dy * dy + dz * dz;
    }
    for (int o = 16; o; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double part[8];
    if ((threadIdx.x & 31) == 0)
        part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            s += part[w];
        atomicAdd(loss, s);
    }
}

// Backward over rows [s_lo, s_hi) of one segment for every line.
__global__ void __launch_bounds__(1024, 1) adj_line_kernel(const AdjParams P, int s_lo, int s_hi)
{
    constexpr int TPL = kAdjTpl, LG = 32 / TPL;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float4 *tiles = reinterpret_cast<float4 *>(smem + 128);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, t = lane % TPL;
    const uint32_t b0 = smem_addr(bar);
    if (threadIdx.x == 0) {
        mbar_init(b0, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)P.p_pad * 16u;
        mbar_arrive_expect_tx(b0, bytes);
        const char *src = static_cast<const char *>(P.charges);
        constexpr uint32_t CH = 32768;
        for (uint32_t off = 0; off < bytes; off += CH)
            bulk_g2s(smem_addr(tiles) + off, src + off, bytes - off < CH ? bytes - off : CH, b0);
    }
    if (!mbar_wait(b0, 0, P.err))
        return;
    const size_t n = (size_t)P.n;
    const float K = (float)kElectroK;
    const long long groups = (P.n + LG - 1) / LG;
    const int nw = blockDim.x >> 5;
    for (long long g = blockIdx.x + (long long)gridDim.x * warp; g < groups;
         g += (long long)gridDim.x * nw) {
        const long long line = g * LG + lane / TPL;
        const bool own = line < P.n;
        const long long l = own ? line : 0;
        float ax = P.abar[l], ay = P.abar[n + l], az = P.abar[2 * n + l];
        const float p0x = P.x[l], p0y = P.y[l], p0z = P.z[l];
        for (int s = s_hi - 1; s >= s_lo; --s) {
            const size_t i = (size_t)s * n + l;
            const float vx = P.x[i], vy = P.y[i], vz = P.z[i];
            // E' at v_s: the forward's pair loop and lane order
            float ex = 0, ey = 0, ez = 0;
#pragma unroll 8
            for (int j = t; j < P.p_pad; j += TPL) {
                const float4 c = tiles[j];
                const float dx = vx - c.x, dy = vy - c.y, dz = vz - c.z;
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float inv = rsqrt_fast(r2);
                const float sc = (c.w * inv) * (inv * inv);
                ex = fmaf(sc, dx, ex);
                ey = fmaf(sc, dy, ey);
                ez = fmaf(sc, dz, ez);
            }
            ex = lane_sum<TPL>(ex);
            ey = lane_sum<TPL>(ey);
            ez = lane_sum<TPL>(ez);
            // lam_s from E = K E' (the forward's IEEE step sequence)
            const float Ex = mul_rn(ex, K), Ey = mul_rn(ey, K), Ez = mul_rn(ez, K);
            const float k2 = add_rn(add_rn(mul_rn(Ex, Ex), mul_rn(Ey, Ey)), mul_rn(Ez, Ez));
            float lam = 1.0f / P.resolution;
            if (P.curvature) {
                const float ix = sub_rn(Ex, p0x), iy = sub_rn(Ey, p0y), iz = sub_rn(Ez, p0z);
                const float cx = sub_rn(mul_rn(iy, p0z), mul_rn(iz, p0y));
                const float cy = sub_rn(mul_rn(iz, p0x), mul_rn(ix, p0z));
                const float cz = sub_rn(mul_rn(ix, p0y), mul_rn(iy, p0x));
                const float c2 = add_rn(add_rn(mul_rn(cx, cx), mul_rn(cy, cy)), mul_rn(cz, cz));
                const float kc = div_rn(sqrt_rn(c2), mul_rn(k2, sqrt_rn(k2)));
                lam = 1.0f / mul_rn(add_rn(kc, 1.0f), P.resolution);
            }
            // mu' = lam (a - u (u.a)) / |E'|
            const float en = sqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex)));
            const float ien = 1.0f / en;
            const float ux = ex * ien, uy = ey * ien, uz = ez * ien;
            const float ua = fmaf(uz, az, fmaf(uy, ay, ux * ax));
            const float f = lam * ien;
            const float mx = f * fmaf(-ux, ua, ax), my = f * fmaf(-uy, ua, ay),
                        mz = f * fmaf(-uz, ua, az);
            // J mu' = sum q (mu/r^3 - 3 r (r.mu)/r^5) = S1 mu - 3 V
            float s1 = 0, wx = 0, wy = 0, wz = 0;
#pragma unroll 4
            for (int j = t; j < P.p_pad; j += TPL) {
                const float4 c = tiles[j];
                const float dx = vx - c.x, dy = vy - c.y, dz = vz - c.z;
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float inv = rsqrt_fast(r2);
                const float inv2 = inv * inv;
                const float qi3 = (c.w * inv) * inv2;
                const float d = fmaf(dz, mz, fmaf(dy, my, dx * mx));
                s1 += qi3;
                const float c3 = (d * inv2) * qi3;
                wx = fmaf(c3, dx, wx);
                wy = fmaf(c3, dy, wy);
                wz = fmaf(c3, dz, wz);
            }
            s1 = lane_sum<TPL>(s1);
            wx = lane_sum<TPL>(wx);
            wy = lane_sum<TPL>(wy);
            wz = lane_sum<TPL>(wz);
            if (own && t == 0) {
                const size_t r = (size_t)(s - s_lo) * n + (size_t)line;
                const size_t R = P.rec_stride;
                P.rec[r] = vx;
                P.rec[R + r] = vy;
                P.rec[2 * R + r] = vz;
                P.rec[3 * R + r] = mx;
                P.rec[4 * R + r] = my;
                P.rec[5 * R + r] = mz;
            }
            const float tx = P.tx[i], ty = P.ty[i], tz = P.tz[i];
            ax = 2.0f * (vx - tx) + ax + fmaf(s1, mx, -3.0f * wx);
            ay = 2.0f * (vy - ty) + ay + fmaf(s1, my, -3.0f * wy);
            az = 2.0f * (vz - tz) + az + fmaf(s1, mz, -3.0f * wz);
        }
        if (own && t == 0) {
            P.abar[l] = ax;
            P.abar[n + l] = ay;
            P.abar[2 * n + l] = az;
        }
    }
}

// Charge gradients over the records of one segment: each thread keeps
// kChargesPerThread charges; the CTA streams its slice of records through
// shared memory; each (slice, charge) FP64 partial has exactly one owner
// thread, so it is updated without atomics and summed at the end.
__global__ void __launch_bounds__(kChargeThreads) adj_charge_kernel(const AdjParams P,
                                                                   long long nrec)
{
    __shared__ float4 rv[kRecChunk], rm[kRecChunk];
    constexpr int C = kChargesPerThread;
    const int j0 = (blockIdx.x * kChargeThreads + threadIdx.x) * C;
    float cx[C], cy[C], cz[C];
    float gx[C], gy[C], gz[C], h[C];
#pragma unroll
    for (int k = 0; k < C; ++k) {
        const int j = min(j0 + k, P.p - 1);
        cx[k] = P.raw[4 * (size_t)j];
        cy[k] = P.raw[4 * (size_t)j + 1];
        cz[k] = P.raw[4 * (size_t)j + 2];
        gx[k] = gy[k] = gz[k] = h[k] = 0;
    }
    const long long per = (nrec + gridDim.y - 1) / gridDim.y;
    const long long r0 = blockIdx.y * per, r1 = min(nrec, r0 + per);
    const size_t R = P.rec_stride;
    for (long long base = r0; base < r1; base += kRecChunk) {
        const int cnt = (int)min((long long)kRecChunk, r1 - base);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
            const size_t r = (size_t)(base + k);
            rv[k] = make_float4(P.rec[r], P.rec[R + r], P.rec[2 * R + r], 0.f);
            rm[k] = make_float4(P.rec[3 * R + r], P.rec[4 * R + r], P.rec[5 * R + r], 0.f);
        }
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < cnt; ++k) {
            const float4 v = rv[k], m = rm[k];
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const float dx = v.x - cx[c], dy = v.y - cy[c], dz = v.z - cz[c];
                const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                const float inv = rsqrt_fast(r2);
                const float inv2 = inv * inv;
                const float inv3 = inv2 * inv;
                const float d = fmaf(dz, m.z, fmaf(dy, m.y, dx * m.x));
                const float w = -3.0f * ((d * inv2) * inv3);
                gx[c] = fmaf(w, dx, fmaf(inv3, m.x, gx[c]));
                gy[c] = fmaf(w, dy, fmaf(inv3, m.y, gy[c]));
                gz[c] = fmaf(w, dz, fmaf(inv3, m.z, gz[c]));
                h[c] = fmaf(d, inv3, h[c]);
            }
        }
    }
    double *part = P.gpart + (size_t)blockIdx.y * 4 * (size_t)P.p;
#pragma unroll
    for (int k = 0; k < C; ++k) {
        const int j = j0 + k;
        if (j < P.p) {
            part[4 * (size_t)j] += (double)gx[k];
            part[4 * (size_t)j + 1] += (double)gy[k];
            part[4 * (size_t)j + 2] += (double)gz[k];
            part[4 * (size_t)j + 3] += (double)h[k];
        }
    }
}

// a_{S-1} = 2 (v_{S-1} - t_{S-1}); records also for the last row (mu = 0
// is never used: the last row has no outgoing step).
__global__ void adj_init_kernel(const AdjParams P)
{
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (l >= P.n)
        return;
    const size_t n = (size_t)P.n, i = (size_t)(P.rows - 1) * n + l;
    P.abar[l] = 2.0f * (P.x[i] - P.tx[i]);
    P.abar[n + l] = 2.0f * (P.y[i] - P.ty[i]);
    P.abar[2 * n + l] = 2.0f * (P.z[i] - P.tz[i]);
}

// grad = (-q G, H) in FP64, summing the slices' partials
__global__ void adj_finish_kernel(const AdjParams P, double *grad)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P.p)
        return;
    double g[4] = {0, 0, 0, 0};
    for (int y = 0; y < P.slices; ++y)
        for (int c = 0; c < 4; ++c)
            g[c] += P.gpart[((size_t)y * P.p + j) * 4 + c];
    const double q = P.raw[4 * (size_t)j + 3];
    grad[4 * (size_t)j] = -q * g[0];
    grad[4 * (size_t)j + 1] = -q * g[1];
    grad[4 * (size_t)j + 2] = -q * g[2];
    grad[4 * (size_t)j + 3] = g[3];
}

} // namespace

int adjoint_charge_blocks(int p)
{
    return (p + kChargeThreads * kChargesPerThread - 1) / (kChargeThreads * kChargesPerThread);
}

cudaError_t launch_adjoint_backward(const AdjParams &P, int nsm, size_t smem, double *loss,
                                    double *grad, cudaStream_t stream)
{
    cudaError_t e = cudaFuncSetAttribute(adj_line_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    const size_t elems = (size_t)P.n * (size_t)P.rows;
    adj_loss_kernel<<<nsm * 4, 256, 0, stream>>>(P.x, P.y, P.z, P.tx, P.ty, P.tz, elems, loss);
    adj_init_kernel<<<(unsigned)((P.n + 255) / 256), 256, 0, stream>>>(P);
    count_launch(2);
    const int seg = P.seg;
    const dim3 cgrid((unsigned)adjoint_charge_blocks(P.p), (unsigned)P.slices);
    for (int hi = P.rows - 1; hi > 0; hi -= seg) {
        const int lo = std::max(0, hi - seg);
        adj_line_kernel<<<nsm, 1024, smem, stream>>>(P, lo, hi);
        adj_charge_kernel<<<cgrid, kChargeThreads, 0, stream>>>(P, (long long)(hi - lo) * P.n);
        count_launch(2);
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
    }
    adj_finish_kernel<<<(P.p + 127) / 128, 128, 0, stream>>>(P, grad);
    count_launch(1);
    return cudaGetLastError();
}

} // namespace em
