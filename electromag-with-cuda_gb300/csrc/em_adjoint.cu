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
// The backward needs E'_s at every vertex.  Either the forward stores it
// (12 B per vertex), or only the vertices are kept (the line state at every
// row, which the forward writes anyway) and the field is recomputed per
// segment of 64 rows, walking the segments from the end; the recompute
// repeats the forward's lane order, so it gives the same bits and the same
// lam_s.
//
// Fused backward (p <= kAdjFusedMaxCharges).  The pair term G(r_sj) mu_s
// feeds both sums: over charges for the line's a_s, over rows and lines for
// charge j's gradient.  A team of W warps takes one line at a time and walks
// its rows backwards; lane l of warp w owns charges k*32W + 32w + l (k < CPL)
// and keeps their four gradient sums in registers across all the rows and
// lines it processes, flushing them every 512 rows into compensated (hi, lo)
// partials of its team.  Each pair is formed once (23 FP32 ops + one rsqrt)
// instead of twice.  Per block of 32 rows, lane l prepares row (top - l):
// u, lam/|E'|, the vertex and 2 (v - t); each row then takes them from that
// lane by shuffle.
//
// Two-pass backward (larger p, up to the shared-memory limit): per segment,
// adj_line_kernel (TPL lanes per line, charges resident in shared memory)
// recomputes E at each stored vertex, forms mu, runs the Jacobian-vector
// pair loop and writes (v_s, mu_s) records; adj_charge_kernel then keeps a
// few charges per thread in registers and streams the segment's records
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

// Loss sum |v - t|^2 over all vertices: each vertex's term in FP32 (within
// about 3e-7 of its exact value; the terms are positive, so the sum keeps
// that relative bound), summed in FP64 (GB300 runs FP64 at 1/64 of the FP32
// rate, so one FP64 add per vertex keeps the kernel at memory speed).  One
// FP64 partial per CTA (part), summed in a fixed order by
// adj_loss_sum_kernel, so the loss repeats bit for bit.
__global__ void __launch_bounds__(256) adj_loss_kernel(const float *x, const float *y,
                                                       const float *z, const float *tx,
                                                       const float *ty, const float *tz,
                                                       size_t elems, double *part)
{
    double acc = 0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < elems;
         i += (size_t)gridDim.x * blockDim.x) {
        const float dx = x[i] - tx[i], dy = y[i] - ty[i], dz = z[i] - tz[i];
        acc += (double)fmaf(dz, dz, fmaf(dy, dy, dx * dx));
    }
    for (int o = 16; o; o >>= 1)
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
    __shared__ double wpart[8];
    if ((threadIdx.x & 31) == 0)
        wpart[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            s += wpart[w];
        part[blockIdx.x] = s;
    }
}

// One warp: lane l sums partials l, l + 32, ... in order, then a fixed
// butterfly.
__global__ void adj_loss_sum_kernel(const double *part, int n, double *loss)
{
    double s = 0;
    for (int i = threadIdx.x; i < n; i += 32)
        s += part[i];
    for (int o = 16; o; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0)
        *loss = s;
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

// One lane's chain of the forward's TPL = 8 charge split: charges t8,
// t8 + 8, ... summed in order into a zero start, for PPT vertices at once
// (each broadcast charge load feeds PPT pairs).  The pair is the forward's
// fast form (ref_trace_kernel, ARITH_FAST).
template <int PPT>
__device__ __forceinline__ void lane_chain(const float4 *tiles, int p_pad, int t8,
                                           const float (&px)[PPT], const float (&py)[PPT],
                                           const float (&pz)[PPT], float (&a)[PPT][3])
{
#pragma unroll
    for (int k = 0; k < PPT; ++k)
        a[k][0] = a[k][1] = a[k][2] = 0.0f;
#pragma unroll 4
    for (int j = t8; j < p_pad; j += 8) {
        const float4 c = tiles[j];
#pragma unroll
        for (int k = 0; k < PPT; ++k) {
            const float dx = px[k] - c.x, dy = py[k] - c.y, dz = pz[k] - c.z;
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float inv = rsqrt_fast(r2);
            const float sc = (c.w * inv) * (inv * inv);
            a[k][0] = fmaf(sc, dx, a[k][0]);
            a[k][1] = fmaf(sc, dy, a[k][1]);
            a[k][2] = fmaf(sc, dz, a[k][2]);
        }
    }
}

template <int PPT>
__device__ __forceinline__ void add_into(float (&a)[PPT][3], const float (&b)[PPT][3])
{
#pragma unroll
    for (int k = 0; k < PPT; ++k)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            a[k][c] = a[k][c] + b[k][c];
}

// E' at PPT vertices (flat element indices e[k]; ok[k] false for none):
// the eight lane sums of the forward, combined as its xor butterfly over
// offsets 4, 2, 1 gives them, ((a0+a4) + (a2+a6)) + ((a1+a5) + (a3+a7))
// (float addition commutes, so every lane of the butterfly holds these
// bits).  Chains run in the order 0, 4, 2, 6, 1, 5, 3, 7 so at most four
// partial sums are live.
template <int PPT>
__device__ __forceinline__ void points_field(const AdjParams &P, const float4 *tiles,
                                             const size_t (&e)[PPT], const bool (&ok)[PPT],
                                             size_t out_shift)
{
    float px[PPT], py[PPT], pz[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        px[k] = ok[k] ? P.x[e[k]] : 0.0f;
        py[k] = ok[k] ? P.y[e[k]] : 0.0f;
        pz[k] = ok[k] ? P.z[e[k]] : 0.0f;
    }
    float A[PPT][3], B[PPT][3], C[PPT][3], D[PPT][3];
    lane_chain<PPT>(tiles, P.p_pad, 0, px, py, pz, A);
    lane_chain<PPT>(tiles, P.p_pad, 4, px, py, pz, B);
    add_into<PPT>(A, B); // a0 + a4
    lane_chain<PPT>(tiles, P.p_pad, 2, px, py, pz, B);
    lane_chain<PPT>(tiles, P.p_pad, 6, px, py, pz, C);
    add_into<PPT>(B, C); // a2 + a6
    add_into<PPT>(A, B);
    lane_chain<PPT>(tiles, P.p_pad, 1, px, py, pz, B);
    lane_chain<PPT>(tiles, P.p_pad, 5, px, py, pz, C);
    add_into<PPT>(B, C); // a1 + a5
    lane_chain<PPT>(tiles, P.p_pad, 3, px, py, pz, C);
    lane_chain<PPT>(tiles, P.p_pad, 7, px, py, pz, D);
    add_into<PPT>(C, D); // a3 + a7
    add_into<PPT>(B, C);
    add_into<PPT>(A, B);
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        if (ok[k]) {
            const size_t o = e[k] - out_shift;
            P.fx[o] = A[k][0];
            P.fy[o] = A[k][1];
            P.fz[o] = A[k][2];
        }
    }
}

// E' = E/K at the stored vertices of rows [s_lo, s_hi), written at row
// (s - f_row0), with the bits of the forward's TPL = 8 sums (points_field).
// Vertex-parallel: the rows' vertices are one contiguous run of the line
// arrays; thread i of T takes elements i, i + T, ... in groups of
// kFieldPts (one broadcast charge load per kFieldPts pairs), then one at a
// time, so every thread's share differs by at most one vertex.
constexpr int kFieldPts = 3;
constexpr int kFieldThreads = 256;

__global__ void __launch_bounds__(kFieldThreads, 3) adj_field_kernel(const AdjParams P, int s_lo,
                                                                  int s_hi)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    const float4 *tiles = reinterpret_cast<const float4 *>(smem + 128);
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
            bulk_g2s(smem_addr(smem + 128) + off, src + off, bytes - off < CH ? bytes - off : CH,
                     b0);
    }
    if (!mbar_wait(b0, 0, P.err))
        return;
    const size_t n = (size_t)P.n;
    const size_t first = (size_t)s_lo * n, last = (size_t)s_hi * n;
    const size_t shift = (size_t)P.f_row0 * n;
    const size_t T = (size_t)gridDim.x * blockDim.x;
    size_t i = first + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (kFieldPts - 1) * T < last; i += kFieldPts * T) {
        size_t e[kFieldPts];
        bool ok[kFieldPts];
#pragma unroll
        for (int k = 0; k < kFieldPts; ++k) {
            e[k] = i + k * T;
            ok[k] = true;
        }
        points_field<kFieldPts>(P, tiles, e, ok, shift);
    }
    for (; i < last; i += T) {
        const size_t e[1] = {i};
        const bool ok[1] = {true};
        points_field<1>(P, tiles, e, ok, shift);
    }
}

// warp index within its team of W warps
__device__ __forceinline__ int wt_of(unsigned tid, int W) { return (int)(tid >> 5) % W; }

__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// Adds a lane's register sums into its team's compensated partials and
// clears them; lane l of warp wt owns records (k*W + wt)*32 + l, its sums
// held as packed pairs (k = 2kp in the low half, 2kp + 1 in the high half).
template <int CPL, int W>
__device__ __forceinline__ void adj_flush(const AdjParams &P, long long team, int wt, int lane,
                                          u64 (&g)[4][CPL / 2])
{
    constexpr int PB = 32 * W * CPL;
    float2 *tp = P.tpart + (size_t)team * 4 * PB + wt * 32 + lane;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
#pragma unroll
        for (int kp = 0; kp < CPL / 2; ++kp) {
            float gv[2];
            f2_unpack(g[c][kp], gv[0], gv[1]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float2 *q = tp + c * PB + (2 * kp + h) * W * 32;
                float2 v = *q;
                float sum, err;
                two_sum_f(v.x, gv[h], sum, err);
                v.x = sum;
                v.y = __fadd_rn(v.y, err);
                *q = v;
            }
            g[c][kp] = 0ull;
        }
    }
}

// The fused backward's records in lane pairs: slot (kp*W + wt)*32 + l of
// the A plane holds {x, x', y, y'} and of the B plane {z, z', q, q'} for the
// lane's charges k = 2kp and 2kp + 1 (plain records (k*W + wt)*32 + l), so
// each pair of them feeds one packed instruction.
__global__ void adj_pair_stage_kernel(const float4 *plain, int p_bwd, int W, float4 *paired)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int half = p_bwd / 2;
    if (i >= half)
        return;
    const int l = i & 31, rest = i >> 5;
    const int kp = rest / W, wt = rest - kp * W;
    const float4 a = plain[((2 * kp) * W + wt) * 32 + l];
    const float4 b = plain[((2 * kp + 1) * W + wt) * 32 + l];
    paired[i] = make_float4(a.x, b.x, a.y, b.y);
    paired[half + i] = make_float4(a.z, b.z, a.w, b.w);
}

// Fused backward over rows [s_lo, s_hi) of every line (see the file
// comment).  blockDim = 128 (4 warps); teams of W warps.  CPL and W are
// compile-time so every shared-memory and partial-sum offset is an
// immediate.
template <int CPL, int W>
__global__ void __launch_bounds__(128, CPL >= 32 ? 2 : 3) adj_fused_kernel(const AdjParams P,
                                                                          int s_lo, int s_hi)
{
    constexpr int kFlushRows = 512;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float4 *red = reinterpret_cast<float4 *>(smem + 128); // [2 parities][4 warps]
    // the lane's charge pairs: A plane {x, x', y, y'}, B plane {z, z', q, q'}
    const ulonglong2 *chA = reinterpret_cast<const ulonglong2 *>(smem + 256) +
                            wt_of(threadIdx.x, W) * 32 + (threadIdx.x & 31);
    const ulonglong2 *chB = chA + 16 * W * CPL;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tpc = (int)(blockDim.x >> 5) / W;
    const int team = warp / W, wt = warp - team * W;
    const uint32_t b0 = smem_addr(bar);
    if (threadIdx.x == 0) {
        mbar_init(b0, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)P.p_bwd * 16u;
        mbar_arrive_expect_tx(b0, bytes);
        const char *src = static_cast<const char *>(P.charges_bwd);
        constexpr uint32_t CHUNK = 32768;
        const uint32_t dst = smem_addr(smem + 256);
        for (uint32_t off = 0; off < bytes; off += CHUNK)
            bulk_g2s(dst + off, src + off, bytes - off < CHUNK ? bytes - off : CHUNK, b0);
    }
    // every warp leaves together if the copy did not land (a team's warps
    // meet at named barriers later, which must never miss a member)
    const bool staged = mbar_wait(b0, 0, P.err);
    if (__syncthreads_or(!staged) || team >= tpc)
        return;
    const long long tid = (long long)blockIdx.x * tpc + team;
    const long long nteams = (long long)gridDim.x * tpc;
    const size_t n = (size_t)P.n;
    const float K = (float)kElectroK;
    const unsigned FULL = 0xffffffffu;

    // x, y, z gradient sums and -3 sum r.mu/r^3 per owned charge, in pairs
    u64 g[4][CPL / 2];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int kp = 0; kp < CPL / 2; ++kp)
            g[c][kp] = 0ull;
    int acc_rows = 0;

    for (long long line = tid; line < P.n; line += nteams) {
        float ax = P.abar[line], ay = P.abar[n + line], az = P.abar[2 * n + line];
        const float p0x = P.x[line], p0y = P.y[line], p0z = P.z[line];
        for (int bh = s_hi; bh > s_lo; bh -= 32) {
            const int bl = max(s_lo, bh - 32);
            // lane l prepares row bh - 1 - l
            float pux = 0, puy = 0, puz = 0, pf = 0;
            float pvx = 0, pvy = 0, pvz = 0, pgx = 0, pgy = 0, pgz = 0;
            const int sl = bh - 1 - lane;
            if (sl >= bl) {
                const size_t i = (size_t)sl * n + (size_t)line;
                pvx = P.x[i];
                pvy = P.y[i];
                pvz = P.z[i];
                pgx = 2.0f * (pvx - P.tx[i]);
                pgy = 2.0f * (pvy - P.ty[i]);
                pgz = 2.0f * (pvz - P.tz[i]);
                const size_t fi = (size_t)(sl - P.f_row0) * n + (size_t)line;
                const float ex = P.fx[fi], ey = P.fy[fi], ez = P.fz[fi];
                // lam_s from E = K E' (the forward's IEEE step sequence)
                const float Ex = mul_rn(ex, K), Ey = mul_rn(ey, K), Ez = mul_rn(ez, K);
                const float k2 =
                    add_rn(add_rn(mul_rn(Ex, Ex), mul_rn(Ey, Ey)), mul_rn(Ez, Ez));
                float lam = 1.0f / P.resolution;
                if (P.curvature) {
                    const float ix = sub_rn(Ex, p0x), iy = sub_rn(Ey, p0y), iz = sub_rn(Ez, p0z);
                    const float cx = sub_rn(mul_rn(iy, p0z), mul_rn(iz, p0y));
                    const float cy = sub_rn(mul_rn(iz, p0x), mul_rn(ix, p0z));
                    const float cz = sub_rn(mul_rn(ix, p0y), mul_rn(iy, p0x));
                    const float c2 =
                        add_rn(add_rn(mul_rn(cx, cx), mul_rn(cy, cy)), mul_rn(cz, cz));
                    const float kc = div_rn(sqrt_rn(c2), mul_rn(k2, sqrt_rn(k2)));
                    lam = 1.0f / mul_rn(add_rn(kc, 1.0f), P.resolution);
                }
                const float en = sqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex)));
                const float ien = 1.0f / en;
                pux = ex * ien;
                puy = ey * ien;
                puz = ez * ien;
                pf = lam * ien;
            }
            for (int s = bh - 1; s >= bl; --s) {
                const int src = bh - 1 - s;
                const float ux = __shfl_sync(FULL, pux, src), uy = __shfl_sync(FULL, puy, src),
                            uz = __shfl_sync(FULL, puz, src), f = __shfl_sync(FULL, pf, src);
                const float vx = __shfl_sync(FULL, pvx, src), vy = __shfl_sync(FULL, pvy, src),
                            vz = __shfl_sync(FULL, pvz, src);
                const float gxs = __shfl_sync(FULL, pgx, src), gys = __shfl_sync(FULL, pgy, src),
                            gzs = __shfl_sync(FULL, pgz, src);
                // mu' = lam (a - u (u.a)) / |E'|
                const float ua = fmaf(uz, az, fmaf(uy, ay, ux * ax));
                const float mx = f * fmaf(-ux, ua, ax), my = f * fmaf(-uy, ua, ay),
                            mz = f * fmaf(-uz, ua, az);
                const float m3x = -3.0f * mx, m3y = -3.0f * my, m3z = -3.0f * mz;
                // G(r) mu = inv3 h, h = mu + (d3 inv2) r with d3 = -3 r.mu:
                // h feeds the charge's position sums and, times q inv3, the
                // line's Jacobian-vector sum l; two charges per packed
                // instruction
                const u64 VX = f2_pack(vx, vx), VY = f2_pack(vy, vy), VZ = f2_pack(vz, vz);
                const u64 MX = f2_pack(mx, mx), MY = f2_pack(my, my), MZ = f2_pack(mz, mz);
                const u64 NX = f2_pack(m3x, m3x), NY = f2_pack(m3y, m3y),
                          NZ = f2_pack(m3z, m3z);
                u64 LX = 0ull, LY = 0ull, LZ = 0ull;
#pragma unroll
                for (int kp = 0; kp < CPL / 2; ++kp) {
                    const ulonglong2 A = chA[kp * W * 32], B = chB[kp * W * 32];
                    const u64 dx = f2_sub(VX, A.x), dy = f2_sub(VY, A.y), dz = f2_sub(VZ, B.x);
                    const u64 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
                    const u64 inv = f2_rsqrt(r2);
                    const u64 inv2 = f2_mul(inv, inv);
                    const u64 inv3 = f2_mul(inv2, inv);
                    const u64 d3 = f2_fma(dz, NZ, f2_fma(dy, NY, f2_mul(dx, NX)));
                    const u64 t = f2_mul(d3, inv2);
                    const u64 hx = f2_fma(t, dx, MX), hy = f2_fma(t, dy, MY),
                              hz = f2_fma(t, dz, MZ);
                    g[0][kp] = f2_fma(inv3, hx, g[0][kp]);
                    g[1][kp] = f2_fma(inv3, hy, g[1][kp]);
                    g[2][kp] = f2_fma(inv3, hz, g[2][kp]);
                    g[3][kp] = f2_fma(d3, inv3, g[3][kp]);
                    const u64 qi3 = f2_mul(B.y, inv3);
                    LX = f2_fma(qi3, hx, LX);
                    LY = f2_fma(qi3, hy, LY);
                    LZ = f2_fma(qi3, hz, LZ);
                }
                float lx, ly, lz;
                {
                    float a, b;
                    f2_unpack(LX, a, b);
                    lx = a + b;
                    f2_unpack(LY, a, b);
                    ly = a + b;
                    f2_unpack(LZ, a, b);
                    lz = a + b;
                }
                // warp sums of (lx, ly, lz): halve the values a lane carries
                // at offsets 16 and 8 (each lane sends the half its partner
                // keeps; the fourth slot is empty), finish with three full
                // levels, so lane 8i holds sum i; then broadcast
                {
                    const bool b16 = lane & 16, b8 = lane & 8;
                    float k0 = b16 ? lz : lx, k1 = b16 ? 0.0f : ly;
                    const float d0 = b16 ? lx : lz, d1 = b16 ? ly : 0.0f;
                    k0 += __shfl_xor_sync(FULL, d0, 16);
                    k1 += __shfl_xor_sync(FULL, d1, 16);
                    float k = b8 ? k1 : k0;
                    k += __shfl_xor_sync(FULL, b8 ? k0 : k1, 8);
                    k += __shfl_xor_sync(FULL, k, 4);
                    k += __shfl_xor_sync(FULL, k, 2);
                    k += __shfl_xor_sync(FULL, k, 1);
                    lx = __shfl_sync(FULL, k, 0);
                    ly = __shfl_sync(FULL, k, 8);
                    lz = __shfl_sync(FULL, k, 16);
                }
                if (W > 1) {
                    // team sum in warp order, identical in every warp; slots
                    // alternate by row parity so one barrier per row suffices
                    float4 *slot = red + (s & 1) * 4;
                    if (lane == 0)
                        slot[warp] = make_float4(lx, ly, lz, 0.0f);
                    asm volatile("bar.sync %0, %1;" ::"r"(1 + team), "r"(32 * W) : "memory");
                    lx = ly = lz = 0;
                    for (int w = 0; w < W; ++w) {
                        const float4 v = slot[team * W + w];
                        lx += v.x;
                        ly += v.y;
                        lz += v.z;
                    }
                }
                ax = (gxs + ax) + lx;
                ay = (gys + ay) + ly;
                az = (gzs + az) + lz;
            }
            acc_rows += bh - bl;
            if (acc_rows >= kFlushRows) {
                adj_flush<CPL, W>(P, tid, wt, lane, g);
                acc_rows = 0;
            }
        }
        if (wt == 0 && lane == 0) {
            P.abar[line] = ax;
            P.abar[n + line] = ay;
            P.abar[2 * n + line] = az;
        }
    }
    if (acc_rows > 0)
        adj_flush<CPL, W>(P, tid, wt, lane, g);
}

// Sums the fused kernel's team partials over one slice of teams into FP64
// (gpart[slice], the layout adj_finish_kernel reads); the fourth sum holds
// -3 sum r.mu/r^3 and is scaled back here.
__global__ void __launch_bounds__(256) adj_team_sum_kernel(const AdjParams P)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P.p)
        return;
    const long long per = (P.teams + gridDim.y - 1) / gridDim.y;
    const long long t0 = blockIdx.y * per, t1 = min(P.teams, t0 + per);
    double acc[4] = {0, 0, 0, 0};
    for (long long t = t0; t < t1; ++t) {
        const float2 *tp = P.tpart + (size_t)t * 4 * (size_t)P.p_bwd + j;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const float2 v = tp[(size_t)c * P.p_bwd];
            acc[c] += (double)v.x + (double)v.y;
        }
    }
    double *out = P.gpart + ((size_t)blockIdx.y * P.p + j) * 4;
    out[0] = acc[0];
    out[1] = acc[1];
    out[2] = acc[2];
    out[3] = acc[3] * (-1.0 / 3.0);
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

int adjoint_loss_parts(int nsm) { return nsm * 4; }

int adjoint_charge_blocks(int p)
{
    return (p + kChargeThreads * kChargesPerThread - 1) / (kChargeThreads * kChargesPerThread);
}

namespace {

void *fused_kernel(int cpl, int w)
{
    switch (cpl) {
    case 4: return (void *)adj_fused_kernel<4, 1>;
    case 8: return (void *)adj_fused_kernel<8, 1>;
    case 16: return (void *)adj_fused_kernel<16, 1>;
    default:
        return w == 4 ? (void *)adj_fused_kernel<32, 4>
                      : w == 2 ? (void *)adj_fused_kernel<32, 2> : (void *)adj_fused_kernel<32, 1>;
    }
}

} // namespace

int adjoint_fused_plan(int p, int nsm, AdjFused *f)
{
    if (p < 1 || p > kAdjFusedMaxCharges)
        return 0;
    int cpl = 32, w = 1;
    if (p <= 128)
        cpl = 4;
    else if (p <= 256)
        cpl = 8;
    else if (p <= 512)
        cpl = 16;
    else
        w = (p + 1023) / 1024; // 1, 2 or 4 warps per line
    if (w == 3)
        w = 4;
    f->cpl = cpl;
    f->team_warps = w;
    f->p_bwd = 32 * w * cpl;
    f->smem = 256 + (size_t)f->p_bwd * 16;
    void *k = fused_kernel(cpl, w);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)f->smem) !=
        cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, f->smem) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return 0;
    }
    f->grid = nsm * per_sm;
    f->teams = (long long)f->grid * (4 / w);
    return 1;
}

namespace {

cudaError_t launch_fused(const AdjParams &P, const AdjFused &f, int lo, int hi,
                         cudaStream_t stream)
{
    const dim3 grid((unsigned)f.grid);
    switch (f.cpl * 8 + f.team_warps) {
    case 4 * 8 + 1: adj_fused_kernel<4, 1><<<grid, 128, f.smem, stream>>>(P, lo, hi); break;
    case 8 * 8 + 1: adj_fused_kernel<8, 1><<<grid, 128, f.smem, stream>>>(P, lo, hi); break;
    case 16 * 8 + 1: adj_fused_kernel<16, 1><<<grid, 128, f.smem, stream>>>(P, lo, hi); break;
    case 32 * 8 + 1: adj_fused_kernel<32, 1><<<grid, 128, f.smem, stream>>>(P, lo, hi); break;
    case 32 * 8 + 2: adj_fused_kernel<32, 2><<<grid, 128, f.smem, stream>>>(P, lo, hi); break;
    case 32 * 8 + 4: adj_fused_kernel<32, 4><<<grid, 128, f.smem, stream>>>(P, lo, hi); break;
    default: return cudaErrorInvalidValue;
    }
    count_launch(1);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_adjoint_pair_stage(const void *plain, int p_bwd, int team_warps,
                                      void *paired, cudaStream_t stream)
{
    const int half = p_bwd / 2;
    if (half <= 0)
        return cudaErrorInvalidValue;
    adj_pair_stage_kernel<<<(half + 255) / 256, 256, 0, stream>>>(
        static_cast<const float4 *>(plain), p_bwd, team_warps, static_cast<float4 *>(paired));
    count_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_backward(const AdjParams &P, const AdjFused *fused, int nsm,
                                    size_t smem, double *loss, double *grad,
                                    cudaStream_t stream, cudaStream_t side, size_t half_elems)
{
    cudaError_t e = cudaFuncSetAttribute(adj_line_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(adj_field_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
    if (e != cudaSuccess)
        return e;
    const size_t elems = (size_t)P.n * (size_t)P.rows;
    // loss[1 .. adjoint_loss_parts(nsm)] hold the per-CTA partials
    adj_loss_kernel<<<nsm * 4, 256, 0, stream>>>(P.x, P.y, P.z, P.tx, P.ty, P.tz, elems,
                                                 loss + 1);
    adj_loss_sum_kernel<<<1, 32, 0, stream>>>(loss + 1, nsm * 4, loss);
    adj_init_kernel<<<(unsigned)((P.n + 255) / 256), 256, 0, stream>>>(P);
    count_launch(3);
    const int seg = P.seg;
    int field_grid = nsm;
    if (fused && !P.stored) {
        int per_sm = 0;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adj_field_kernel,
                                                               kFieldThreads, smem)) !=
            cudaSuccess)
            return e;
        field_grid = nsm * (per_sm > 0 ? per_sm : 1);
    }
    if (fused) {
        if (P.stored) {
            if ((e = launch_fused(P, *fused, 0, P.rows - 1, stream)) != cudaSuccess)
                return e;
        } else {
            // the recompute of the next segment overlaps the fused kernel of
            // this one (each fills the SMs the other's last CTAs leave);
            // buffer half k % 2, reused once the fused kernel of segment
            // k - 2 has read it
            cudaEvent_t ev[5] = {};
            for (int k = 0; k < 5 && e == cudaSuccess; ++k)
                e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
            cudaEvent_t *field_done = ev, *fused_done = ev + 2, start = ev[4];
            if (e == cudaSuccess)
                e = cudaEventRecord(start, stream); // forward, loss and init are in
            if (e == cudaSuccess)
                e = cudaStreamWaitEvent(side, start, 0);
            int k = 0;
            for (int hi = P.rows - 1; hi > 0 && e == cudaSuccess; hi -= seg, ++k) {
                const int lo = std::max(0, hi - seg), h = k & 1;
                AdjParams Q = P;
                Q.f_row0 = lo;
                Q.fx = P.fx + h * half_elems;
                Q.fy = P.fy + h * half_elems;
                Q.fz = P.fz + h * half_elems;
                if (k >= 2)
                    e = cudaStreamWaitEvent(side, fused_done[h], 0);
                if (e != cudaSuccess)
                    break;
                adj_field_kernel<<<field_grid, kFieldThreads, smem, side>>>(Q, lo, hi);
                count_launch(1);
                e = cudaGetLastError();
                if (e == cudaSuccess)
                    e = cudaEventRecord(field_done[h], side);
                if (e == cudaSuccess)
                    e = cudaStreamWaitEvent(stream, field_done[h], 0);
                if (e == cudaSuccess)
                    e = launch_fused(Q, *fused, lo, hi, stream);
                if (e == cudaSuccess)
                    e = cudaEventRecord(fused_done[h], stream);
            }
            for (int j = 0; j < 5; ++j)
                if (ev[j])
                    cudaEventDestroy(ev[j]);
            if (e != cudaSuccess)
                return e;
        }
        const dim3 sgrid((unsigned)((P.p + 255) / 256), (unsigned)P.slices);
        adj_team_sum_kernel<<<sgrid, 256, 0, stream>>>(P);
        count_launch(1);
    } else {
        const dim3 cgrid((unsigned)adjoint_charge_blocks(P.p), (unsigned)P.slices);
        for (int hi = P.rows - 1; hi > 0; hi -= seg) {
            const int lo = std::max(0, hi - seg);
            adj_line_kernel<<<nsm, 1024, smem, stream>>>(P, lo, hi);
            adj_charge_kernel<<<cgrid, kChargeThreads, 0, stream>>>(P, (long long)(hi - lo) * P.n);
            count_launch(2);
            if ((e = cudaGetLastError()) != cudaSuccess)
                return e;
        }
    }
    adj_finish_kernel<<<(P.p + 127) / 128, 128, 0, stream>>>(P, grad);
    count_launch(1);
    return cudaGetLastError();
}

} // namespace em
