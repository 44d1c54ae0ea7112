// Field-line tracer over the reference's SoA line layout (CalcField_CPU
// semantics, ElectroMag/src/CPU_Implement.cpp:38-527).
//
// Work decomposition.  A warp traces a group of 32/TPL lines for all steps;
// TPL lanes share one line and split its charge sum (lane t takes charges
// t, t+TPL, ...), combining the partial fields with an xor butterfly so every
// lane of the line holds the same bits.  Groups are dealt to CTAs round-robin
// (group g -> CTA g mod grid) so every SM gets the same number of lines.
//
// Charges live in shared memory.  If the padded set fits, one thread stages
// it once with bulk (TMA) copies and the CTA never synchronises again.
// Otherwise a producer warp streams fixed-size tiles through a ring of
// `stages` buffers (full/empty mbarriers); all compute warps consume every
// tile, idle warps only take part in the barrier protocol.
//
// Arithmetic.  ARITH_FAST: r2 by FMA, rsqrtf, s = q*inv^3, a += s*r; the
// Coulomb constant is applied once per vertex.  ARITH_EXACT: the reference's
// operation order with one IEEE rounding per operation (__f*_rn intrinsics,
// no contraction), which reproduces the strict x86 build bit for bit.  The
// per-vertex step (curvature, vec3SetInvLen, include/Vector.h:157-164) uses
// the IEEE sequence in both modes.
#include <algorithm>
#include <type_traits>

#include "em_device.cuh"
#include "em_ext.cuh"
#include "em_internal.h"
#include "em_math.cuh"

namespace em {
namespace {

// One pair, fast form: a += q * r / |r|^3.
template <class T, class C>
__device__ __forceinline__ void pair_fast(T px, T py, T pz, const C &c, T &ax, T &ay, T &az)
{
    const T dx = px - c.x, dy = py - c.y, dz = pz - c.z;
    const T r2 = fma(dz, dz, fma(dy, dy, dx * dx));
    const T inv = rsqrt_fast(r2);
    const T s = (c.q * inv) * (inv * inv);
    ax = fma(s, dx, ax);
    ay = fma(s, dy, ay);
    az = fma(s, dz, az);
}

// One pair, the reference's sequence.  three_arg: PartField(charge, point, k)
// = r*k*q / (r2*sqrt(r2)) (include/Electrostatics.h:38-51, the SSE paths);
// otherwise PartField(charge, point) = r * (k*q / (r2*sqrt(r2))) (:53-60).
template <class T, class C>
__device__ __forceinline__ void pair_exact(T px, T py, T pz, const C &c, T K, bool three_arg,
                                           T &ax, T &ay, T &az)
{
    const T rx = sub_rn(px, c.x), ry = sub_rn(py, c.y), rz = sub_rn(pz, c.z);
    const T l2 = add_rn(add_rn(mul_rn(rx, rx), mul_rn(ry, ry)), mul_rn(rz, rz));
    const T d = mul_rn(l2, sqrt_rn(l2));
    if (three_arg) {
        ax = add_rn(ax, div_rn(mul_rn(mul_rn(rx, K), c.q), d));
        ay = add_rn(ay, div_rn(mul_rn(mul_rn(ry, K), c.q), d));
        az = add_rn(az, div_rn(mul_rn(mul_rn(rz, K), c.q), d));
    } else {
        const T s = div_rn(mul_rn(K, c.q), d);
        ax = add_rn(ax, mul_rn(rx, s));
        ay = add_rn(ay, mul_rn(ry, s));
        az = add_rn(az, mul_rn(rz, s));
    }
}

// The term of pair_exact (FP32), with the branch-free rounded root and
// quotients: the same bits when it returns true (operands inside the checked
// range: r^2 in [2^-40, 2^40] and every numerator in exact_range).
template <class C>
__device__ __forceinline__ bool pair_exact_nb(float px, float py, float pz, const C &c, float K,
                                              bool three_arg, float &tx, float &ty, float &tz)
{
    const float rx = sub_rn(px, c.x), ry = sub_rn(py, c.y), rz = sub_rn(pz, c.z);
    const float l2 = add_rn(add_rn(mul_rn(rx, rx), mul_rn(ry, ry)), mul_rn(rz, rz));
    const float d = mul_rn(l2, sqrt_rn_nb(l2));
    const float y = rcp_rn_nb(d);
    bool ok = l2 >= 0x1p-40f && l2 <= 0x1p40f;
    if (three_arg) {
        const float nx = mul_rn(mul_rn(rx, K), c.q), ny = mul_rn(mul_rn(ry, K), c.q),
                    nz = mul_rn(mul_rn(rz, K), c.q);
        ok = ok && exact_range(nx) && exact_range(ny) && exact_range(nz);
        tx = div_rn_nb(nx, d, y);
        ty = div_rn_nb(ny, d, y);
        tz = div_rn_nb(nz, d, y);
    } else {
        const float n0 = mul_rn(K, c.q);
        ok = ok && exact_range(n0);
        const float s = div_rn_nb(n0, d, y);
        tx = mul_rn(rx, s);
        ty = mul_rn(ry, s);
        tz = mul_rn(rz, s);
    }
    return ok;
}

// Per-line field accumulator: scalar components, plus packed pairs for the
// .f32x2 path (kept across charge tiles so tiling never changes the sum).
template <class T> struct Acc {
    T x = 0, y = 0, z = 0;
    u64 X = 0, Y = 0, Z = 0;
};

// Adds the charges held in shared memory [0, count) to lane t's partial sum.
template <class T, int TPL, int ARITH, class Rec>
__device__ __forceinline__ void accumulate(const Rec *tile, int count, int t, T px, T py, T pz,
                                           T K, bool three_arg, bool nb, float4 *xbuf, Acc<T> &a)
{
    if (ARITH == ARITH_FAST2) {
        // charge pairs t, t+TPL, ... ; count is a multiple of 2*TPL; the tile
        // holds its {xa,xb,ya,yb} plane, then its {za,zb,qa,qb} plane
        const ulonglong2 *tp = reinterpret_cast<const ulonglong2 *>(tile);
        const int G = count / 2;
        const u64 PX = f2_pack(px, px), PY = f2_pack(py, py), PZ = f2_pack(pz, pz);
#pragma unroll 4
        for (int jp = t; jp < G; jp += TPL)
            pair2_fast(PX, PY, PZ, tp[jp], tp[G + jp], a.X, a.Y, a.Z);
    } else if (ARITH == ARITH_FAST) {
#pragma unroll kUnroll
        for (int j = t; j < count; j += TPL)
            pair_fast<T>(px, py, pz, load_charge(tile, j), a.x, a.y, a.z);
    } else if constexpr (sizeof(T) == 4 && TPL > 1) {
        // TPL lanes per line: lane t forms the terms of charges j0 + u TPL + t
        // (eight per lane in flight, from the branch-free rounded operations,
        // redone with the compiler's rounded operations when an operand
        // leaves its checked range); every lane of the line then takes each
        // round's TPL terms in charge order and adds them, so all of them
        // hold the reference's sum (no reduction after).  The terms travel
        // by shuffles (4 lanes) or through the warp's term buffer xbuf (8
        // lanes: one broadcast 16-byte load per charge instead of three
        // shuffles), laid out [round][lane of the line][line] so that both
        // the stores and the reads take whole wavefronts.  count is a
        // multiple of 8 TPL (the padding granule).
        constexpr int G = 32 / TPL; // lines per warp
        const int g = (threadIdx.x & 31) / TPL;
        const int base = (threadIdx.x & 31) & ~(TPL - 1);
        for (int j0 = 0; j0 < count; j0 += 8 * TPL) {
            T tx[8], ty[8], tz[8];
            bool ok = nb;
            if (nb) {
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    ok &= pair_exact_nb(px, py, pz, load_charge(tile, j0 + u * TPL + t), K,
                                        three_arg, tx[u], ty[u], tz[u]);
            }
            if (!ok) {
                for (int u = 0; u < 8; ++u) {
                    T ex = 0, ey = 0, ez = 0;
                    pair_exact<T>(px, py, pz, load_charge(tile, j0 + u * TPL + t), K, three_arg,
                                  ex, ey, ez);
                    tx[u] = ex;
                    ty[u] = ey;
                    tz[u] = ez;
                }
            }
            if constexpr (TPL >= kExactSmemTpl) {
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    xbuf[(u * TPL + t) * G + g] = make_float4(tx[u], ty[u], tz[u], 0.0f);
                __syncwarp();
#pragma unroll
                for (int u = 0; u < 8; ++u) {
#pragma unroll
                    for (int k = 0; k < TPL; ++k) {
                        const float4 v = xbuf[(u * TPL + k) * G + g];
                        a.x = add_rn(a.x, v.x);
                        a.y = add_rn(a.y, v.y);
                        a.z = add_rn(a.z, v.z);
                    }
                }
                __syncwarp(); // the buffer is rewritten by the next batch
            } else {
#pragma unroll
                for (int u = 0; u < 8; ++u) {
#pragma unroll
                    for (int k = 0; k < TPL; ++k) {
                        a.x = add_rn(a.x, __shfl_sync(0xffffffffu, tx[u], base + k));
                        a.y = add_rn(a.y, __shfl_sync(0xffffffffu, ty[u], base + k));
                        a.z = add_rn(a.z, __shfl_sync(0xffffffffu, tz[u], base + k));
                    }
                }
            }
        }
    } else if constexpr (sizeof(T) == 4) {
        // one lane per line (the reference's charge order): the terms of
        // consecutive charges are independent, only the sums are ordered.
        // Sixteen terms at a time (eight for a last odd granule) from the
        // branch-free rounded operations (the same bits), a rare pass
        // redoing them with the compiler's rounded operations when an
        // operand leaves its checked range, then the sums in charge order;
        // count is a multiple of 8 (the padding granule).  (Sixteen in
        // flight: the reference's default run 174 ms, eight 188.)
        auto batch = [&](int j0, auto bn) {
            constexpr int B = decltype(bn)::value;
            T tx[B], ty[B], tz[B];
            bool ok = nb;
            if (nb) {
#pragma unroll
                for (int u = 0; u < B; ++u)
                    ok &= pair_exact_nb(px, py, pz, load_charge(tile, j0 + u * TPL), K,
                                        three_arg, tx[u], ty[u], tz[u]);
            }
            if (!ok) {
                for (int u = 0; u < B; ++u) {
                    T ex = 0, ey = 0, ez = 0;
                    pair_exact<T>(px, py, pz, load_charge(tile, j0 + u * TPL), K, three_arg,
                                  ex, ey, ez);
                    tx[u] = ex;
                    ty[u] = ey;
                    tz[u] = ez;
                }
            }
#pragma unroll
            for (int u = 0; u < B; ++u) {
                a.x = add_rn(a.x, tx[u]);
                a.y = add_rn(a.y, ty[u]);
                a.z = add_rn(a.z, tz[u]);
            }
        };
        int j0 = t;
        for (; j0 + 15 * TPL < count; j0 += 16 * TPL)
            batch(j0, std::integral_constant<int, 16>{});
        if (j0 < count)
            batch(j0, std::integral_constant<int, 8>{});
    } else {
#pragma unroll 2
        for (int j = t; j < count; j += TPL)
            pair_exact<T>(px, py, pz, load_charge(tile, j), K, three_arg, a.x, a.y, a.z);
    }
}

// Folds the packed halves into the scalar components (packed path only).
template <class T, int ARITH>
__device__ __forceinline__ void acc_finish(Acc<T> &a)
{
    if (ARITH == ARITH_FAST2) {
        float l, h;
        f2_unpack(a.X, l, h);
        a.x = l + h;
        f2_unpack(a.Y, l, h);
        a.y = l + h;
        f2_unpack(a.Z, l, h);
        a.z = l + h;
    }
}

// KL lines per lane (fast scalar form only): one broadcast charge load feeds
// KL independent pair chains, which doubles the work in flight per warp.
template <class T, int TPL, int ARITH, int KL, class Rec>
__device__ __forceinline__ void accumulate_k(const Rec *tile, int count, int t, const T *px,
                                             const T *py, const T *pz, T K, bool three_arg,
                                             bool nb, float4 *xbuf, Acc<T> *a)
{
    if (ARITH == ARITH_FAST2 && KL > 1) {
        // a charge pair (two LDS.128) feeds KL lines, two charges per
        // packed instruction
        const ulonglong2 *tp = reinterpret_cast<const ulonglong2 *>(tile);
        const int G = count / 2;
        u64 PX[KL], PY[KL], PZ[KL];
#pragma unroll
        for (int k = 0; k < KL; ++k) {
            PX[k] = f2_pack(px[k], px[k]);
            PY[k] = f2_pack(py[k], py[k]);
            PZ[k] = f2_pack(pz[k], pz[k]);
        }
#pragma unroll 2
        for (int jp = t; jp < G; jp += TPL) {
            const ulonglong2 A = tp[jp], B = tp[G + jp];
#pragma unroll
            for (int k = 0; k < KL; ++k)
                pair2_fast(PX[k], PY[k], PZ[k], A, B, a[k].X, a[k].Y, a[k].Z);
        }
    } else if (KL == 1) {
        accumulate<T, TPL, ARITH>(tile, count, t, px[0], py[0], pz[0], K, three_arg, nb, xbuf,
                                  a[0]);
    } else {
#pragma unroll 8
        for (int j = t; j < count; j += TPL) {
            const auto c = load_charge(tile, j);
#pragma unroll
            for (int k = 0; k < KL; ++k)
                pair_fast<T>(px[k], py[k], pz[k], c, a[k].x, a[k].y, a[k].z);
        }
    }
}

// Mixed arithmetic (FP32 records in the paired layout, two charges per
// packed .f32x2 instruction): the pairs of records [0, count) of KL lines
// for lane t of TPL.
//
// Term.  With y = rsqrt(r2) (relative error d) and w = y*y, the product
// r2*w = 1 + 2d, and q/|r|^3 = q y^3 (2.5 - 1.5 r2 w) + O(d^2): one Newton
// correction.  Written as v * (r2 w - 5/3) with v = q y w it costs two
// operations beyond the plain term and yields -(2/3) q/|r|^3; the factor
// -3/2 (and the rounding of 5/3 to FP32, a constant factor) goes into the
// per-vertex scale kMixScale.  14 FMA-pipe operations per pair against the
// plain term's 12.
//
// Sums.  Each lane adds its terms into FP32 chunk sums of kMixChunk charge
// pairs (both halves folded), which enter compensated (hi, lo) sums.  l2
// collects sum_j |t_j|^2 = sum_j q_j^2 y_j^4 (one more packed FMA per
// charge pair, from q y and v), which the per-vertex test compares with
// |E|^2: the rounding error of the FP32 sum grows with the size of the
// terms, not of their sum.  (Squared chunk sums would cost less but miss
// terms that cancel inside a chunk, such as the two charges of a dipole
// stored side by side.)
constexpr int kMixChunk = 32; // charge pairs per lane and chunk (kMixC53, kMixScale: em_ext.cuh)

template <int TPL, int KL>
__device__ __forceinline__ void accumulate_mixed(const float4 *tile, int count, int t,
                                                 const float *px, const float *py,
                                                 const float *pz, CF *hx, CF *hy, CF *hz,
                                                 float *l2)
{
    const ulonglong2 *tp = reinterpret_cast<const ulonglong2 *>(tile);
    const int G = count / 2; // charge pairs: {xa,xb,ya,yb} plane, then {za,zb,qa,qb}
    const u64 C53 = f2_pack(kMixC53, kMixC53);
    u64 PX[KL], PY[KL], PZ[KL], L2[KL];
#pragma unroll
    for (int k = 0; k < KL; ++k) {
        PX[k] = f2_pack(px[k], px[k]);
        PY[k] = f2_pack(py[k], py[k]);
        PZ[k] = f2_pack(pz[k], pz[k]);
        L2[k] = 0ull;
    }
    for (int j0 = t; j0 < G; j0 += TPL * kMixChunk) {
        const int j1 = min(G, j0 + TPL * kMixChunk);
        u64 AX[KL], AY[KL], AZ[KL];
#pragma unroll
        for (int k = 0; k < KL; ++k)
            AX[k] = AY[k] = AZ[k] = 0ull;
#pragma unroll 4
        for (int jp = j0; jp < j1; jp += TPL) {
            const ulonglong2 A = tp[jp], B = tp[G + jp];
#pragma unroll
            for (int k = 0; k < KL; ++k) {
                const u64 dx = f2_sub(PX[k], A.x), dy = f2_sub(PY[k], A.y),
                          dz = f2_sub(PZ[k], B.x);
                const u64 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
                const u64 y = f2_rsqrt(r2);
                const u64 w = f2_mul(y, y);
                const u64 qy = f2_mul(B.y, y);
                const u64 v = f2_mul(qy, w);
                const u64 sc = f2_mul(v, f2_fma(r2, w, C53));
                AX[k] = f2_fma(sc, dx, AX[k]);
                AY[k] = f2_fma(sc, dy, AY[k]);
                AZ[k] = f2_fma(sc, dz, AZ[k]);
                L2[k] = f2_fma(qy, v, L2[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < KL; ++k) {
            float a, b;
            f2_unpack(AX[k], a, b);
            const float sx = a + b;
            f2_unpack(AY[k], a, b);
            const float sy = a + b;
            f2_unpack(AZ[k], a, b);
            const float sz = a + b;
            hx[k].add(sx);
            hy[k].add(sy);
            hz[k].add(sz);
        }
    }
#pragma unroll
    for (int k = 0; k < KL; ++k) {
        float a, b;
        f2_unpack(L2[k], a, b);
        l2[k] += a + b;
    }
}

// Double-float field (q r/|r|^3 summed, no Coulomb constant) at an FP32
// point from staged paired-layout records (blocks of `block` records: the
// block's A plane, then its B plane) in shared memory (resident charges) or
// global memory (streamed), computed by the whole warp: lane l takes charge
// pairs l, l + 32, ..., two per iteration with both loads issued first;
// every lane returns the same sums.
__device__ __noinline__ void refine_df_warp(const float4 *rec, int p_pad, int block, int lane,
                                            float px, float py, float pz, double &fx,
                                            double &fy, double &fz)
{
    CF hx, hy, hz;
    const int half = block / 2, npair = p_pad / 2;
    auto add = [&](const float4 &A, const float4 &B) {
        DF tx, ty, tz;
        float r2h;
        df_pair(px, py, pz, make_float4(A.x, A.z, B.x, B.z), tx, ty, tz, r2h);
        cf_add_df(hx, tx);
        cf_add_df(hy, ty);
        cf_add_df(hz, tz);
        df_pair(px, py, pz, make_float4(A.y, A.w, B.y, B.w), tx, ty, tz, r2h);
        cf_add_df(hx, tx);
        cf_add_df(hy, ty);
        cf_add_df(hz, tz);
    };
    auto at = [&](int gp, float4 &A, float4 &B) {
        const int b = gp / half, jp = gp - b * half;
        A = rec[(size_t)b * block + jp];
        B = rec[(size_t)b * block + half + jp];
    };
    int gp = lane;
    for (; gp + 32 < npair; gp += 64) {
        float4 A0, B0, A1, B1;
        at(gp, A0, B0);
        at(gp + 32, A1, B1);
        add(A0, B0);
        add(A1, B1);
    }
    if (gp < npair) {
        float4 A0, B0;
        at(gp, A0, B0);
        add(A0, B0);
    }
    fx = group_sum<double, 32>((double)hx.h + (double)hx.l);
    fy = group_sum<double, 32>((double)hy.h + (double)hy.l);
    fz = group_sum<double, 32>((double)hz.h + (double)hz.l);
}

// End of a step in the mixed arithmetic for the KL lines of lane t: the
// group's compensated sums, scaled back to the field in FP64 and rounded
// once; the test of the sum's conditioning (sum_j |t_j|^2 > kappa^2 |E|^2,
// from the chunk sums); the double-float field of every flagged vertex,
// each computed by the whole warp; the reference's step in FP32 and the
// position accumulated in FP64.
template <int TPL, int KL>
__device__ __forceinline__ void finish_mixed(const RefTraceParams<float> &P,
                                             const float4 *rec, int step, int t,
                                             int lane, const long long *line, const bool *own,
                                             float *px, float *py, float *pz, double *qx,
                                             double *qy, double *qz, CF *hx, CF *hy, CF *hz,
                                             const float *l2)
{
    const size_t n = (size_t)P.n;
    // the scale back to the field (kMixScale times the Coulomb constant) as
    // a double-float pair: (h + l) * scale rounded once, in FP32
    constexpr double kScale = kMixScale * kElectroK;
    constexpr float kScaleH = (float)kScale;
    constexpr float kScaleL = (float)(kScale - (double)kScaleH);
    // l2 is in q/r^2 units, the sums in the terms' scaled units
    const float lim2 = (float)(P.kappa2 * (kMixScale * kMixScale));
    float ex[KL], ey[KL], ez[KL];
    bool redo[KL];
#pragma unroll
    for (int k = 0; k < KL; ++k) {
        group_two_sum<TPL>(hx[k]);
        group_two_sum<TPL>(hy[k]);
        group_two_sum<TPL>(hz[k]);
        const float l2s = group_sum<float, TPL>(l2[k]);
        const float h2 = fmaf(hx[k].h, hx[k].h, fmaf(hy[k].h, hy[k].h, hz[k].h * hz[k].h));
        redo[k] = own[k] && l2s > lim2 * h2;
        ex[k] = fmaf(hx[k].h, kScaleH, fmaf(hx[k].h, kScaleL, hx[k].l * kScaleH));
        ey[k] = fmaf(hy[k].h, kScaleH, fmaf(hy[k].h, kScaleL, hy[k].l * kScaleH));
        ez[k] = fmaf(hz[k].h, kScaleH, fmaf(hz[k].h, kScaleL, hz[k].l * kScaleH));
    }
#pragma unroll
    for (int k = 0; k < KL; ++k) {
        unsigned m = __ballot_sync(0xffffffffu, redo[k] && t == 0);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const float rx = __shfl_sync(0xffffffffu, px[k], src);
            const float ry = __shfl_sync(0xffffffffu, py[k], src);
            const float rz = __shfl_sync(0xffffffffu, pz[k], src);
            double fx, fy, fz;
            refine_df_warp(rec, P.p_pad, P.tile_recs, lane, rx, ry, rz, fx, fy, fz);
            if (lane / TPL == src / TPL) {
                ex[k] = (float)(fx * kElectroK);
                ey[k] = (float)(fy * kElectroK);
                ez[k] = (float)(fz * kElectroK);
            }
            if (lane == src && P.refines)
                atomicAdd(P.refines, 1ull);
        }
    }
    const bool curvature = P.rule != RULE_FIXED;
#pragma unroll
    for (int k = 0; k < KL; ++k) {
        if (P.ox && own[k] && t == 0) {
            const size_t fi = (size_t)(step - 1) * n + (size_t)line[k];
            store_stream(P.ox + fi, ex[k]);
            store_stream(P.oy + fi, ey[k]);
            store_stream(P.oz + fi, ez[k]);
        }
        float r0x = px[k], r0y = py[k], r0z = pz[k];
        if (P.rule == RULE_SSE && own[k]) {
            r0x = ld_seed(P.seed_x + line[k]);
            r0y = ld_seed(P.seed_y + line[k]);
            r0z = ld_seed(P.seed_z + line[k]);
        }
        float sx, sy, sz;
        step_of<float>(ex[k], ey[k], ez[k], r0x, r0y, r0z, curvature, P.resolution, sx, sy, sz);
        // the FP64 position on the group's first lane, its FP32 copy to all
        if (t == 0) {
            qx[k] += (double)sx;
            qy[k] += (double)sy;
            qz[k] += (double)sz;
            px[k] = (float)qx[k];
            py[k] = (float)qy[k];
            pz[k] = (float)qz[k];
        }
        const int lead = lane & ~(TPL - 1);
        px[k] = __shfl_sync(0xffffffffu, px[k], lead);
        py[k] = __shfl_sync(0xffffffffu, py[k], lead);
        pz[k] = __shfl_sync(0xffffffffu, pz[k], lead);
        if (own[k] && t == 0) {
            const size_t idx = (size_t)step * n + (size_t)line[k];
            store_stream(P.x + idx, px[k]);
            store_stream(P.y + idx, py[k]);
            store_stream(P.z + idx, pz[k]);
        }
    }
}

template <class T, int TPL, int ARITH, int KL, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) ref_trace_kernel(const RefTraceParams<T> P)
{
    using Rec = typename ChargeRec<T>::type;
    constexpr int LG = 32 / TPL;   // line slots per warp (lanes / TPL)
    constexpr int LPW = LG * KL;   // lines per warp
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    Rec *tiles = reinterpret_cast<Rec *>(smem + 128);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const bool streamed = !P.resident;
    const int ncw = streamed ? nwarps - 1 : nwarps;
    const int NST = streamed ? P.stages : 1;
    if (NST > 8 || ncw < 1) {
        if (threadIdx.x == 0)
            atomicCAS(P.err, 0, EM_DEVERR_CONFIG);
        return;
    }
    const uint32_t full0 = smem_addr(bars), empty0 = smem_addr(bars + 8);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, ncw);
        }
        fence_mbar_init();
    }
    __syncthreads();

    const long long cta_groups =
        blockIdx.x < P.n_groups ? (P.n_groups - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const int rounds = (int)((cta_groups + ncw - 1) / ncw);
    const T K = (T)kElectroK;
    const bool curvature = P.rule != RULE_FIXED;
    const bool three_arg = P.rule == RULE_SSE;
    // exact arithmetic: the branch-free rounded operations once verified on
    // this device (else the compiler's rounded operations for every pair)
    const bool nb = ARITH == ARITH_EXACT && P.exact_nb != 0;
    // exact arithmetic, 8 lanes per line: this warp's term buffer, after the
    // charge tiles (the planner reserves it; other shapes never touch it)
    float4 *xbuf = reinterpret_cast<float4 *>(
                       smem + 128 +
                       (size_t)(streamed ? P.stages * P.tile_recs : P.p_pad) * sizeof(Rec)) +
                   (size_t)warp * (kExactTermBytesPerWarp / 16);
    const int t = lane % TPL;
    const size_t n = (size_t)P.n;

    if (!streamed) {
        if (threadIdx.x == 0) {
            const uint32_t bytes = (uint32_t)P.p_pad * (uint32_t)sizeof(Rec);
            mbar_arrive_expect_tx(full0, bytes);
            const char *src = static_cast<const char *>(P.charges);
            const uint32_t dst = smem_addr(tiles);
            constexpr uint32_t CH = 32768;
            for (uint32_t off = 0; off < bytes; off += CH)
                bulk_g2s(dst + off, src + off, bytes - off < CH ? bytes - off : CH, full0);
        }
        if (!mbar_wait(full0, 0, P.err))
            return;
    }

    if (streamed && warp == nwarps - 1) {
        // ---- producer warp: one lane issues every tile copy -------------------
        if (lane == 0) {
            const uint32_t tb = (uint32_t)P.tile_recs * (uint32_t)sizeof(Rec);
            const char *src = static_cast<const char *>(P.charges);
            uint32_t it = 0;
            bool ok = true;
            for (int r = 0; r < rounds && ok; ++r)
                for (int step = 1; step < P.total_steps && ok; ++step)
                    for (int tile = 0; tile < P.n_tiles; ++tile, ++it) {
                        const uint32_t s = it % NST, ph = (it / NST) & 1;
                        if (it >= (uint32_t)NST && !mbar_wait(empty0 + 8 * s, ph ^ 1, P.err)) {
                            ok = false;
                            break;
                        }
                        mbar_arrive_expect_tx(full0 + 8 * s, tb);
                        bulk_g2s(smem_addr(tiles) + s * tb, src + (size_t)tile * tb, tb,
                                 full0 + 8 * s);
                    }
            // Drain: the latest copy on each stage must have landed before
            // the CTA may exit (bounded like every other wait).
            const uint32_t last = it;
            for (uint32_t k = 0; k < (uint32_t)NST && k < last; ++k) {
                const uint32_t j = last - 1 - k;
                mbar_wait(full0 + 8 * (j % NST), (j / NST) & 1, P.err);
            }
        }
        return;
    }

    // ---- compute warps --------------------------------------------------------
    // Groups: dealt round-robin to CTAs, or, with resident charges and a
    // group counter (the mixed form, whose re-evaluations make some groups
    // slower than others), taken one at a time by whichever warp is free.
    constexpr bool kQueue = ARITH == ARITH_MIXED;
    const bool queued = kQueue && !streamed && P.group_ctr;
    uint32_t it = 0;
    for (int r = 0; queued || r < rounds; ++r) {
        long long gk = (long long)r * ncw + warp;
        long long g = blockIdx.x + (long long)gridDim.x * gk;
        bool active = gk < cta_groups;
        if (queued) {
            unsigned long long q = 0;
            if (lane == 0)
                q = atomicAdd(P.group_ctr, 1ull);
            g = (long long)__shfl_sync(0xffffffffu, q, 0);
            active = g < P.n_groups;
        }
        if (!streamed && !active)
            break;
        long long line[KL];
        bool own[KL];
        T px[KL], py[KL], pz[KL];
        double qx[KL], qy[KL], qz[KL]; // mixed: the FP64 position
#pragma unroll
        for (int k = 0; k < KL; ++k) {
            // slot k of the warp's lines: consecutive lanes -> consecutive lines
            line[k] = g * LPW + k * LG + lane / TPL;
            own[k] = active && line[k] < P.n;
            px[k] = py[k] = pz[k] = 0;
            if (own[k]) {
                px[k] = P.x[line[k]];
                py[k] = P.y[line[k]];
                pz[k] = P.z[line[k]];
            }
            qx[k] = (double)px[k];
            qy[k] = (double)py[k];
            qz[k] = (double)pz[k];
        }
        for (int step = 1; step < P.total_steps; ++step) {
            Acc<T> acc[KL];
            CF hx[KL], hy[KL], hz[KL];
            float l2[KL];
#pragma unroll
            for (int k = 0; k < KL; ++k)
                l2[k] = 0.0f;
            auto charges_of = [&](const Rec *tp, int count) {
                if constexpr (ARITH == ARITH_MIXED)
                    accumulate_mixed<TPL, KL>(reinterpret_cast<const float4 *>(tp), count, t,
                                              reinterpret_cast<const float *>(px),
                                              reinterpret_cast<const float *>(py),
                                              reinterpret_cast<const float *>(pz), hx, hy, hz,
                                              l2);
                else
                    accumulate_k<T, TPL, ARITH, KL>(tp, count, t, px, py, pz, K, three_arg, nb, xbuf,
                                                    acc);
            };
            if (!streamed) {
                charges_of(tiles, P.p_pad);
            } else {
                for (int tile = 0; tile < P.n_tiles; ++tile, ++it) {
                    const uint32_t s = it % NST, ph = (it / NST) & 1;
                    if (!mbar_wait(full0 + 8 * s, ph, P.err))
                        return;
                    if (active)
                        charges_of(tiles + s * P.tile_recs, P.tile_recs);
                    __syncwarp();
                    if (lane == 0)
                        mbar_arrive(empty0 + 8 * s);
                }
                if (!active)
                    continue;
            }
            if constexpr (ARITH == ARITH_MIXED) {
                // re-evaluations read the records from shared memory when
                // they are resident there, else from the staged copy
                finish_mixed<TPL, KL>(P,
                                      streamed ? static_cast<const float4 *>(P.charges)
                                               : reinterpret_cast<const float4 *>(tiles),
                                      step, t, lane, line, own, px, py, pz, qx, qy, qz, hx,
                                      hy, hz, l2);
                continue;
            }
#pragma unroll
            for (int k = 0; k < KL; ++k) {
                acc_finish<T, ARITH>(acc[k]);
                T ax = acc[k].x, ay = acc[k].y, az = acc[k].z;
                // (the exact arithmetic's lanes already hold the line's sum)
                if (TPL > 1 && ARITH != ARITH_EXACT) {
                    ax = line_reduce<T, TPL>(ax);
                    ay = line_reduce<T, TPL>(ay);
                    az = line_reduce<T, TPL>(az);
                }
                if (P.fx && own[k] && t == 0) {
                    const size_t fi = (size_t)(step - 1) * n + (size_t)line[k];
                    store_stream(P.fx + fi, ax);
                    store_stream(P.fy + fi, ay);
                    store_stream(P.fz + fi, az);
                }
                if (ARITH != ARITH_EXACT) {
                    ax = mul_rn(ax, K);
                    ay = mul_rn(ay, K);
                    az = mul_rn(az, K);
                }
                // curvature vector: the seed for the SSE rule, loaded once in the
                // reference (CPU_Implement.cpp:254-256) and never updated, here
                // re-read from row 0 each step so it holds no registers during
                // the pair loop; the previous point for the generic rule
                // (CPU_Implement.cpp:148-153)
                T r0x = px[k], r0y = py[k], r0z = pz[k];
                if (P.rule == RULE_SSE && own[k]) {
                    r0x = ld_seed(P.seed_x + line[k]);
                    r0y = ld_seed(P.seed_y + line[k]);
                    r0z = ld_seed(P.seed_z + line[k]);
                }
                advance<T>(ax, ay, az, r0x, r0y, r0z, curvature, P.resolution, px[k], py[k],
                           pz[k]);
                if (own[k] && t == 0) {
                    const size_t idx = (size_t)step * n + (size_t)line[k];
                    store_stream(P.x + idx, px[k]);
                    store_stream(P.y + idx, py[k]);
                    store_stream(P.z + idx, pz[k]);
                }
            }
        }
    }
}

// Copies p charge records into the staged buffer of p_pad records, filling
// [p, p_pad) with the pad record {1e15, 1e15, 1e15, 0} (its contribution is
// exactly zero in every arithmetic), in plain {x,y,z,q} order (paired = 0)
// or, for the packed form (1), in blocks of `block` records (one charge
// tile): the block's {xa,xb,ya,yb} records, then its {za,zb,qa,qb} records,
// so the lanes of a line read consecutive 16-B slots (no bank conflicts).
template <class T>
__global__ void stage_kernel(const T *raw, int p, T *staged, int p_pad, int paired, int block)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p_pad)
        return;
    T v[4];
    if (i < p) {
        for (int c = 0; c < 4; ++c)
            v[c] = raw[4 * (size_t)i + c];
    } else {
        v[0] = v[1] = v[2] = T(1e15);
        v[3] = T(0);
    }
    if (!paired) {
        for (int c = 0; c < 4; ++c)
            staged[4 * (size_t)i + c] = v[c];
    } else {
        const int G = block / 2;      // pairs per block
        const int jp = i >> 1, h = i & 1;
        const size_t b0 = 4 * (size_t)(jp / G) * block; // block start (floats)
        const size_t w = 4 * (size_t)(jp % G);
        staged[b0 + w + h] = v[0];                    // A: {xa,xb,ya,yb}
        staged[b0 + w + 2 + h] = v[1];
        staged[b0 + 4 * (size_t)G + w + h] = v[2];    // B: {za,zb,qa,qb}
        staged[b0 + 4 * (size_t)G + w + 2 + h] = v[3];
    }
}

template <class T, int TPL, int ARITH, int KL, int MAXT>
cudaError_t launch_one(const RefTraceParams<T> &p, const LaunchCfg &cfg, cudaStream_t stream)
{
    auto kern = ref_trace_kernel<T, TPL, ARITH, KL, MAXT>;
    const int threads = 32 * (cfg.warps + (cfg.resident ? 0 : 1));
    if (threads > MAXT)
        return cudaErrorInvalidConfiguration;
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess)
        return e;
    kern<<<cfg.grid, threads, cfg.smem, stream>>>(p);
    count_launch(1);
    return cudaGetLastError();
}

// Fast scalar form: KL lines per lane, register budget by thread bound
// (1024 threads -> 64 registers, 768 -> 80).
template <class T, int TPL>
cudaError_t launch_fast(const RefTraceParams<T> &p, const LaunchCfg &cfg, cudaStream_t stream)
{
    const int threads = 32 * (cfg.warps + (cfg.resident ? 0 : 1));
    if (cfg.kl == 2)
        return threads <= 768 ? launch_one<T, TPL, ARITH_FAST, 2, 768>(p, cfg, stream)
                              : launch_one<T, TPL, ARITH_FAST, 2, 1024>(p, cfg, stream);
    return threads <= 768 ? launch_one<T, TPL, ARITH_FAST, 1, 768>(p, cfg, stream)
                          : launch_one<T, TPL, ARITH_FAST, 1, 1024>(p, cfg, stream);
}

// Mixed form: up to 512 threads per CTA (128 registers: two lines' packed
// chunk sums, compensated sums and FP64 positions).
template <class T, int TPL>
cudaError_t launch_mixed(const RefTraceParams<T> &p, const LaunchCfg &cfg, cudaStream_t stream)
{
    return cfg.kl == 2 ? launch_one<T, TPL, ARITH_MIXED, 2, 512>(p, cfg, stream)
                       : launch_one<T, TPL, ARITH_MIXED, 1, 512>(p, cfg, stream);
}

template <class T, int TPL>
cudaError_t launch_packed(const RefTraceParams<T> &p, const LaunchCfg &cfg, cudaStream_t stream)
{
    return cfg.kl == 2 ? launch_one<T, TPL, ARITH_FAST2, 2, 1024>(p, cfg, stream)
                       : launch_one<T, TPL, ARITH_FAST2, 1, 1024>(p, cfg, stream);
}

} // namespace

template <class T>
cudaError_t launch_ref_trace(const RefTraceParams<T> &params, const LaunchCfg &cfg, int arith,
                             cudaStream_t stream)
{
    RefTraceParams<T> p = params;
    if (!p.seed_x) {
        p.seed_x = p.x;
        p.seed_y = p.y;
        p.seed_z = p.z;
    }
    if (cfg.kl != 1 && (cfg.kl != 2 || arith == ARITH_EXACT))
        return cudaErrorInvalidValue;
    if (arith == ARITH_EXACT) {
        if (cfg.tpl == 1)
            return launch_one<T, 1, ARITH_EXACT, 1, exact_max_threads(1)>(p, cfg, stream);
        if constexpr (sizeof(T) == 4) {
            if (cfg.tpl == 4)
                return launch_one<T, 4, ARITH_EXACT, 1, exact_max_threads(4)>(p, cfg, stream);
            if (cfg.tpl == 8)
                return launch_one<T, 8, ARITH_EXACT, 1, exact_max_threads(8)>(p, cfg, stream);
        }
        return cudaErrorInvalidValue;
    }
    if (arith == ARITH_MIXED) {
        if constexpr (sizeof(T) != 4) {
            return cudaErrorInvalidValue;
        } else {
            switch (cfg.tpl) {
            case 1: return launch_mixed<T, 1>(p, cfg, stream);
            case 2: return launch_mixed<T, 2>(p, cfg, stream);
            case 4: return launch_mixed<T, 4>(p, cfg, stream);
            case 8: return launch_mixed<T, 8>(p, cfg, stream);
            default: return cudaErrorInvalidValue;
            }
        }
    }
    if (arith == ARITH_FAST2) {
        if (sizeof(T) != 4)
            return cudaErrorInvalidValue;
        switch (cfg.tpl) {
        case 1: return launch_packed<T, 1>(p, cfg, stream);
        case 2: return launch_packed<T, 2>(p, cfg, stream);
        case 4: return launch_packed<T, 4>(p, cfg, stream);
        case 8: return launch_packed<T, 8>(p, cfg, stream);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (cfg.tpl) {
    case 1: return launch_fast<T, 1>(p, cfg, stream);
    case 2: return launch_fast<T, 2>(p, cfg, stream);
    case 4: return launch_fast<T, 4>(p, cfg, stream);
    case 8: return launch_fast<T, 8>(p, cfg, stream);
    default: return cudaErrorInvalidValue;
    }
}

namespace {

// v *= K with the kernel's own rounding (mul_rn), over m values: the field
// the fast arithmetic stored before its per-vertex Coulomb factor.
template <class T> __global__ void scale_k_kernel(T *v, size_t m)
{
    const T K = (T)kElectroK;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (size_t)gridDim.x * blockDim.x)
        v[i] = mul_rn(v[i], K);
}

} // namespace

template <class T> cudaError_t launch_scale_coulomb(T *v, size_t m, cudaStream_t stream)
{
    if (!m)
        return cudaSuccess;
    const size_t blocks = std::min<size_t>((m + 255) / 256, 152 * 16);
    scale_k_kernel<T><<<(unsigned)blocks, 256, 0, stream>>>(v, m);
    count_launch(1);
    return cudaGetLastError();
}

template cudaError_t launch_scale_coulomb<float>(float *, size_t, cudaStream_t);
template cudaError_t launch_scale_coulomb<double>(double *, size_t, cudaStream_t);

template <class T>
cudaError_t launch_stage_charges(const void *raw, int p, void *staged, int p_pad, int paired,
                                 int block, cudaStream_t stream)
{
    if (p_pad <= 0)
        return cudaSuccess;
    if (paired && (block <= 0 || (block & 1) || p_pad % block))
        return cudaErrorInvalidValue;
    stage_kernel<T><<<(p_pad + 127) / 128, 128, 0, stream>>>(
        static_cast<const T *>(raw), p, static_cast<T *>(staged), p_pad, paired, block);
    count_launch(1);
    return cudaGetLastError();
}

template cudaError_t launch_ref_trace<float>(const RefTraceParams<float> &, const LaunchCfg &,
                                             int, cudaStream_t);
template cudaError_t launch_ref_trace<double>(const RefTraceParams<double> &,
                                              const LaunchCfg &, int, cudaStream_t);
template cudaError_t launch_stage_charges<float>(const void *, int, void *, int, int, int,
                                                 cudaStream_t);
template cudaError_t launch_stage_charges<double>(const void *, int, void *, int, int, int,
                                                  cudaStream_t);

} // namespace em
