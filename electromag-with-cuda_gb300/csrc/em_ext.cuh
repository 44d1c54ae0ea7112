// Device pieces of the extended tracer shared by the single-set kernel
// (em_trace_ext.cu) and the batched kernel (em_trace_batch.cu): pair loops
// with the nearest-negative-charge tracking, the mixed-precision forms, the
// lane-group reductions and their runtime width dispatch, the step vector.
#pragma once

#include "em_device.cuh"
#include "em_internal.h"
#include "em_math.cuh"

namespace em {
namespace {

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// Compensated value (hi, lo).
struct CF {
    float h = 0, l = 0;
    __device__ __forceinline__ void add(float v)
    {
        float e;
        two_sum(h, v, h, e);
        l = __fadd_rn(l, e);
    }
};

template <class T> struct ExtLane {
    T px, py, pz;         // evaluation point (FP32 copy in mixed mode)
    double dx, dy, dz;    // mixed: FP64 position accumulator
};

// ---------------------------------------------------------------------------
// Pair loops over shared-memory records [0, count) of one tile, lane t of
// TPL; [0, jneg) are negative charges (nearest one tracked).
template <int TPL>
__device__ __forceinline__ void pairs_fast(const float4 *tile, int jneg, int count, int t,
                                           float px, float py, float pz, float &ax, float &ay,
                                           float &az, float &dneg)
{
#pragma unroll 4
    for (int j = t; j < jneg; j += TPL) {
        const float4 c = tile[j];
        const float dx = px - c.x, dy = py - c.y, dz = pz - c.z;
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        dneg = fminf(dneg, r2);
        const float inv = rsqrt_fast(r2);
        const float s = (c.w * inv) * (inv * inv);
        ax = fmaf(s, dx, ax);
        ay = fmaf(s, dy, ay);
        az = fmaf(s, dz, az);
    }
#pragma unroll 8
    for (int j = jneg + t; j < count; j += TPL) {
        const float4 c = tile[j];
        const float dx = px - c.x, dy = py - c.y, dz = pz - c.z;
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float inv = rsqrt_fast(r2);
        const float s = (c.w * inv) * (inv * inv);
        ax = fmaf(s, dx, ax);
        ay = fmaf(s, dy, ay);
        az = fmaf(s, dz, az);
    }
}

template <int TPL>
__device__ __forceinline__ void pairs_fast(const ChargeD *tile, int jneg, int count, int t,
                                           double px, double py, double pz, double &ax,
                                           double &ay, double &az, double &dneg)
{
    for (int j = t; j < count; j += TPL) {
        const double2 *r = reinterpret_cast<const double2 *>(tile + j);
        const double2 a = r[0], b = r[1];
        const double dx = px - a.x, dy = py - a.y, dz = pz - b.x;
        const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
        if (j < jneg)
            dneg = fmin(dneg, r2);
        const double inv = rsqrt(r2);
        const double s = (b.y * inv) * (inv * inv);
        ax = fma(s, dx, ax);
        ay = fma(s, dy, ay);
        az = fma(s, dz, az);
    }
}

// Mixed arithmetic: FP32 records in the paired layout (blocks of `block`
// records, each block's A plane {xa, xb, ya, yb} of block/2 float4, then its
// B plane {za, zb, qa, qb}), two charges per packed .f32x2 instruction.
//
// Term.  With y = rsqrt(r2) (relative error d) and w = y*y, the product
// r2*w = 1 + 2d, and q/|r|^3 = q y^3 (2.5 - 1.5 r2 w) + O(d^2): one Newton
// correction.  Written as v * (r2 w - 5/3) with v = q y w it costs two
// operations beyond the plain term and yields -(2/3) q/|r|^3; the factor
// -3/2 (and the rounding of 5/3 to FP32, a constant factor) goes into the
// per-vertex scale kMixScale.
constexpr float kMixC53 = -1.66666663f; // -5/3 rounded to FP32
// -(3/2) / ((1 + kMixC53) / (1 - 5/3)): the terms' scale back to q r/|r|^3
constexpr double kMixScale = -1.5 / ((1.0 + (double)kMixC53) / (1.0 - 5.0 / 3.0));
// charge pairs per lane and compensated chunk of the extended tracer (16
// terms: 64 left 0.09 % of the 4096-charge set's vertices at 1.1-1.6e-6)
constexpr int kMixChunkPairs = 8;

// Charge pairs [lo, hi) of one paired block (planes A, B) for lane t of
// TPL: FP32 chunk sums of kMixChunkPairs pairs (both halves folded) into the
// compensated sums; L2 collects sum_j q_j^2 y_j^4 (the conditioning test's
// measure, from q y and v); for NEG (the negative block) dmin the nearest
// distance^2.
template <int TPL, bool NEG>
__device__ __forceinline__ void mixed_pk_range(const ulonglong2 *A, const ulonglong2 *B, int lo,
                                               int hi, int t, u64 PX, u64 PY, u64 PZ, CF &hx,
                                               CF &hy, CF &hz, float &dmin, u64 &L2)
{
    const u64 C53 = f2_pack(kMixC53, kMixC53);
    u64 AX, AY, AZ;
    auto term = [&](int jp) {
        const ulonglong2 a = A[jp], b = B[jp];
        const u64 dx = f2_sub(PX, a.x), dy = f2_sub(PY, a.y), dz = f2_sub(PZ, b.x);
        const u64 r2 = f2_fma(dz, dz, f2_fma(dy, dy, f2_mul(dx, dx)));
        if (NEG) {
            float ra, rb;
            f2_unpack(r2, ra, rb);
            dmin = fminf(dmin, fminf(ra, rb));
        }
        const u64 y = f2_rsqrt(r2);
        const u64 w = f2_mul(y, y);
        const u64 qy = f2_mul(b.y, y);
        const u64 v = f2_mul(qy, w);
        const u64 sc = f2_mul(v, f2_fma(r2, w, C53));
        AX = f2_fma(sc, dx, AX);
        AY = f2_fma(sc, dy, AY);
        AZ = f2_fma(sc, dz, AZ);
        L2 = f2_fma(qy, v, L2);
    };
    for (int j0 = lo + t; j0 < hi; j0 += TPL * kMixChunkPairs) {
        AX = AY = AZ = 0ull;
        if (j0 + TPL * (kMixChunkPairs - 1) < hi) {
            // a full chunk: a fixed trip count, unrolled
#pragma unroll
            for (int u = 0; u < kMixChunkPairs; ++u)
                term(j0 + u * TPL);
        } else {
            // a short range (the tail kernels' rows): unrolled as well, so
            // its pairs overlap instead of forming one latency chain
#pragma unroll 4
            for (int jp = j0; jp < hi; jp += TPL)
                term(jp);
        }
        float u, v;
        f2_unpack(AX, u, v);
        hx.add(u + v);
        f2_unpack(AY, u, v);
        hy.add(u + v);
        f2_unpack(AZ, u, v);
        hz.add(u + v);
    }
}

// Mixed pairs [lo, hi) of one paired block whose first jn2 pairs are
// negative charges (nearest one tracked); l2 gets sum_j q_j^2 / r_j^4.  The
// sums are in the terms' scaled units (times kMixScale: q r/|r|^3).
template <int TPL>
__device__ __forceinline__ void mixed_pk(const ulonglong2 *A, const ulonglong2 *B, int jn2,
                                         int lo, int hi, int t, float px, float py, float pz,
                                         CF &hx, CF &hy, CF &hz, float &dneg, float &l2)
{
    const u64 PX = f2_pack(px, px), PY = f2_pack(py, py), PZ = f2_pack(pz, pz);
    u64 L2 = 0ull;
    float dn = 3.0e38f, unused = 0;
    mixed_pk_range<TPL, true>(A, B, lo, min(hi, jn2), t, PX, PY, PZ, hx, hy, hz, dn, L2);
    mixed_pk_range<TPL, false>(A, B, max(lo, jn2), hi, t, PX, PY, PZ, hx, hy, hz, unused, L2);
    float u, v;
    f2_unpack(L2, u, v);
    l2 += u + v;
    dneg = fminf(dneg, dn);
}

// Mixed pairs over one staged tile: `tile` is a paired block of `count`
// records whose first jneg are negative charges.
template <int TPL>
__device__ __forceinline__ void pairs_mixed(const float4 *tile, int jneg, int count, int t,
                                            float px, float py, float pz, CF &hx, CF &hy, CF &hz,
                                            float &dneg, float &l2)
{
    const ulonglong2 *A = reinterpret_cast<const ulonglong2 *>(tile);
    mixed_pk<TPL>(A, A + count / 2, jneg / 2, 0, count / 2, t, px, py, pz, hx, hy, hz, dneg, l2);
}

// ---------------------------------------------------------------------------
// Double-float arithmetic (a value is h + l, two FP32 words, about 48 bits):
// error-free sums and products by the classical transformations (Knuth's
// two-sum, Dekker's fast two-sum, the FMA two-product), every operation an
// explicitly rounded intrinsic so nothing is contracted.  The evaluation
// point is an FP32 vertex, so r = p - c is exact as a pair; the pair term
// q r / |r|^3 is formed to about 2^-41 relative, on the FP32 pipes only
// (GB300 runs FP64 at 1/64 of the FP32 rate).
struct DF {
    float h, l;
};

__device__ __forceinline__ DF df_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float ap = __fsub_rn(s, bp);
    return {s, __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp))};
}

// |a| >= |b| (or a = 0)
__device__ __forceinline__ DF df_fast(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DF df_mul(DF a, DF b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return df_fast(p, e);
}

__device__ __forceinline__ DF df_mul_f(DF a, float b)
{
    const float p = __fmul_rn(a.h, b);
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return df_fast(p, e);
}

// Square of a double-float as an unnormalised pair: the product of the
// high words exactly (FMA), the cross term folded into the low word (the
// low word squared, below 2^-48 of the result, is dropped).
__device__ __forceinline__ void df_sqr_parts(DF a, float &p, float &e)
{
    p = __fmul_rn(a.h, a.h);
    e = __fmaf_rn(a.h, a.h, -p);
    e = __fmaf_rn(__fadd_rn(a.h, a.h), a.l, e);
}

// a * b for double-float a and b as an unnormalised pair (the caller's
// compensated accumulator takes the two words separately)
__device__ __forceinline__ DF df_mul_raw(DF a, DF b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return {p, e};
}

// q r / |r|^3 for the FP32 point p and charge c, each component a DF; r2h
// gets |r|^2 rounded to FP32 (for the nearest-negative test).
//   r = p - c exactly (two-sums); |r|^2 from the three exact squares, the
//   high words summed by two-sums and the low words added plainly (about
//   2^-46 relative); y0 = rsqrt(|r|^2) in FP32 and eps = 1 - |r|^2 y0^2 in
//   double-float, so |r|^-3 = y0^3 (1 - eps)^(-3/2) = y0^3 (1 + 1.5 eps)
//   to within 15/8 eps^2 (|eps| below about 2^-21.9: about 2^-41 relative).
__device__ __forceinline__ void df_pair(float px, float py, float pz, const float4 &c, DF &tx,
                                        DF &ty, DF &tz, float &r2h)
{
    const DF dx = df_two_sum(px, -c.x), dy = df_two_sum(py, -c.y), dz = df_two_sum(pz, -c.z);
    float sx, ex, sy, ey, sz, ez;
    df_sqr_parts(dx, sx, ex);
    df_sqr_parts(dy, sy, ey);
    df_sqr_parts(dz, sz, ez);
    const DF s1 = df_two_sum(sx, sy);
    const DF s2 = df_two_sum(s1.h, sz);
    const DF r2 = df_fast(s2.h, __fadd_rn(__fadd_rn(__fadd_rn(ex, ey), ez),
                                          __fadd_rn(s1.l, s2.l)));
    r2h = r2.h;
    const float y0 = rsqrt_fast(r2.h);
    const float y2h = __fmul_rn(y0, y0);
    const DF y2 = {y2h, __fmaf_rn(y0, y0, -y2h)};
    const DF t = df_mul(r2, y2);                              // 1 - eps
    const float eps = __fsub_rn(__fsub_rn(1.0f, t.h), t.l);   // t.h is within 2^-21 of 1
    const DF y3 = df_mul_f(y2, y0);                           // y0^3
    const DF s = df_fast(y3.h, __fmaf_rn(y3.h, __fmul_rn(1.5f, eps), y3.l));
    const DF qs = df_mul_f(s, c.w);
    tx = df_mul_raw(qs, dx);
    ty = df_mul_raw(qs, dy);
    tz = df_mul_raw(qs, dz);
}

// The compensated accumulator takes a double-float term: its high word with
// a two-sum, its low word added to the low sum.
__device__ __forceinline__ void cf_add_df(CF &a, DF v)
{
    float e;
    two_sum(a.h, v.h, a.h, e);
    a.l = __fadd_rn(a.l, __fadd_rn(e, v.l));
}

// Double-float pairs over shared-memory records [0, count), lane t of TPL;
// [0, jneg) are negative charges (nearest one tracked).
template <int TPL>
__device__ __forceinline__ void pairs_df64(const float4 *tile, int jneg, int count, int t,
                                           float px, float py, float pz, CF &hx, CF &hy, CF &hz,
                                           float &dneg)
{
#pragma unroll 2
    for (int j = t; j < count; j += TPL) {
        DF tx, ty, tz;
        float r2h;
        df_pair(px, py, pz, tile[j], tx, ty, tz, r2h);
        if (j < jneg)
            dneg = fminf(dneg, r2h);
        cf_add_df(hx, tx);
        cf_add_df(hy, ty);
        cf_add_df(hz, tz);
    }
}

// Double-float (F64: FP64) field at an FP32 point from paired-layout
// records (blocks of `block` records, as staged for the mixed mode), charge
// pairs [lo, hi) of the whole staged set, lane t of TPL taking pairs
// lo + t, lo + t + TPL, ...; the lane's partial sums in FP64 (summed later
// across the group).
template <int TPL, bool F64>
__device__ __forceinline__ void field_pk(const float4 *rec, int block, int lo, int hi, int t,
                                         float px, float py, float pz, double &ax, double &ay,
                                         double &az)
{
    const int half = block / 2;
    int gp = lo + t;
    int b = gp / half, jp = gp - b * half;
    CF hx, hy, hz;
    double sx = 0, sy = 0, sz = 0;
    auto term = [&](const float4 &c) {
        if constexpr (F64) {
            const double dx = (double)px - (double)c.x, dy = (double)py - (double)c.y,
                         dz = (double)pz - (double)c.z;
            const double r2 = fma(dz, dz, fma(dy, dy, dx * dx));
            const double inv = 1.0 / sqrt(r2);
            const double s = (double)c.w * inv * inv * inv;
            sx = fma(s, dx, sx);
            sy = fma(s, dy, sy);
            sz = fma(s, dz, sz);
        } else {
            DF tx, ty, tz;
            float r2h;
            df_pair(px, py, pz, c, tx, ty, tz, r2h);
            cf_add_df(hx, tx);
            cf_add_df(hy, ty);
            cf_add_df(hz, tz);
        }
    };
    for (; gp < hi; gp += TPL) {
        const float4 A = rec[(size_t)b * block + jp];
        const float4 B = rec[(size_t)b * block + half + jp];
        term(make_float4(A.x, A.z, B.x, B.z));
        term(make_float4(A.y, A.w, B.y, B.w));
        jp += TPL;
        while (jp >= half) {
            jp -= half;
            ++b;
        }
    }
    if constexpr (F64) {
        ax += sx;
        ay += sy;
        az += sz;
    } else {
        ax += (double)hx.h + (double)hx.l;
        ay += (double)hy.h + (double)hy.l;
        az += (double)hz.h + (double)hz.l;
    }
}

template <class T, int TPL>
__device__ __forceinline__ T group_min(T v)
{
#pragma unroll
    for (int o = TPL / 2; o >= 1; o >>= 1)
        v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int TPL>
__device__ __forceinline__ void group_two_sum(CF &c)
{
#pragma unroll
    for (int o = TPL / 2; o >= 1; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, c.h, o);
        const float ol = __shfl_xor_sync(0xffffffffu, c.l, o);
        // both partners compute the same sum: order the operands by lane
        // half so the bits agree
        float a = c.h, b = oh, la = c.l, lb = ol;
        if ((threadIdx.x & o) != 0) {
            a = oh;
            b = c.h;
            la = ol;
            lb = c.l;
        }
        float s, e;
        two_sum(a, b, s, e);
        c.h = s;
        c.l = __fadd_rn(__fadd_rn(la, lb), e);
    }
}

template <class T, int TPL>
__device__ __forceinline__ T group_sum(T v)
{
#pragma unroll
    for (int o = TPL / 2; o >= 1; o >>= 1) {
        const T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = (threadIdx.x & o) ? w + v : v + w;
    }
    return v;
}

// Step vector of the reference rule (CPU_Implement.cpp:327-331): returns
// E / ((k+1) res |E|) with the reference's IEEE sequence; k2 = |E|^2.
template <class T>
__device__ __forceinline__ void step_vector(T ex, T ey, T ez, T r0x, T r0y, T r0z, T res, T &sx,
                                            T &sy, T &sz, T &k2)
{
    k2 = add_rn(add_rn(mul_rn(ex, ex), mul_rn(ey, ey)), mul_rn(ez, ez));
    const T ix = sub_rn(ex, r0x), iy = sub_rn(ey, r0y), iz = sub_rn(ez, r0z);
    const T cx = sub_rn(mul_rn(iy, r0z), mul_rn(iz, r0y));
    const T cy = sub_rn(mul_rn(iz, r0x), mul_rn(ix, r0z));
    const T cz = sub_rn(mul_rn(ix, r0y), mul_rn(iy, r0x));
    const T c2 = add_rn(add_rn(mul_rn(cx, cx), mul_rn(cy, cy)), mul_rn(cz, cz));
    const T kc = div_rn(sqrt_rn(c2), mul_rn(k2, sqrt_rn(k2)));
    const T s = mul_rn(mul_rn(add_rn(kc, T(1)), res), sqrt_rn(k2));
    sx = div_rn(ex, s);
    sy = div_rn(ey, s);
    sz = div_rn(ez, s);
}


// ---- group-size dispatch -------------------------------------------------
// A warp's lane groups start TPL lanes wide and may double (up to the whole
// warp) when the work queue runs dry; the pair loops stay specialised per
// width, chosen once per step-iteration.
template <class T, int MODE, class Rec>
__device__ __forceinline__ void tile_pairs(int tg, const Rec *tile, int jn, int count, int t,
                                           const ExtLane<T> &st, T &ax, T &ay, T &az, T &dneg,
                                           float &dall, CF &hx, CF &hy, CF &hz)
{
#define EM_TILE_PAIRS(G)                                                                       \
    if constexpr (MODE == EXT_MIXED)                                                           \
        pairs_mixed<G>(tile, jn, count, t, st.px, st.py, st.pz, hx, hy, hz, dneg, dall);       \
    else if constexpr (MODE == EXT_DF64)                                                       \
        pairs_df64<G>(tile, jn, count, t, st.px, st.py, st.pz, hx, hy, hz, dneg);              \
    else                                                                                       \
        pairs_fast<G>(tile, jn, count, t, st.px, st.py, st.pz, ax, ay, az, dneg);
    switch (tg) {
    case 4: EM_TILE_PAIRS(4) break;
    case 8: EM_TILE_PAIRS(8) break;
    case 16: EM_TILE_PAIRS(16) break;
    default: EM_TILE_PAIRS(32) break;
    }
#undef EM_TILE_PAIRS
}

template <class T, int MODE>
__device__ __forceinline__ void combine_group(int tg, T &ax, T &ay, T &az, T &dneg, float &dall,
                                              CF &hx, CF &hy, CF &hz)
{
#define EM_COMBINE(G)                                                                          \
    if constexpr (MODE == EXT_MIXED || MODE == EXT_DF64) {                                     \
        group_two_sum<G>(hx);                                                                  \
        group_two_sum<G>(hy);                                                                  \
        group_two_sum<G>(hz);                                                                  \
        ax = (T)__fadd_rn(hx.h, hx.l);                                                         \
        ay = (T)__fadd_rn(hy.h, hy.l);                                                         \
        az = (T)__fadd_rn(hz.h, hz.l);                                                         \
        if constexpr (MODE == EXT_MIXED)                                                       \
            dall = group_sum<float, G>(dall);                                                  \
    } else {                                                                                   \
        ax = group_sum<T, G>(ax);                                                              \
        ay = group_sum<T, G>(ay);                                                              \
        az = group_sum<T, G>(az);                                                              \
    }                                                                                          \
    dneg = group_min<T, G>(dneg);
    switch (tg) {
    case 4: { EM_COMBINE(4) } break;
    case 8: { EM_COMBINE(8) } break;
    case 16: { EM_COMBINE(16) } break;
    default: { EM_COMBINE(32) } break;
    }
#undef EM_COMBINE
}

} // namespace
} // namespace em
