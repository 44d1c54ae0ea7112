// Extended field-line tracer: lines seeded around charges, stopped within a
// radius of a negative charge, at a zero/invalid field or at a per-line step
// limit.  The stepping rule is the reference's (CPU_Implement.cpp:322-338:
// curvature against the line's seed, unit field step scaled by 1/(k+1)).
//
// Work decomposition.  A lane group (TPL lanes) owns one line at a time and
// splits its charge sum; the warp's groups advance in lockstep, one field
// evaluation per step-iteration.  When lines end, the warp ballots its
// finished groups and takes that many new lines from a device work queue
// with a single atomic (warp-ballot compaction), so lanes never idle while
// lines remain.
//
// Charges are staged negatives-first, each block padded to the loop granule:
// only the negative block tracks the nearest negative charge (one FMNMX per
// pair).  Charges sit in shared memory: staged once when they fit, otherwise
// streamed through a ring of tiles by a producer warp, with the CTA stepping
// in lockstep (one CTA-wide vote per step-iteration decides whether any line
// is left).
//
// Precision modes (template MODE):
//   EXT_FAST   T = float or double: r^2 by FMA, reciprocal square root,
//              s = q inv^3, a += s r.  With T = double this is the all-FP64
//              path.
//   EXT_MIXED  T = float pair sums with a first-order Newton correction of
//              inv^3 (s = s0 (2.5 - 1.5 r^2 inv^2), removing the rsqrt error
//              to first order), two-sum compensated accumulation across
//              chunks of 64 charges and across lanes, the line position in
//              FP64, and a double-float (or, with refine_fp64, FP64)
//              re-evaluation of the whole field where the sum is
//              ill-conditioned: sum_j |t_j|^2 > kappa^2 |E|^2.
//   EXT_DF64   T = float: double-float pairs (two FP32 words each, about
//              48 bits; the FP32 vertex makes r = p - c exact), compensated
//              sums, the field and the step in FP64, the position in FP64:
//              FP64-class fields on the FP32 pipes.
#include "em_device.cuh"
#include "em_ext.cuh"
#include "em_internal.h"
#include "em_math.cuh"

namespace em {
namespace {

// ---------------------------------------------------------------------------
// Staging: stable partition of p raw records into
//   [negatives | pad to gran][positives | pad to p_pad], one CTA of 1024.
// block > 0 (the mixed mode): in the paired layout, blocks of `block`
// records, each the block's A plane {xa, xb, ya, yb} then its B plane
// {za, zb, qa, qb} (record pairs 2i, 2i + 1 of the block).
// meta[0] = size of the padded negative block (records).
// qabs[0] = largest |q| (float).
template <class T>
__device__ __forceinline__ void stage_put(T *staged, int block, int r, T x, T y, T z, T q)
{
    if (block == 0) {
        T *d = staged + 4 * (size_t)r;
        d[0] = x;
        d[1] = y;
        d[2] = z;
        d[3] = q;
        return;
    }
    const int b = r / block, i = r - b * block, jp = i >> 1, h = i & 1;
    T *A = staged + 4 * ((size_t)b * block + jp);
    T *B = staged + 4 * ((size_t)b * block + block / 2 + jp);
    A[h] = x;
    A[2 + h] = y;
    B[h] = z;
    B[2 + h] = q;
}

template <class T>
__global__ void __launch_bounds__(1024)
    ext_stage_kernel(const T *raw, int p, T *staged, int p_pad, int gran, int block, int *meta,
                     float *qabs)
{
    __shared__ int scan[1024];
    __shared__ float qm[32];
    const int tid = threadIdx.x;
    const int per = (p + 1023) / 1024;
    const int b = tid * per, e = min(p, b + per);
    int neg = 0;
    float qmax = 0;
    for (int i = b; i < e; ++i) {
        const T q = raw[4 * (size_t)i + 3];
        neg += q < T(0);
        qmax = fmaxf(qmax, fabsf((float)q));
    }
    scan[tid] = neg;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = tid >= off ? scan[tid - off] : 0;
        __syncthreads();
        scan[tid] += v;
        __syncthreads();
    }
    const int total_neg = scan[1023];
    const int neg_pad = (total_neg + gran - 1) / gran * gran;
    int wn = scan[tid] - neg;       // negatives before this chunk
    int wp = neg_pad + (b - wn);    // positives go after the padded block
    if (b > p)
        wp = neg_pad;
    for (int i = b; i < e; ++i) {
        const T *r = raw + 4 * (size_t)i;
        stage_put(staged, block, r[3] < T(0) ? wn++ : wp++, r[0], r[1], r[2], r[3]);
    }
    // pad records {1e15, 1e15, 1e15, 0}: exactly zero contribution
    const int pos_end = neg_pad + (p - total_neg);
    for (int i = tid; i < p_pad; i += 1024) {
        if ((i >= total_neg && i < neg_pad) || i >= pos_end)
            stage_put(staged, block, i, T(1e15), T(1e15), T(1e15), T(0));
    }
    for (int o = 16; o; o >>= 1)
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, o));
    if ((tid & 31) == 0)
        qm[tid >> 5] = qmax;
    __syncthreads();
    if (tid == 0) {
        float m = 0;
        for (int w = 0; w < 32; ++w)
            m = fmaxf(m, qm[w]);
        meta[0] = neg_pad;
        *qabs = m;
    }
}

// The group's field once its lanes are combined: times K, and in the
// double-float mode the FP64 field from the two words of each sum.
template <class T, int MODE>
__device__ __forceinline__ void ext_field(T &ax, T &ay, T &az, const CF &hx, const CF &hy,
                                          const CF &hz, double &Edx, double &Edy, double &Edz)
{
    Edx = Edy = Edz = 0;
    if constexpr (MODE == EXT_MIXED) {
        // the sums are in the packed terms' scaled units: times kMixScale
        // and the Coulomb constant, a double-float pair, rounded once
        constexpr double kScale = kMixScale * kElectroK;
        constexpr float kScaleH = (float)kScale;
        constexpr float kScaleL = (float)(kScale - (double)kScaleH);
        ax = fmaf(hx.h, kScaleH, fmaf(hx.h, kScaleL, hx.l * kScaleH));
        ay = fmaf(hy.h, kScaleH, fmaf(hy.h, kScaleL, hy.l * kScaleH));
        az = fmaf(hz.h, kScaleH, fmaf(hz.h, kScaleL, hz.l * kScaleH));
        return;
    }
    const T K = (T)kElectroK;
    ax = mul_rn(ax, K);
    ay = mul_rn(ay, K);
    az = mul_rn(az, K);
    if constexpr (MODE == EXT_DF64) {
        Edx = ((double)hx.h + (double)hx.l) * kElectroK;
        Edy = ((double)hy.h + (double)hy.l) * kElectroK;
        Edz = ((double)hz.h + (double)hz.l) * kElectroK;
        ax = (T)Edx;
        ay = (T)Edy;
        az = (T)Edz;
    }
}

// The mixed mode's test of the FP32 sum's conditioning: l2 = sum_j q_j^2 /
// r_j^4 (no Coulomb constant), (ax, ay, az) the field with it; true where
// sqrt(l2) K > kappa |E|.
template <class T>
__device__ __forceinline__ bool ext_ill_conditioned(const ExtParams<T> &P, float l2, T ax, T ay,
                                                    T az)
{
    const double e2 = (double)ax * ax + (double)ay * ay + (double)az * az;
    return (double)l2 * (kElectroK * kElectroK) > P.kappa2 * e2;
}

// One vertex of a live line once its field is known: the field store, the
// termination tests, the step (the reference rule in the mode's arithmetic,
// curvature against the seed r0) and the vertex store; lane t == 0 of the
// group stores.  Returns the termination class, or -1 if the line goes on
// (s then names its next row).
template <class T, int MODE>
__device__ __forceinline__ int ext_vertex(const ExtParams<T> &P, long long line, int &s, int lim,
                                          ExtLane<T> &st, int t, T ax, T ay, T az, double Edx,
                                          double Edy, double Edz, T dneg, T r0x, T r0y, T r0z)
{
    const size_t n = (size_t)P.n;
    const size_t row = (size_t)(s - 1) * n + (size_t)line;
    if (P.ex && t == 0) {
        P.ex[row] = ax;
        P.ey[row] = ay;
        P.ez[row] = az;
    }
    if (dneg < (T)P.term_r2)
        return EM_TERM_CHARGE_DEV;
    T sx, sy, sz, k2;
    T nx, ny, nz;
    if constexpr (MODE == EXT_DF64) {
        // the step in FP64 from the FP64 field
        double dsx, dsy, dsz, dk2;
        step_vector<double>(Edx, Edy, Edz, (double)r0x, (double)r0y, (double)r0z, P.resolution,
                            dsx, dsy, dsz, dk2);
        k2 = (T)dk2;
        if (dk2 > 0.0 && !(k2 > T(0)))
            k2 = T(1); // a positive FP64 |E|^2 below the FP32 range
        st.dx += dsx;
        st.dy += dsy;
        st.dz += dsz;
        nx = (T)st.dx;
        ny = (T)st.dy;
        nz = (T)st.dz;
    } else if constexpr (MODE == EXT_MIXED) {
        step_vector<T>(ax, ay, az, r0x, r0y, r0z, (T)P.resolution, sx, sy, sz, k2);
        st.dx += (double)sx;
        st.dy += (double)sy;
        st.dz += (double)sz;
        nx = (T)st.dx;
        ny = (T)st.dy;
        nz = (T)st.dz;
    } else {
        step_vector<T>(ax, ay, az, r0x, r0y, r0z, (T)P.resolution, sx, sy, sz, k2);
        nx = add_rn(st.px, sx);
        ny = add_rn(st.py, sy);
        nz = add_rn(st.pz, sz);
    }
    if (!(k2 > T(0)) || !isfinite(nx) || !isfinite(ny) || !isfinite(nz))
        return EM_TERM_NULL_DEV;
    st.px = nx;
    st.py = ny;
    st.pz = nz;
    const size_t w = (size_t)s * n + (size_t)line;
    if (t == 0) {
        store_stream(P.x + w, nx);
        store_stream(P.y + w, ny);
        store_stream(P.z + w, nz);
    }
    ++s;
    return s >= lim ? EM_TERM_STEPS_DEV : -1;
}

__device__ __forceinline__ void live_count_drop(unsigned long long *c)
{
    atomicAdd(c, ~0ull); // minus one
}

template <class T, int TPL, int MODE>
__global__ void __launch_bounds__(ext_cta_threads(MODE), 1)
    ext_trace_kernel(const ExtParams<T> P)
{
    using Rec = typename ChargeRec<T>::type;
    constexpr int LG = 32 / TPL; // line slots per warp
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
    const int jneg_all = *P.meta; // padded negative block (records)

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
        // ---- producer: tiles of every step-iteration while any line lives ---
        const uint32_t tb = (uint32_t)P.tile_recs * (uint32_t)sizeof(Rec);
        const char *src = static_cast<const char *>(P.charges);
        uint32_t it = 0;
        bool ok = true;
        while (__syncthreads_or(0)) {
            if (lane == 0 && ok && *(volatile int *)P.err == 0) {
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
            }
            __syncwarp();
        }
        if (lane == 0) {
            for (uint32_t k = 0; k < (uint32_t)NST && k < it; ++k) {
                const uint32_t j = it - 1 - k;
                mbar_wait(full0 + 8 * (j % NST), (j / NST) & 1, P.err);
            }
        }
        return;
    }

    // ---- line slots ------------------------------------------------------------
    int tg = TPL;                   // current lanes per line
    int t = lane & (tg - 1);
    const long long total_slots = (long long)gridDim.x * ncw * LG;
    bool queue_empty = total_slots >= P.n;
    long long line = ((long long)blockIdx.x * ncw + warp) * LG + lane / TPL;
    int s = 1, lim = 0;
    ExtLane<T> st;
    st.px = st.py = st.pz = 0;
    st.dx = st.dy = st.dz = 0;
    unsigned long long evals = 0, refines = 0;

    // Loads line `l`'s seed and limit; returns false if the line needs no
    // evaluation (limit < 2), after recording its result.
    auto start_line = [&](long long l) -> bool {
        st.px = P.x[l];
        st.py = P.y[l];
        st.pz = P.z[l];
        st.dx = (double)st.px;
        st.dy = (double)st.py;
        st.dz = (double)st.pz;
        lim = P.max_steps;
        if (P.steps_per_line)
            lim = max(1, min(P.steps_per_line[l], P.max_steps));
        s = 1;
        if (lim < 2) {
            if (t == 0) {
                P.len[l] = 1;
                P.cls[l] = EM_TERM_STEPS_DEV;
                if (P.tail_lines > 0)
                    live_count_drop(P.live_count);
            }
            return false;
        }
        return true;
    };

    bool live = line < P.n && start_line(line);
    bool need = line < P.n && !live; // slot needs a new line
    if (line >= P.n)
        line = -1;
    // refill (warp-ballot): finished slots take new lines with one atomic
    auto refill = [&]() {
        for (int guard = 0; guard < 1 << 20; ++guard) {
            const unsigned m = __ballot_sync(0xffffffffu, t == 0 && need);
            if (!m)
                break;
            const int first = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == first)
                base = atomicAdd(P.next_line, (unsigned long long)__popc(m));
            base = __shfl_sync(0xffffffffu, base, first);
            if ((long long)(base + __popc(m)) + total_slots >= P.n)
                queue_empty = true;
            const long long mine =
                (long long)(base + __popc(m & ((1u << lane) - 1u))) + total_slots;
            const long long nl = __shfl_sync(0xffffffffu, mine, lane - t);
            if (need) {
                if (nl < P.n) {
                    line = nl;
                    live = start_line(line);
                    need = !live;
                } else {
                    line = -1;
                    live = false;
                    need = false;
                }
            }
        }
    };
    refill();

    // With no lines left to hand out, a warp whose live lines fit in half
    // of its groups compacts them into wider groups (more lanes per line),
    // so the last, longest lines run on more lanes.
    auto regroup = [&]() {
        if (!P.regroup || !queue_empty || tg >= 32)
            return;
        const unsigned lead = __ballot_sync(0xffffffffu, t == 0 && live);
        const int nlive = __popc(lead);
        int ng = tg;
        while (ng < 32 && nlive <= (32 / ng) / 2)
            ng *= 2;
        if (ng == tg)
            return;
        const int k = lane / ng;
        const bool has = k < nlive;
        const int src = has ? (int)__fns(lead, 0, k + 1) : 0;
        line = __shfl_sync(0xffffffffu, line, src);
        s = __shfl_sync(0xffffffffu, s, src);
        lim = __shfl_sync(0xffffffffu, lim, src);
        st.px = __shfl_sync(0xffffffffu, st.px, src);
        st.py = __shfl_sync(0xffffffffu, st.py, src);
        st.pz = __shfl_sync(0xffffffffu, st.pz, src);
        st.dx = __shfl_sync(0xffffffffu, st.dx, src);
        st.dy = __shfl_sync(0xffffffffu, st.dy, src);
        st.dz = __shfl_sync(0xffffffffu, st.dz, src);
        live = has;
        need = false;
        if (!has)
            line = -1;
        tg = ng;
        t = lane & (tg - 1);
    };
    regroup();

    uint32_t it = 0;
    bool failed = false;
    unsigned tail_iter = 0;
    bool tail_check = false;
    bool in_ring = true; // streamed: still consuming the tile ring
    unsigned long long live_seen = 0, next_seen = 0;
    for (;;) {
        const bool any = streamed ? __syncthreads_or(live) != 0 : __any_sync(0xffffffffu, live);
        if (!any)
            break;
        const bool wlive = __any_sync(0xffffffffu, live);
        if (streamed && in_ring && !wlive && queue_empty) {
            // no line now and none to come: leave the tile ring (every tile
            // of the rows so far is consumed; the producer's later waits
            // count one consumer fewer) instead of waiting on every tile
            __syncwarp();
            if (lane == 0)
                for (int k = 0; k < NST; ++k)
                    mbar_arrive_drop(empty0 + 8 * k);
            in_ring = false;
        }
        // every 8th iteration lane 0 reads the queue head (a warp whose lines
        // all run long would otherwise learn that the queue is dry only when
        // one of them ends) and, with the hand-off, the number of lines still
        // traced here; used after the pair loop, so the loads' latency hides
        // under it
        if ((++tail_iter & 7) == 0 && (!queue_empty || P.tail_lines > 0)) {
            tail_check = true;
            if (lane == 0) {
                next_seen = *(volatile unsigned long long *)P.next_line;
                if (P.tail_lines > 0)
                    live_seen = *(volatile unsigned long long *)P.live_count;
            }
        }
        // ---- field (and nearest negative charge) at the current vertex -----
        T ax = 0, ay = 0, az = 0, dneg = T(3.0e38);
        float dall = 0.0f; // mixed: sum of q^2/r^4 over the pairs
        CF hx, hy, hz;
        if (!streamed) {
            tile_pairs<T, MODE>(tg, tiles, jneg_all, P.p_pad, t, st, ax, ay, az, dneg, dall, hx,
                                hy, hz);
        } else {
            for (int tile = 0; in_ring && tile < P.n_tiles; ++tile, ++it) {
                const uint32_t sg = it % NST, ph = (it / NST) & 1;
                // on a failed wait the warp stops computing but keeps voting,
                // so the CTA-wide loop still ends for every thread
                if (!failed && !mbar_wait(full0 + 8 * sg, ph, P.err))
                    failed = true;
                if (!failed) {
                    const int base = tile * P.tile_recs;
                    const int jn = min(max(jneg_all - base, 0), P.tile_recs);
                    const Rec *tp = tiles + sg * P.tile_recs;
                    // a warp with no live line only keeps the tile ring
                    // turning (the CTA runs while any of its lines lives)
                    if (wlive)
                        tile_pairs<T, MODE>(tg, tp, jn, P.tile_recs, t, st, ax, ay, az, dneg,
                                            dall, hx, hy, hz);
                    __syncwarp();
                    if (lane == 0)
                        mbar_arrive(empty0 + 8 * sg);
                }
            }
            if (failed) {
                live = false;
                need = false;
                line = -1;
                continue;
            }
        }
        // ---- combine the group's lanes -------------------------------------
        combine_group<T, MODE>(tg, ax, ay, az, dneg, dall, hx, hy, hz);
        double Edx, Edy, Edz;
        ext_field<T, MODE>(ax, ay, az, hx, hy, hz, Edx, Edy, Edz);

        if constexpr (MODE == EXT_MIXED) {
            // the FP32 sum's error grows with the size of its terms: where
            // sum |t_j|^2 > kappa^2 |E|^2 (cancellation, nulls) redo the field
            // in double-float (on the FP32 pipes) or, with refine_fp64, FP64
            const bool redo = live && ext_ill_conditioned(P, dall, ax, ay, az);
            // each flagged vertex in turn, its field split over the whole
            // warp (records from shared memory when resident)
            unsigned m = __ballot_sync(0xffffffffu, redo && t == 0);
            const float4 *rec = streamed ? reinterpret_cast<const float4 *>(P.charges)
                                         : reinterpret_cast<const float4 *>(tiles);
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                const float rx = __shfl_sync(0xffffffffu, (float)st.px, src);
                const float ry = __shfl_sync(0xffffffffu, (float)st.py, src);
                const float rz = __shfl_sync(0xffffffffu, (float)st.pz, src);
                double fx = 0, fy = 0, fz = 0;
                if (!P.refine_fp64)
                    field_pk<32, false>(rec, P.stage_recs, 0, P.p_pad / 2, lane, rx, ry, rz, fx,
                                        fy, fz);
                else
                    field_pk<32, true>(rec, P.stage_recs, 0, P.p_pad / 2, lane, rx, ry, rz, fx,
                                       fy, fz);
                fx = group_sum<double, 32>(fx);
                fy = group_sum<double, 32>(fy);
                fz = group_sum<double, 32>(fz);
                if (lane / tg == src / tg) {
                    ax = (T)(fx * kElectroK);
                    ay = (T)(fy * kElectroK);
                    az = (T)(fz * kElectroK);
                }
                refines += (lane == src);
            }
        }
        // tail hand-off: with the queue dry, once few enough lines are left
        // the warp's lines go to the tail kernels (warp-uniform decision)
        bool hand_off = false;
        if (tail_check) {
            const unsigned long long ns = __shfl_sync(0xffffffffu, next_seen, 0);
            if ((long long)ns + total_slots >= P.n)
                queue_empty = true;
            if (P.tail_lines > 0)
                hand_off = queue_empty && __shfl_sync(0xffffffffu, live_seen, 0) <=
                                              (unsigned long long)P.tail_lines;
            tail_check = false;
        }
        if (live) {
            evals += (t == 0);
            const int cls = ext_vertex<T, MODE>(P, line, s, lim, st, t, ax, ay, az, Edx, Edy,
                                                Edz, dneg, ld_seed(P.x + line),
                                                ld_seed(P.y + line), ld_seed(P.z + line));
            if (cls >= 0) {
                if (t == 0) {
                    P.len[line] = s;
                    P.cls[line] = cls;
                    if (P.tail_lines > 0)
                        live_count_drop(P.live_count);
                }
                live = false;
                need = true;
            } else if (hand_off) {
                if (t == 0) {
                    const unsigned long long k = atomicAdd(P.cont_count, 1ull);
                    ExtCont<T> c;
                    c.line = line;
                    c.s = s;
                    c.lim = lim;
                    c.px = st.px;
                    c.py = st.py;
                    c.pz = st.pz;
                    c.dx = st.dx;
                    c.dy = st.dy;
                    c.dz = st.dz;
                    static_cast<ExtCont<T> *>(P.cont)[k] = c;
                    live_count_drop(P.live_count);
                }
                live = false;
                need = true;
            }
        }
        refill();
        regroup();
    }
    // counters: one atomic per warp
    for (int o = 16; o; o >>= 1) {
        evals += __shfl_xor_sync(0xffffffffu, evals, o);
        refines += __shfl_xor_sync(0xffffffffu, refines, o);
    }
    if (lane == 0) {
        atomicAdd(P.evals, evals);
        if (refines)
            atomicAdd(P.refines, refines);
    }
}

// Four warp-wide reductions at once — sums of a, b, c and the minimum of d
// — in six shuffles instead of twenty: at offsets 16 and 8 each lane hands
// its partner the half of its values the partner keeps, then three full
// levels; lane 8i ends with value i (a, b, c, d), as do the other lanes of
// its block of eight.
__device__ __forceinline__ float warp_reduce4(float a, float b, float c, float d, int lane)
{
    const unsigned FULL = 0xffffffffu;
    const bool h16 = lane & 16, h8 = lane & 8;
    float k0 = h16 ? c : a, k1 = h16 ? d : b;
    const float r0 = __shfl_xor_sync(FULL, h16 ? a : c, 16);
    const float r1 = __shfl_xor_sync(FULL, h16 ? b : d, 16);
    k0 = k0 + r0;
    k1 = h16 ? fminf(k1, r1) : k1 + r1;
    float k = h8 ? k1 : k0;
    const float r = __shfl_xor_sync(FULL, h8 ? k0 : k1, 8);
    const bool mn = h16 && h8;
    k = mn ? fminf(k, r) : k + r;
#pragma unroll
    for (int o = 4; o >= 1; o >>= 1) {
        const float q = __shfl_xor_sync(FULL, k, o);
        k = mn ? fminf(k, q) : k + q;
    }
    return k;
}

// The compensated modes' per-warp sums — three (hi, lo) sums X, Y, Z and an
// item W of the nearest negative distance^2 (minimum) and sum q^2/r^4 — in
// twelve shuffles instead of forty: at offsets 16 and 8 each lane hands its
// partner the half of its items the partner keeps, then three full levels
// with the operands ordered by lane half (both partners get the same bits);
// lane 8i ends with item i as (f, g): (hi, lo), or (dneg, l2) for W.
__device__ __forceinline__ void warp_reduce_cf(const CF &x, const CF &y, const CF &z, float dneg,
                                               float l2, int lane, float &f, float &g)
{
    const unsigned FULL = 0xffffffffu;
    auto cf = [](float ah, float al, float bh, float bl, float &h, float &l) {
        float sum, err;
        two_sum(ah, bh, sum, err);
        h = sum;
        l = __fadd_rn(__fadd_rn(al, bl), err);
    };
    const bool h16 = lane & 16, h8 = lane & 8;
    // offset 16: the lower half keeps X and Y, the upper half Z and W
    float k0h = h16 ? z.h : x.h, k0l = h16 ? z.l : x.l;
    float k1h = h16 ? dneg : y.h, k1l = h16 ? l2 : y.l;
    const float s0h = __shfl_xor_sync(FULL, h16 ? x.h : z.h, 16);
    const float s0l = __shfl_xor_sync(FULL, h16 ? x.l : z.l, 16);
    const float s1h = __shfl_xor_sync(FULL, h16 ? y.h : dneg, 16);
    const float s1l = __shfl_xor_sync(FULL, h16 ? y.l : l2, 16);
    cf(k0h, k0l, s0h, s0l, k0h, k0l);
    if (h16) {
        k1h = fminf(k1h, s1h);
        k1l = __fadd_rn(k1l, s1l);
    } else {
        cf(k1h, k1l, s1h, s1l, k1h, k1l);
    }
    // offset 8: item i = 2 h16 + h8 stays
    float ih = h8 ? k1h : k0h, il = h8 ? k1l : k0l;
    const float rh = __shfl_xor_sync(FULL, h8 ? k0h : k1h, 8);
    const float rl = __shfl_xor_sync(FULL, h8 ? k0l : k1l, 8);
    const bool w = h16 && h8;
    if (w) {
        ih = fminf(ih, rh);
        il = __fadd_rn(il, rl);
    } else {
        cf(ih, il, rh, rl, ih, il);
    }
#pragma unroll
    for (int o = 4; o >= 1; o >>= 1) {
        const float oh = __shfl_xor_sync(FULL, ih, o);
        const float ol = __shfl_xor_sync(FULL, il, o);
        const bool up = lane & o;
        const float ah = up ? oh : ih, bh = up ? ih : oh;
        const float al = up ? ol : il, bl = up ? il : ol;
        if (w) {
            ih = fminf(ah, bh);
            il = __fadd_rn(al, bl);
        } else {
            cf(ah, al, bh, bl, ih, il);
        }
    }
    f = ih;
    g = il;
}

// The four totals over a group of 16 warps from their slots (x, y, z: sums;
// w: minimum), in every lane, in nine shuffles: lanes l and l + 16 hold slot
// l mod 16; offsets 8 and 4 trade halves, 2 and 1 finish, and each total is
// read from a lane that holds it.  Every warp of the group gets the same
// bits (the same operations on the same slots).
__device__ __forceinline__ void slots_reduce16(float4 v, int lane, float &a, float &b, float &c,
                                               float &d)
{
    const unsigned FULL = 0xffffffffu;
    const bool h8 = lane & 8, h4 = lane & 4;
    float k0 = h8 ? v.z : v.x, k1 = h8 ? v.w : v.y;
    const float r0 = __shfl_xor_sync(FULL, h8 ? v.x : v.z, 8);
    const float r1 = __shfl_xor_sync(FULL, h8 ? v.y : v.w, 8);
    k0 = k0 + r0;
    k1 = h8 ? fminf(k1, r1) : k1 + r1;
    float k = h4 ? k1 : k0;
    const float r = __shfl_xor_sync(FULL, h4 ? k0 : k1, 4);
    const bool mn = h8 && h4;
    k = mn ? fminf(k, r) : k + r;
#pragma unroll
    for (int o = 2; o >= 1; o >>= 1) {
        const float q = __shfl_xor_sync(FULL, k, o);
        k = mn ? fminf(k, q) : k + q;
    }
    a = __shfl_sync(FULL, k, 0);
    b = __shfl_sync(FULL, k, 4);
    c = __shfl_sync(FULL, k, 8);
    d = __shfl_sync(FULL, k, 12);
}

// ---------------------------------------------------------------------------
// The handed-off lines with streamed charges, W = P.wide warps per line (a
// group); the groups of a CTA share the tile ring, so they step in
// lockstep, three CTA barriers per row.  Warp w of a group sums the charges
// of its W-th of each tile with all 32 lanes; the warps' sums meet in shared
// memory, the group's first warp (its lead) combines them, runs the vertex
// step and publishes the new vertex, which the other warps read after the
// row's last barrier.  A group whose line ends takes the next handed-off
// line.  (Resident charges: ext_wide_res_kernel.)
template <class T, int MODE>
__global__ void __launch_bounds__(kExtWideThreads, 1) ext_wide_kernel(const ExtParams<T> P)
{
    using Rec = typename ChargeRec<T>::type;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ T slots[32][8];       // each warp's sums (T words, no conversions)
    __shared__ double rslots[32][4]; // each warp's re-evaluation sums
    __shared__ long long grp_next[32];
    __shared__ T grp_pos[32][3];     // the lead's vertex after the step
    __shared__ int grp_flag[32];     // 1: the line goes on; 2: re-evaluate
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    Rec *tiles = reinterpret_cast<Rec *>(smem + 128);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int ncw = nwarps - 1;
    const int NST = P.stages;
    const int W = P.wide;
    if (P.resident || NST > 8 || ncw < 1 || ncw > 32 || W < 1 || ncw % W != 0) {
        if (threadIdx.x == 0)
            atomicCAS(P.err, 0, EM_DEVERR_CONFIG);
        return;
    }
    const uint32_t full0 = smem_addr(bars), empty0 = smem_addr(bars + 8);
    if (threadIdx.x == 0) {
        for (int k = 0; k < NST; ++k) {
            mbar_init(full0 + 8 * k, 1);
            mbar_init(empty0 + 8 * k, ncw);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int jneg_all = *P.meta;
    const long long count = (long long)*P.cont_in_count;
    const ExtCont<T> *cont = static_cast<const ExtCont<T> *>(P.cont_in);
    __shared__ unsigned long long sh_live;

    if (warp == nwarps - 1) {
        // ---- producer: the tiles of every row while any group has a line;
        // it passes the consumers' CTA barriers in the same order
        __syncthreads(); // first lines taken
        const uint32_t tb = (uint32_t)P.tile_recs * (uint32_t)sizeof(Rec);
        const char *src = static_cast<const char *>(P.charges);
        uint32_t it = 0;
        bool ok = true;
        while (__syncthreads_or(0)) {
            if (lane == 0 && ok && *(volatile int *)P.err == 0) {
                for (int tile = 0; tile < P.n_tiles; ++tile, ++it) {
                    const uint32_t sg = it % NST, ph = (it / NST) & 1;
                    if (it >= (uint32_t)NST && !mbar_wait(empty0 + 8 * sg, ph ^ 1, P.err)) {
                        ok = false;
                        break;
                    }
                    // the last tile may be shorter (tiles of several staged
                    // tiles; p_pad is a multiple of the staged tile)
                    const uint32_t bytes =
                        (uint32_t)min(P.tile_recs, P.p_pad - tile * P.tile_recs) *
                        (uint32_t)sizeof(Rec);
                    mbar_arrive_expect_tx(full0 + 8 * sg, bytes);
                    bulk_g2s(smem_addr(tiles) + sg * tb, src + (size_t)tile * tb, bytes,
                             full0 + 8 * sg);
                }
            }
            __syncwarp();
            __syncthreads_or(0); // the warps' sums are in the slots
            if constexpr (MODE == EXT_MIXED) {
                if (__syncthreads_or(0))
                    __syncthreads(); // re-evaluation sums
            }
            __syncthreads(); // next lines taken
        }
        if (lane == 0) {
            for (uint32_t k = 0; k < (uint32_t)NST && k < it; ++k) {
                const uint32_t j = it - 1 - k;
                mbar_wait(full0 + 8 * (j % NST), (j / NST) & 1, P.err);
            }
        }
        return;
    }

    // ---- consumers --------------------------------------------------------
    const int g = warp / W, wg = warp - g * W;
    const bool lead = wg == 0;
    const int t = wg * 32 + lane; // thread index within the group
    long long line = -1;
    int s = 1, lim = 0;
    bool live = false;
    ExtLane<T> st;
    st.px = st.py = st.pz = 0;
    st.dx = st.dy = st.dz = 0;
    unsigned long long evals = 0, refines = 0;
    auto take = [&]() {
        const long long k = grp_next[g];
        if (k < count) {
            const ExtCont<T> c = cont[k];
            line = c.line;
            s = c.s;
            lim = c.lim;
            st.px = c.px;
            st.py = c.py;
            st.pz = c.pz;
            st.dx = c.dx;
            st.dy = c.dy;
            st.dz = c.dz;
            live = true;
        } else {
            line = -1;
            live = false;
        }
    };
    auto save = [&]() {
        const unsigned long long k = atomicAdd(P.cont_count, 1ull);
        ExtCont<T> c;
        c.line = line;
        c.s = s;
        c.lim = lim;
        c.px = st.px;
        c.py = st.py;
        c.pz = st.pz;
        c.dx = st.dx;
        c.dy = st.dy;
        c.dz = st.dz;
        static_cast<ExtCont<T> *>(P.cont)[k] = c;
    };
    if (lead && lane == 0)
        grp_next[g] = (long long)atomicAdd(P.cont_next, 1ull);
    __syncthreads(); // first lines taken
    take();

    // this warp's W-th of the staged records (the re-evaluation's share), of
    // a full wide tile and of the last, shorter one: fixed for the whole
    // launch, so no division per row or tile
    const int pb = (int)((long long)P.p_pad * wg / W);
    const int pe = (int)((long long)P.p_pad * (wg + 1) / W);
    const int last_recs = P.p_pad - (P.n_tiles - 1) * P.tile_recs;
    const int tb_ = (int)((long long)P.tile_recs * wg / W);
    const int te = (int)((long long)P.tile_recs * (wg + 1) / W);
    const int lb = (int)((long long)last_recs * wg / W);
    const int le = (int)((long long)last_recs * (wg + 1) / W);
    // mixed: the warp's W-th of all staged charge pairs (the
    // re-evaluation's share)
    const int rb = (int)((long long)(P.p_pad / 2) * wg / W);
    const int re = (int)((long long)(P.p_pad / 2) * (wg + 1) / W);

    uint32_t it = 0;
    bool failed = false;
    bool in_ring = true; // still consuming the tile ring
    unsigned row_iter = 0;
    for (;;) {
        if (!__syncthreads_or(live))
            break;
        if (in_ring && !live) {
            // a group without a line now has none to come: its warps leave
            // the tile ring (all tiles of earlier rows are consumed)
            if (lane == 0)
                for (int k = 0; k < NST; ++k)
                    mbar_arrive_drop(empty0 + 8 * k);
            in_ring = false;
        }
        // every 8th row: are few enough lines left to hand them on to a
        // wider launch?  (read here, used after the next barrier)
        const bool tail_check = P.tail_lines > 0 && (++row_iter & 7) == 0;
        if (tail_check && threadIdx.x == 0)
            sh_live = *(volatile unsigned long long *)P.live_count;
        // the seed (the lead's curvature reference), read while the pairs run
        T r0x = 0, r0y = 0, r0z = 0;
        if (lead && live) {
            r0x = ld_seed(P.x + line);
            r0y = ld_seed(P.y + line);
            r0z = ld_seed(P.z + line);
        }
        T ax = 0, ay = 0, az = 0, dneg = T(3.0e38);
        float dall = 0.0f; // mixed: sum of q^2/r^4 over the pairs
        CF hx, hy, hz;
        for (int tile = 0; in_ring && tile < P.n_tiles; ++tile, ++it) {
            const uint32_t sg = it % NST, ph = (it / NST) & 1;
            if (!failed && !mbar_wait(full0 + 8 * sg, ph, P.err))
                failed = true;
            if (!failed) {
                const int base = tile * P.tile_recs;
                const bool last_tile = tile == P.n_tiles - 1;
                const int b = last_tile ? lb : tb_, e = last_tile ? le : te;
                if constexpr (MODE == EXT_MIXED) {
                    // paired blocks of the staged tile size: the warp's
                    // W-th of the wide tile's charge pairs [b/2, e/2), block
                    // by block
                    const int SR = P.stage_recs, half = SR / 2;
                    const ulonglong2 *blk =
                        reinterpret_cast<const ulonglong2 *>(tiles + sg * P.tile_recs);
                    for (int k = (b / 2) / half; live && k * half < e / 2; ++k) {
                        const int lo = max(b / 2 - k * half, 0);
                        const int hi = min(e / 2 - k * half, half);
                        const int jk = min(max(jneg_all - (base + k * SR), 0), SR);
                        const ulonglong2 *Ak = blk + (size_t)k * SR;
                        mixed_pk<32>(Ak, Ak + half, jk / 2, lo, hi, lane, st.px, st.py, st.pz,
                                     hx, hy, hz, dneg, dall);
                    }
                } else {
                    const int jt = min(max(jneg_all - base, 0), P.tile_recs);
                    const int jn = min(max(jt - b, 0), e - b);
                    if (live)
                        tile_pairs<T, MODE>(32, tiles + sg * P.tile_recs + b, jn, e - b, lane,
                                            st, ax, ay, az, dneg, dall, hx, hy, hz);
                }
                __syncwarp();
                if (lane == 0)
                    mbar_arrive(empty0 + 8 * sg);
            }
        }
        // ---- each warp's sums into the slots (words 0..5 the field, 6 dneg,
        // 7 l2), the values reduced together where they are FP32 words
        if constexpr (MODE == EXT_MIXED || MODE == EXT_DF64) {
            float f, g2;
            warp_reduce_cf(hx, hy, hz, dneg, dall, lane, f, g2);
            if ((lane & 7) == 0) {
                slots[warp][2 * (lane >> 3)] = f;
                slots[warp][2 * (lane >> 3) + 1] = g2;
            }
        } else if constexpr (sizeof(T) == 4) {
            const float k = warp_reduce4(ax, ay, az, dneg, lane);
            if ((lane & 7) == 0)
                slots[warp][lane == 24 ? 6 : lane >> 3] = k;
        } else {
            ax = group_sum<T, 32>(ax);
            ay = group_sum<T, 32>(ay);
            az = group_sum<T, 32>(az);
            dneg = group_min<T, 32>(dneg);
            if (lane == 0) {
                T *o = slots[warp];
                o[0] = ax;
                o[1] = ay;
                o[2] = az;
                o[6] = dneg;
            }
        }
        // a wait that gave up in any warp stops every group (CTA-uniform)
        if (__syncthreads_or(failed)) {
            live = false;
            failed = true;
        }
        const bool hand_off = tail_check && sh_live <= (unsigned long long)P.tail_lines;
        // ---- the lead combines the group's sums (lane w takes warp w's) ----
        double Edx = 0, Edy = 0, Edz = 0;
        bool redo = false;
        if (lead) {
            const T *gs = slots[g * W + (lane < W ? lane : 0)];
            const bool mine = lane < W;
            if constexpr (MODE == EXT_MIXED || MODE == EXT_DF64) {
                hx.h = mine ? gs[0] : 0.0f;
                hx.l = mine ? gs[1] : 0.0f;
                hy.h = mine ? gs[2] : 0.0f;
                hy.l = mine ? gs[3] : 0.0f;
                hz.h = mine ? gs[4] : 0.0f;
                hz.l = mine ? gs[5] : 0.0f;
                group_two_sum<32>(hx);
                group_two_sum<32>(hy);
                group_two_sum<32>(hz);
                ax = (T)__fadd_rn(hx.h, hx.l);
                ay = (T)__fadd_rn(hy.h, hy.l);
                az = (T)__fadd_rn(hz.h, hz.l);
                if constexpr (MODE == EXT_MIXED)
                    dall = group_sum<float, 32>(mine ? (float)gs[7] : 0.0f);
            } else {
                ax = group_sum<T, 32>(mine ? gs[0] : T(0));
                ay = group_sum<T, 32>(mine ? gs[1] : T(0));
                az = group_sum<T, 32>(mine ? gs[2] : T(0));
            }
            dneg = group_min<T, 32>(mine ? gs[6] : T(3.0e38));
            ext_field<T, MODE>(ax, ay, az, hx, hy, hz, Edx, Edy, Edz);
            if constexpr (MODE == EXT_MIXED) {
                redo = live && ext_ill_conditioned(P, dall, ax, ay, az);
                if (lane == 0)
                    grp_flag[g] = redo ? 2 : 0;
            }
        }
        if constexpr (MODE == EXT_MIXED) {
            // an ill-conditioned sum: the group re-evaluates the field in
            // double-float (or FP64), each warp its W-th of the staged records
            if (__syncthreads_or(redo)) {
                const bool gredo = grp_flag[g] == 2;
                double fx = 0, fy = 0, fz = 0;
                if (gredo) {
                    const float4 *cr = reinterpret_cast<const float4 *>(P.charges);
                    if (!P.refine_fp64)
                        field_pk<32, false>(cr, P.stage_recs, rb, re, lane, (float)st.px,
                                            (float)st.py, (float)st.pz, fx, fy, fz);
                    else
                        field_pk<32, true>(cr, P.stage_recs, rb, re, lane, (float)st.px,
                                           (float)st.py, (float)st.pz, fx, fy, fz);
                    fx = group_sum<double, 32>(fx);
                    fy = group_sum<double, 32>(fy);
                    fz = group_sum<double, 32>(fz);
                    if (lane == 0) {
                        rslots[warp][0] = fx;
                        rslots[warp][1] = fy;
                        rslots[warp][2] = fz;
                    }
                }
                __syncthreads();
                if (lead && redo) {
                    const double *gs = rslots[g * W + (lane < W ? lane : 0)];
                    const bool mine = lane < W;
                    fx = group_sum<double, 32>(mine ? gs[0] : 0.0);
                    fy = group_sum<double, 32>(mine ? gs[1] : 0.0);
                    fz = group_sum<double, 32>(mine ? gs[2] : 0.0);
                    ax = (T)(fx * kElectroK);
                    ay = (T)(fy * kElectroK);
                    az = (T)(fz * kElectroK);
                    refines += (lane == 0);
                }
            }
        }
        // ---- the lead's vertex step ----------------------------------------
        bool need = false;
        if (lead && live) {
            evals += (lane == 0);
            const int cls = ext_vertex<T, MODE>(P, line, s, lim, st, t, ax, ay, az, Edx, Edy,
                                                Edz, dneg, r0x, r0y, r0z);
            int flag = 1;
            if (cls >= 0) {
                if (lane == 0) {
                    P.len[line] = s;
                    P.cls[line] = cls;
                    if (P.tail_lines > 0)
                        live_count_drop(P.live_count);
                    grp_next[g] = (long long)atomicAdd(P.cont_next, 1ull);
                }
                flag = 0;
                need = true;
            } else if (hand_off) {
                // every input line was taken at the start (a group each),
                // so nothing is left behind
                if (lane == 0) {
                    save();
                    live_count_drop(P.live_count);
                }
                flag = 0;
            }
            if (lane == 0) {
                grp_flag[g] = flag | (need ? 4 : 0);
                grp_pos[g][0] = st.px;
                grp_pos[g][1] = st.py;
                grp_pos[g][2] = st.pz;
            }
        }
        __syncthreads(); // the leads' vertices and next lines are out
        if (live && !failed) {
            const int flag = grp_flag[g];
            if (flag & 4) {
                take();
            } else if (flag & 1) {
                if (!lead) {
                    st.px = grp_pos[g][0];
                    st.py = grp_pos[g][1];
                    st.pz = grp_pos[g][2];
                }
            } else {
                live = false;
            }
        }
    }
    // counters: one atomic per warp
    for (int o = 16; o; o >>= 1) {
        evals += __shfl_xor_sync(0xffffffffu, evals, o);
        refines += __shfl_xor_sync(0xffffffffu, refines, o);
    }
    if (lane == 0) {
        atomicAdd(P.evals, evals);
        if (refines)
            atomicAdd(P.refines, refines);
    }
}

// Barrier over the nthreads threads (whole warps) of one line group; id 1..15
// (0 is the CTA barrier).
__device__ __forceinline__ void group_barrier(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ---------------------------------------------------------------------------
// The handed-off lines with resident charges.  The same work as
// ext_wide_kernel, but the groups of a CTA run independently and a row costs
// one barrier, over the group only: each warp sums its W-th of the resident
// records and puts its sums into the row's slots (two sets, by row parity);
// after the barrier every warp of the group combines the W slots in the same
// order and runs the vertex step itself, so all of them hold the same vertex
// without a second exchange; warp 0, lane 0 of the group stores.  A group
// takes another barrier only where it needs one as a whole: a re-evaluation
// (mixed) and its next line's index.  The live-line count behind the
// hand-off test is loaded one row before it is used, off the row's chain.
template <class T, int MODE>
__global__ void __launch_bounds__(kExtWideThreads, 1) ext_wide_res_kernel(const ExtParams<T> P)
{
    using Rec = typename ChargeRec<T>::type;
    constexpr int MW = kExtWideThreads / 32;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(16) T slots[2][MW][8]; // each warp's sums, by row parity
    __shared__ double rslots[MW][4]; // each warp's re-evaluation sums
    __shared__ long long grp_next[MW];
    __shared__ unsigned long long grp_live[2][MW];
    __shared__ T grp_pos[MW][3]; // the first warp's vertex after the step
    __shared__ int grp_flag[MW];
    // FP32 steps run in every warp of a group (no second exchange); steps
    // with FP64 parts (mixed position, double-float, FP64) run on the
    // group's first warp only: repeated in every warp they queue on the
    // FP64 pipe (mixed 18.4 -> 25.8 ms, double-float 47 -> 95 ms)
    // (FP32, measured on the 4096-charge set with termination: every warp
    // combining and stepping 8.9 ms, the first warp alone publishing 9.15;
    // the four sums reduced together, 6 + 9 shuffles per warp and row
    // instead of 20 + 20: 9.5 ms before)
    constexpr bool kFp32 = MODE == EXT_FAST && sizeof(T) == 4;
    constexpr bool kAllStep = kFp32;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    Rec *tiles = reinterpret_cast<Rec *>(smem + 128);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int W = P.wide;
    if (!P.resident || nwarps > MW || W < 1 || nwarps % W != 0) {
        if (threadIdx.x == 0)
            atomicCAS(P.err, 0, EM_DEVERR_CONFIG);
        return;
    }
    const uint32_t full0 = smem_addr(bars);
    if (threadIdx.x == 0) {
        mbar_init(full0, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)P.p_pad * (uint32_t)sizeof(Rec);
        mbar_arrive_expect_tx(full0, bytes);
        const char *src = static_cast<const char *>(P.charges);
        const uint32_t dst = smem_addr(tiles);
        constexpr uint32_t CH = 32768;
        for (uint32_t off = 0; off < bytes; off += CH)
            bulk_g2s(dst + off, src + off, bytes - off < CH ? bytes - off : CH, full0);
    }
    // a wait that gave up anywhere stops the whole CTA before the groups part
    if (__syncthreads_or(!mbar_wait(full0, 0, P.err)))
        return;

    const int jneg_all = *P.meta;
    const long long count = (long long)*P.cont_in_count;
    const ExtCont<T> *cont = static_cast<const ExtCont<T> *>(P.cont_in);
    const int g = warp / W, wg = warp - g * W;
    const int t = wg * 32 + lane; // thread index within the group
    const int gthreads = 32 * W;
    auto gsync = [&]() {
        if (W == 1)
            __syncwarp();
        else
            group_barrier(1 + g, gthreads);
    };
    long long line = -1;
    int s = 1, lim = 0;
    bool live = false;
    ExtLane<T> st;
    T r0x = 0, r0y = 0, r0z = 0;
    auto take = [&]() {
        const long long k = grp_next[g];
        live = k < count;
        if (live) {
            const ExtCont<T> c = cont[k];
            line = c.line;
            s = c.s;
            lim = c.lim;
            st.px = c.px;
            st.py = c.py;
            st.pz = c.pz;
            st.dx = c.dx;
            st.dy = c.dy;
            st.dz = c.dz;
            r0x = ld_seed(P.x + line);
            r0y = ld_seed(P.y + line);
            r0z = ld_seed(P.z + line);
        }
    };
    if (t == 0)
        grp_next[g] = (long long)atomicAdd(P.cont_next, 1ull);
    gsync();
    take();

    // this warp's W-th of the resident records, fixed for the launch
    const int pb = (int)((long long)P.p_pad * wg / W);
    const int pe = (int)((long long)P.p_pad * (wg + 1) / W);
    const int jn = min(max(jneg_all - pb, 0), pe - pb);
    // mixed (paired layout, one block): the warp's W-th of the charge pairs
    const int rb = (int)((long long)(P.p_pad / 2) * wg / W);
    const int re = (int)((long long)(P.p_pad / 2) * (wg + 1) / W);
    const float4 *recs = reinterpret_cast<const float4 *>(tiles);

    unsigned long long evals = 0, refines = 0, live_seen = ~0ull;
    // the group's sums from the row's slots (lane w takes warp w's), in the
    // same order in every warp
    auto combine = [&](int par, T &ax, T &ay, T &az, T &dneg, float &dall, CF &hx, CF &hy,
                       CF &hz, double &Edx, double &Edy, double &Edz) {
        const bool mine = lane < W;
        const T *gs = slots[par][g * W + (mine ? lane : 0)];
        if constexpr (kFp32) {
            if (W == 16) {
                const float4 v =
                    *reinterpret_cast<const float4 *>(slots[par][g * W + (lane & 15)]);
                slots_reduce16(v, lane, ax, ay, az, dneg);
            } else {
                ax = group_sum<T, 32>(mine ? gs[0] : T(0));
                ay = group_sum<T, 32>(mine ? gs[1] : T(0));
                az = group_sum<T, 32>(mine ? gs[2] : T(0));
                dneg = group_min<T, 32>(mine ? gs[3] : T(3.0e38));
            }
            ext_field<T, MODE>(ax, ay, az, hx, hy, hz, Edx, Edy, Edz);
            return;
        } else if constexpr (MODE == EXT_MIXED || MODE == EXT_DF64) {
            hx.h = mine ? gs[0] : 0.0f;
            hx.l = mine ? gs[1] : 0.0f;
            hy.h = mine ? gs[2] : 0.0f;
            hy.l = mine ? gs[3] : 0.0f;
            hz.h = mine ? gs[4] : 0.0f;
            hz.l = mine ? gs[5] : 0.0f;
            group_two_sum<32>(hx);
            group_two_sum<32>(hy);
            group_two_sum<32>(hz);
            ax = (T)__fadd_rn(hx.h, hx.l);
            ay = (T)__fadd_rn(hy.h, hy.l);
            az = (T)__fadd_rn(hz.h, hz.l);
            if constexpr (MODE == EXT_MIXED)
                dall = group_sum<float, 32>(mine ? (float)gs[7] : 0.0f);
        } else {
            ax = group_sum<T, 32>(mine ? gs[0] : T(0));
            ay = group_sum<T, 32>(mine ? gs[1] : T(0));
            az = group_sum<T, 32>(mine ? gs[2] : T(0));
        }
        dneg = group_min<T, 32>(mine ? gs[6] : T(3.0e38));
        ext_field<T, MODE>(ax, ay, az, hx, hy, hz, Edx, Edy, Edz);
    };
    // a finished line (t == 0): its length and class, the next line's index
    auto finish = [&](int cls) {
        P.len[line] = s;
        P.cls[line] = cls;
        if (P.tail_lines > 0)
            live_count_drop(P.live_count);
        grp_next[g] = (long long)atomicAdd(P.cont_next, 1ull);
    };
    // a line handed on to a wider launch (t == 0); every input line was
    // taken at the start (a group each), so nothing is left behind
    auto save = [&]() {
        const unsigned long long k = atomicAdd(P.cont_count, 1ull);
        ExtCont<T> c;
        c.line = line;
        c.s = s;
        c.lim = lim;
        c.px = st.px;
        c.py = st.py;
        c.pz = st.pz;
        c.dx = st.dx;
        c.dy = st.dy;
        c.dz = st.dz;
        static_cast<ExtCont<T> *>(P.cont)[k] = c;
        live_count_drop(P.live_count);
    };
    // the first warp's vertex step: 1 the line goes on, 4 it ended and the
    // next line's index is out, 0 it was handed on
    auto step = [&](int par, bool use_row, T ax, T ay, T az, double Edx, double Edy,
                    double Edz, T dneg) -> int {
        const bool hand_off = use_row && grp_live[par][g] <= (unsigned long long)P.tail_lines;
        evals += (t == 0);
        const int cls = ext_vertex<T, MODE>(P, line, s, lim, st, t, ax, ay, az, Edx, Edy, Edz,
                                            dneg, r0x, r0y, r0z);
        if (cls >= 0) {
            if (t == 0)
                finish(cls);
            return 4;
        }
        if (hand_off) {
            if (t == 0)
                save();
            return 0;
        }
        return 1;
    };
    unsigned row_iter = 0;
    while (live) {
        const int par = row_iter & 1;
        // every 8th row: the live-line count, loaded a row before its use
        const bool load_row = P.tail_lines > 0 && (row_iter & 7) == 7;
        const bool use_row = P.tail_lines > 0 && (row_iter & 7) == 0 && row_iter > 0;
        ++row_iter;
        if (t == 0 && load_row)
            live_seen = *(volatile unsigned long long *)P.live_count;

        T ax = 0, ay = 0, az = 0, dneg = T(3.0e38);
        float dall = 0.0f; // mixed: sum of q^2/r^4 over the pairs
        CF hx, hy, hz;
        if constexpr (MODE == EXT_MIXED) {
            const ulonglong2 *A = reinterpret_cast<const ulonglong2 *>(tiles);
            mixed_pk<32>(A, A + P.p_pad / 2, jneg_all / 2, rb, re, lane, st.px, st.py, st.pz, hx,
                         hy, hz, dneg, dall);
        } else {
            tile_pairs<T, MODE>(32, tiles + pb, jn, pe - pb, lane, st, ax, ay, az, dneg, dall,
                                hx, hy, hz);
        }
        if constexpr (!kFp32 && MODE != EXT_MIXED && MODE != EXT_DF64) {
            ax = group_sum<T, 32>(ax);
            ay = group_sum<T, 32>(ay);
            az = group_sum<T, 32>(az);
        }
        if constexpr (kFp32) {
            // FP32: the four sums at once; slot words 0..3 = x, y, z, dneg
            const float k = warp_reduce4(ax, ay, az, dneg, lane);
            if ((lane & 7) == 0)
                slots[par][warp][lane >> 3] = k;
        } else if constexpr (MODE == EXT_MIXED || MODE == EXT_DF64) {
            // the compensated sums, dneg and l2 at once; slot words
            // 2i, 2i + 1 = item i (hx, hy, hz, then dneg and l2)
            float f, g2;
            warp_reduce_cf(hx, hy, hz, dneg, dall, lane, f, g2);
            if ((lane & 7) == 0) {
                slots[par][warp][2 * (lane >> 3)] = f;
                slots[par][warp][2 * (lane >> 3) + 1] = g2;
            }
        } else {
            dneg = group_min<T, 32>(dneg);
            if (lane == 0) {
                T *o = slots[par][warp];
                if constexpr (MODE == EXT_MIXED || MODE == EXT_DF64) {
                    o[0] = hx.h;
                    o[1] = hx.l;
                    o[2] = hy.h;
                    o[3] = hy.l;
                    o[4] = hz.h;
                    o[5] = hz.l;
                } else {
                    o[0] = ax;
                    o[1] = ay;
                    o[2] = az;
                }
                o[6] = dneg;
                o[7] = (T)dall;
            }
        }
        if (t == 0 && use_row)
            grp_live[par][g] = live_seen;
        gsync();

        if constexpr (kAllStep) {
            // ---- every warp combines the group's sums and steps ------------
            double Edx = 0, Edy = 0, Edz = 0;
            combine(par, ax, ay, az, dneg, dall, hx, hy, hz, Edx, Edy, Edz);
            const bool hand_off = use_row && grp_live[par][g] <= (unsigned long long)P.tail_lines;
            evals += (t == 0);
            const int cls = ext_vertex<T, MODE>(P, line, s, lim, st, t, ax, ay, az, Edx, Edy,
                                                Edz, dneg, r0x, r0y, r0z);
            if (cls >= 0) {
                if (t == 0)
                    finish(cls);
                gsync();
                take();
            } else if (hand_off) {
                if (t == 0)
                    save();
                live = false;
            }
        } else {
            // ---- the group's first warp combines and steps, then publishes
            int flag = 0; // 1: the line goes on, 2: re-evaluate, 4: next line taken
            double Edx = 0, Edy = 0, Edz = 0;
            if (wg == 0) {
                combine(par, ax, ay, az, dneg, dall, hx, hy, hz, Edx, Edy, Edz);
                bool redo = false;
                if constexpr (MODE == EXT_MIXED)
                    redo = ext_ill_conditioned(P, dall, ax, ay, az);
                flag = redo ? 2 : step(par, use_row, ax, ay, az, Edx, Edy, Edz, dneg);
                if (lane == 0) {
                    grp_flag[g] = flag;
                    grp_pos[g][0] = st.px;
                    grp_pos[g][1] = st.py;
                    grp_pos[g][2] = st.pz;
                }
            }
            gsync();
            flag = grp_flag[g];
            if constexpr (MODE == EXT_MIXED) {
                if (flag == 2) {
                    // an ill-conditioned sum: the group re-evaluates the field
                    // in double-float (or FP64), each warp its W-th of the
                    // resident records
                    double fx = 0, fy = 0, fz = 0;
                    if (!P.refine_fp64)
                        field_pk<32, false>(recs, P.p_pad, rb, re, lane, (float)st.px,
                                            (float)st.py, (float)st.pz, fx, fy, fz);
                    else
                        field_pk<32, true>(recs, P.p_pad, rb, re, lane, (float)st.px,
                                           (float)st.py, (float)st.pz, fx, fy, fz);
                    fx = group_sum<double, 32>(fx);
                    fy = group_sum<double, 32>(fy);
                    fz = group_sum<double, 32>(fz);
                    if (lane == 0) {
                        rslots[warp][0] = fx;
                        rslots[warp][1] = fy;
                        rslots[warp][2] = fz;
                    }
                    gsync();
                    if (wg == 0) {
                        const bool mine = lane < W;
                        const double *rs = rslots[g * W + (mine ? lane : 0)];
                        fx = group_sum<double, 32>(mine ? rs[0] : 0.0);
                        fy = group_sum<double, 32>(mine ? rs[1] : 0.0);
                        fz = group_sum<double, 32>(mine ? rs[2] : 0.0);
                        ax = (T)(fx * kElectroK);
                        ay = (T)(fy * kElectroK);
                        az = (T)(fz * kElectroK);
                        refines += (t == 0);
                        flag = step(par, use_row, ax, ay, az, Edx, Edy, Edz, dneg);
                        if (lane == 0) {
                            grp_flag[g] = flag;
                            grp_pos[g][0] = st.px;
                            grp_pos[g][1] = st.py;
                            grp_pos[g][2] = st.pz;
                        }
                    }
                    gsync();
                    flag = grp_flag[g];
                }
            }
            if (flag & 4) {
                take();
            } else if (flag & 1) {
                if (wg != 0) {
                    st.px = grp_pos[g][0];
                    st.py = grp_pos[g][1];
                    st.pz = grp_pos[g][2];
                }
            } else {
                live = false;
            }
        }
    }
    // counters: one atomic per warp
    for (int o = 16; o; o >>= 1) {
        evals += __shfl_xor_sync(0xffffffffu, evals, o);
        refines += __shfl_xor_sync(0xffffffffu, refines, o);
    }
    if (lane == 0) {
        if (evals)
            atomicAdd(P.evals, evals);
        if (refines)
            atomicAdd(P.refines, refines);
    }
}

template <class T, int MODE>
cudaError_t launch_ext_wide_mode(const ExtParams<T> &p, const LaunchCfg &cfg,
                                 cudaStream_t stream)
{
    auto kern = cfg.resident ? ext_wide_res_kernel<T, MODE> : ext_wide_kernel<T, MODE>;
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess)
        return e;
    const int threads = 32 * (cfg.warps + (cfg.resident ? 0 : 1));
    kern<<<cfg.grid, threads, cfg.smem, stream>>>(p);
    count_launch(1);
    return cudaGetLastError();
}

template <class T, int TPL, int MODE>
cudaError_t launch_ext_one(const ExtParams<T> &p, const LaunchCfg &cfg, cudaStream_t stream)
{
    auto kern = ext_trace_kernel<T, TPL, MODE>;
    cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg.smem);
    if (e != cudaSuccess)
        return e;
    const int threads = 32 * (cfg.warps + (cfg.resident ? 0 : 1));
    kern<<<cfg.grid, threads, cfg.smem, stream>>>(p);
    count_launch(1);
    return cudaGetLastError();
}

template <class T, int MODE>
cudaError_t launch_ext_mode(const ExtParams<T> &p, const LaunchCfg &cfg, cudaStream_t stream)
{
    switch (cfg.tpl) {
    case 4: return launch_ext_one<T, 4, MODE>(p, cfg, stream);
    case 8: return launch_ext_one<T, 8, MODE>(p, cfg, stream);
    case 16: return launch_ext_one<T, 16, MODE>(p, cfg, stream);
    case 32: return launch_ext_one<T, 32, MODE>(p, cfg, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace

template <class T>
cudaError_t launch_ext_stage(const void *raw, int p, void *staged, int p_pad, int gran,
                             int block, int *meta, float *qabs, cudaStream_t stream)
{
    if (block < 0 || (block && (block & 1 || p_pad % block)))
        return cudaErrorInvalidValue;
    ext_stage_kernel<T><<<1, 1024, 0, stream>>>(static_cast<const T *>(raw), p,
                                                static_cast<T *>(staged), p_pad, gran, block,
                                                meta, qabs);
    count_launch(1);
    return cudaGetLastError();
}

template <>
cudaError_t launch_ext_trace<float>(const ExtParams<float> &p, const LaunchCfg &cfg, int mode,
                                    cudaStream_t stream)
{
    if (mode == EXT_DF64)
        return launch_ext_mode<float, EXT_DF64>(p, cfg, stream);
    return mode == EXT_MIXED ? launch_ext_mode<float, EXT_MIXED>(p, cfg, stream)
                             : launch_ext_mode<float, EXT_FAST>(p, cfg, stream);
}

template <>
cudaError_t launch_ext_trace<double>(const ExtParams<double> &p, const LaunchCfg &cfg, int mode,
                                     cudaStream_t stream)
{
    if (mode != EXT_FAST)
        return cudaErrorInvalidValue;
    return launch_ext_mode<double, EXT_FAST>(p, cfg, stream);
}

template <>
cudaError_t launch_ext_wide<float>(const ExtParams<float> &p, const LaunchCfg &cfg, int mode,
                                   cudaStream_t stream)
{
    if (mode == EXT_DF64)
        return launch_ext_wide_mode<float, EXT_DF64>(p, cfg, stream);
    return mode == EXT_MIXED ? launch_ext_wide_mode<float, EXT_MIXED>(p, cfg, stream)
                             : launch_ext_wide_mode<float, EXT_FAST>(p, cfg, stream);
}

template <>
cudaError_t launch_ext_wide<double>(const ExtParams<double> &p, const LaunchCfg &cfg, int mode,
                                    cudaStream_t stream)
{
    if (mode != EXT_FAST)
        return cudaErrorInvalidValue;
    return launch_ext_wide_mode<double, EXT_FAST>(p, cfg, stream);
}

template cudaError_t launch_ext_stage<float>(const void *, int, void *, int, int, int, int *,
                                             float *, cudaStream_t);
template cudaError_t launch_ext_stage<double>(const void *, int, void *, int, int, int, int *,
                                              float *, cudaStream_t);

} // namespace em
