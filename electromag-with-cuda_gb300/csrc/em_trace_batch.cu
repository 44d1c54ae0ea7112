// Batched tracing of many independent charge sets (the extended method:
// seeded lines, termination at negative charges, per-line step limits) in
// persistent launches fed by a device work queue.
//
// Work items are (set, chunk of lines).  A persistent CTA takes an item from
// the queue, stages that set's charges in shared memory (one bulk copy when
// they fit, otherwise a producer warp streams tiles through a ring while the
// CTA steps in lockstep), and its warps trace the chunk's lines with the
// single-set kernel's machinery: lane groups, warp-ballot refill from a
// CTA-local line counter, and wider groups for the last lines.
//
// A phase bounds the field evaluations a line may take (its budget); lines
// still running then save their state and join a continuation list.  A
// one-CTA kernel sorts that list by set and builds the next phase's items,
// whose budget is four times larger, the last unlimited.  No CTA is held
// for thousands of steps by a single line while items wait, and every
// launch reads its item count from device memory, so the whole sequence is
// graph-capturable.
#include "em_device.cuh"
#include "em_ext.cuh"
#include "em_internal.h"
#include "em_math.cuh"

namespace em {
namespace {

// ---- staging: one CTA per set, negatives first (as ext_stage_kernel) ------
__global__ void __launch_bounds__(256) batch_stage_kernel(const float *raw,
                                                          const long long *coff,
                                                          const long long *soff, const int *spad,
                                                          int gran, float *staged, int *snneg,
                                                          float *sqabs)
{
    const int set = blockIdx.x;
    const long long c0 = coff[set];
    const int p = (int)(coff[set + 1] - c0);
    const int pp = spad[set];
    float *dst = staged + 4 * soff[set];
    const float *src = raw + 4 * c0;
    __shared__ int scan[256];
    __shared__ float qm[8];
    const int tid = threadIdx.x;
    const int per = (p + 255) / 256;
    const int b = tid * per, e = min(p, b + per);
    int neg = 0;
    float qmax = 0;
    for (int i = b; i < e; ++i) {
        const float q = src[4 * (size_t)i + 3];
        neg += q < 0.f;
        qmax = fmaxf(qmax, fabsf(q));
    }
    scan[tid] = neg;
    __syncthreads();
    for (int off = 1; off < 256; off <<= 1) {
        const int v = tid >= off ? scan[tid - off] : 0;
        __syncthreads();
        scan[tid] += v;
        __syncthreads();
    }
    const int total_neg = scan[255];
    const int neg_pad = (total_neg + gran - 1) / gran * gran;
    int wn = scan[tid] - neg;
    int wp = neg_pad + (b - wn);
    for (int i = b; i < e; ++i) {
        const float *r = src + 4 * (size_t)i;
        float *d = dst + 4 * (size_t)(r[3] < 0.f ? wn++ : wp++);
        d[0] = r[0];
        d[1] = r[1];
        d[2] = r[2];
        d[3] = r[3];
    }
    const int pos_end = neg_pad + (p - total_neg);
    for (int i = tid; i < pp; i += 256) {
        if ((i >= total_neg && i < neg_pad) || i >= pos_end) {
            float *d = dst + 4 * (size_t)i;
            d[0] = d[1] = d[2] = 1e15f;
            d[3] = 0.f;
        }
    }
    for (int o = 16; o; o >>= 1)
        qmax = fmaxf(qmax, __shfl_xor_sync(0xffffffffu, qmax, o));
    if ((tid & 31) == 0)
        qm[tid >> 5] = qmax;
    __syncthreads();
    if (tid == 0) {
        float m = 0;
        for (int w = 0; w < 8; ++w)
            m = fmaxf(m, qm[w]);
        snneg[set] = neg_pad;
        sqabs[set] = m;
    }
}

// ---- continuation list -> next phase's items (one CTA) ---------------------
// counts per set, scan (largest set first), scatter of line ids by set, then
// items of at most item_lines lines per set.
__device__ __forceinline__ int set_of(const long long *line_off, int nsets, long long id)
{
    int lo = 0, hi = nsets; // line_off[lo] <= id < line_off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (line_off[mid] <= id)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(1024) batch_sort_kernel(BatchQueues Q, const long long *line_off,
                                                          int nsets, int item_lines)
{
    const int tid = threadIdx.x;
    const long long c = (long long)*Q.cont_count;
    for (int s = tid; s < nsets; s += 1024)
        Q.set_count[s] = 0;
    __syncthreads();
    for (long long i = tid; i < c; i += 1024)
        atomicAdd(&Q.set_count[set_of(line_off, nsets, Q.cont[i])], 1);
    __syncthreads();
    if (tid == 0) {
        // sequential scan over sets (few thousand at most), largest set
        // first: line offsets and item offsets, so the next phase deals the
        // longest items first
        long long lo = 0;
        int it = 0;
        for (int o = 0; o < nsets; ++o) {
            const int s = Q.set_order[o];
            const int k = Q.set_count[s];
            Q.set_line_off[s] = lo;
            Q.set_item_off[s] = it;
            lo += k;
            it += (k + item_lines - 1) / item_lines;
        }
        *Q.next_nitems = it;
    }
    __syncthreads();
    for (int s = tid; s < nsets; s += 1024)
        Q.set_fill[s] = 0;
    __syncthreads();
    for (long long i = tid; i < c; i += 1024) {
        const long long id = Q.cont[i];
        const int s = set_of(line_off, nsets, id);
        const int slot = atomicAdd(&Q.set_fill[s], 1);
        Q.cont_sorted[Q.set_line_off[s] + slot] = id;
    }
    __syncthreads();
    for (int s = tid; s < nsets; s += 1024) {
        const int k = Q.set_count[s];
        const long long lo = Q.set_line_off[s];
        int w = Q.set_item_off[s];
        for (int b = 0; b < k; b += item_lines, ++w)
            Q.next_items[w] = make_int4(s, (int)(lo + b), (int)(lo + min(k, b + item_lines)), 0);
    }
    __syncthreads();
    if (tid == 0) {
        *Q.cont_count = 0;   // the next phase appends from zero
        *Q.next_item_ctr = 0;
    }
}

// ---- the persistent tracing kernel ----------------------------------------
template <int TPL>
__global__ void __launch_bounds__(1024, 1) batch_trace_kernel(const BatchParams P)
{
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    float4 *tiles = reinterpret_cast<float4 *>(smem + 256);
    int *s_ctl = reinterpret_cast<int *>(smem + 160); // [0] item, [1] next line

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int ncw = nwarps - 1;               // last warp: copies
    const int NST = P.stages;
    if (NST > 8 || NST < 1 || ncw < 1) {
        if (threadIdx.x == 0)
            atomicCAS(P.err, 0, EM_DEVERR_CONFIG);
        return;
    }
    // bars: [0] resident load, [1..8] ring full, [9..16] ring empty
    const uint32_t res0 = smem_addr(bars), full0 = smem_addr(bars + 1),
                   empty0 = smem_addr(bars + 9);
    if (threadIdx.x == 0) {
        mbar_init(res0, 1);
        for (int s = 0; s < NST; ++s) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, ncw);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const size_t nl = (size_t)P.nlines;
    const float term_r2 = (float)P.term_r2;
    const float res = (float)P.res;
    const int nitems = *P.nitems;
    uint32_t res_loads = 0, it = 0;
    unsigned long long evals = 0;
    bool failed = false;

    for (;;) {
        if (threadIdx.x == 0)
            s_ctl[0] = (int)atomicAdd(P.item_ctr, 1u);
        __syncthreads();
        const int item = s_ctl[0];
        if (item >= nitems)
            break;
        const int4 I = P.items[item];
        const int set = I.x, ibeg = I.y, iend = I.z;
        const int pp = P.spad[set];
        const int jneg = P.snneg[set];
        const unsigned long long pset = (unsigned long long)(P.coff[set + 1] - P.coff[set]);
        const float4 *src = P.staged + P.soff[set];
        const bool resident = pp <= P.resident_cap;
        const int ntiles = resident ? 1 : (pp + P.tile_recs - 1) / P.tile_recs;
        if (threadIdx.x == 0)
            s_ctl[1] = ibeg;
        if (resident && threadIdx.x == 0) {
            const uint32_t bytes = (uint32_t)pp * 16u;
            mbar_arrive_expect_tx(res0, bytes);
            constexpr uint32_t CH = 32768;
            for (uint32_t off = 0; off < bytes; off += CH)
                bulk_g2s(smem_addr(tiles) + off, reinterpret_cast<const char *>(src) + off,
                         bytes - off < CH ? bytes - off : CH, res0);
        }
        __syncthreads();

        if (warp == ncw) {
            // ---- copy warp ---------------------------------------------------
            if (resident) {
                if (lane == 0 && !mbar_wait(res0, res_loads & 1, P.err))
                    failed = true;
            } else {
                const uint32_t tb = (uint32_t)P.tile_recs * 16u;
                while (__syncthreads_or(0)) {
                    if (lane == 0 && !failed && *(volatile int *)P.err == 0) {
                        for (int tile = 0; tile < ntiles; ++tile, ++it) {
                            const uint32_t s = it % NST, ph = (it / NST) & 1;
                            if (it >= (uint32_t)NST &&
                                !mbar_wait(empty0 + 8 * s, ph ^ 1, P.err)) {
                                failed = true;
                                break;
                            }
                            const int base = tile * P.tile_recs;
                            const int cnt = min(P.tile_recs, pp - base);
                            mbar_arrive_expect_tx(full0 + 8 * s, (uint32_t)cnt * 16u);
                            bulk_g2s(smem_addr(tiles) + s * tb,
                                     reinterpret_cast<const char *>(src + base),
                                     (uint32_t)cnt * 16u, full0 + 8 * s);
                        }
                    }
                    __syncwarp();
                }
            }
        } else {
            // ---- compute warps -------------------------------------------------
            if (resident && !mbar_wait(res0, res_loads & 1, P.err))
                failed = true;
            int tg = TPL, t = lane & (TPL - 1);
            long long line = -1;
            int s = 1, lim = 0, used = 0;
            float px = 0, py = 0, pz = 0;
            bool live = false, need = !failed, dry = false;

            auto start_line = [&](long long id) -> bool {
                line = id;
                if (P.phase == 0) {
                    px = P.sx[id];
                    py = P.sy[id];
                    pz = P.sz[id];
                    s = 1;
                    if (t == 0 && P.store_rows > 0) {
                        P.vx[id] = px;
                        P.vy[id] = py;
                        P.vz[id] = pz;
                    }
                } else {
                    px = P.st_x[id];
                    py = P.st_y[id];
                    pz = P.st_z[id];
                    s = P.st_s[id];
                }
                used = 0;
                lim = P.max_steps;
                if (P.steps_per_line)
                    lim = max(1, min(P.steps_per_line[id], P.max_steps));
                if (s >= lim) {
                    if (t == 0) {
                        P.len[id] = s;
                        P.cls[id] = EM_TERM_STEPS_DEV;
                        P.lx[id] = px;
                        P.ly[id] = py;
                        P.lz[id] = pz;
                    }
                    return false;
                }
                return true;
            };
            auto refill = [&]() {
                for (int guard = 0; guard < 1 << 20; ++guard) {
                    const unsigned m = __ballot_sync(0xffffffffu, t == 0 && need);
                    if (!m)
                        break;
                    const int first = __ffs(m) - 1;
                    int base = 0;
                    if (lane == first)
                        base = atomicAdd(&s_ctl[1], __popc(m));
                    base = __shfl_sync(0xffffffffu, base, first);
                    if (base + __popc(m) >= iend)
                        dry = true;
                    const int mine = base + __popc(m & ((1u << lane) - 1u));
                    const int k = __shfl_sync(0xffffffffu, mine, lane - t);
                    if (need) {
                        if (k < iend) {
                            const long long id = P.phase == 0 ? (long long)k : P.cont_in[k];
                            live = start_line(id);
                            need = !live;
                        } else {
                            line = -1;
                            live = false;
                            need = false;
                        }
                    }
                }
            };
            auto regroup = [&]() {
                if (!P.regroup || !dry || tg >= 32)
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
                const int src_lane = has ? (int)__fns(lead, 0, k + 1) : 0;
                line = __shfl_sync(0xffffffffu, line, src_lane);
                s = __shfl_sync(0xffffffffu, s, src_lane);
                lim = __shfl_sync(0xffffffffu, lim, src_lane);
                used = __shfl_sync(0xffffffffu, used, src_lane);
                px = __shfl_sync(0xffffffffu, px, src_lane);
                py = __shfl_sync(0xffffffffu, py, src_lane);
                pz = __shfl_sync(0xffffffffu, pz, src_lane);
                live = has;
                need = false;
                if (!has)
                    line = -1;
                tg = ng;
                t = lane & (tg - 1);
            };
            refill();
            regroup();
            ExtLane<float> st;
            for (;;) {
                const bool any = resident ? __any_sync(0xffffffffu, live)
                                          : __syncthreads_or(live) != 0;
                if (!any)
                    break;
                const bool wlive = __any_sync(0xffffffffu, live);
                float ax = 0, ay = 0, az = 0, dneg = 3.0e38f, dall = 3.0e38f;
                CF hx, hy, hz;
                st.px = px;
                st.py = py;
                st.pz = pz;
                if (resident) {
                    tile_pairs<float, EXT_FAST>(tg, tiles, jneg, pp, t, st, ax, ay, az, dneg,
                                                dall, hx, hy, hz);
                } else {
                    for (int tile = 0; tile < ntiles; ++tile, ++it) {
                        const uint32_t sg = it % NST, ph = (it / NST) & 1;
                        if (!failed && !mbar_wait(full0 + 8 * sg, ph, P.err))
                            failed = true;
                        if (!failed) {
                            const int base = tile * P.tile_recs;
                            const int cnt = min(P.tile_recs, pp - base);
                            const int jn = min(max(jneg - base, 0), cnt);
                            // a warp with no live line only keeps the ring
                            // turning
                            if (wlive)
                                tile_pairs<float, EXT_FAST>(tg, tiles + sg * P.tile_recs, jn, cnt,
                                                            t, st, ax, ay, az, dneg, dall, hx, hy,
                                                            hz);
                            __syncwarp();
                            if (lane == 0)
                                mbar_arrive(empty0 + 8 * sg);
                        }
                    }
                    if (failed) {
                        live = need = false;
                        line = -1;
                        continue;
                    }
                }
                combine_group<float, EXT_FAST>(tg, ax, ay, az, dneg, dall, hx, hy, hz);
                const float K = (float)kElectroK;
                ax = mul_rn(ax, K);
                ay = mul_rn(ay, K);
                az = mul_rn(az, K);
                if (live) {
                    evals += (t == 0) ? pset : 0ull;
                    ++used;
                    int cls = -1;
                    if (dneg < term_r2) {
                        cls = EM_TERM_CHARGE_DEV;
                    } else {
                        const float r0x = ld_seed(P.sx + line), r0y = ld_seed(P.sy + line),
                                    r0z = ld_seed(P.sz + line);
                        float sx, sy, sz, k2;
                        step_vector<float>(ax, ay, az, r0x, r0y, r0z, res, sx, sy, sz, k2);
                        const float nx = add_rn(px, sx), ny = add_rn(py, sy), nz = add_rn(pz, sz);
                        if (!(k2 > 0.f) || !isfinite(nx) || !isfinite(ny) || !isfinite(nz)) {
                            cls = EM_TERM_NULL_DEV;
                        } else {
                            px = nx;
                            py = ny;
                            pz = nz;
                            if (t == 0 && s < P.store_rows) {
                                const size_t w = (size_t)s * nl + (size_t)line;
                                store_stream(P.vx + w, nx);
                                store_stream(P.vy + w, ny);
                                store_stream(P.vz + w, nz);
                            }
                            ++s;
                            if (s >= lim)
                                cls = EM_TERM_STEPS_DEV;
                        }
                    }
                    if (cls >= 0) {
                        if (t == 0) {
                            P.len[line] = s;
                            P.cls[line] = cls;
                            P.lx[line] = px;
                            P.ly[line] = py;
                            P.lz[line] = pz;
                        }
                        live = false;
                        need = true;
                    } else if (P.budget > 0 && used >= P.budget) {
                        // out of this phase's budget: save the state, continue
                        // in the next phase
                        if (t == 0) {
                            P.st_x[line] = px;
                            P.st_y[line] = py;
                            P.st_z[line] = pz;
                            P.st_s[line] = s;
                            const unsigned long long slot = atomicAdd(P.cont_count, 1ull);
                            P.cont_out[slot] = line;
                        }
                        live = false;
                        need = true;
                    }
                }
                refill();
                regroup();
            }
        }
        __syncthreads();
        if (resident)
            ++res_loads;
    }
    for (int o = 16; o; o >>= 1)
        evals += __shfl_xor_sync(0xffffffffu, evals, o);
    if (lane == 0 && evals)
        atomicAdd(P.evals, evals);
}

template <int TPL>
cudaError_t launch_batch_one(const BatchParams &p, int grid, int threads, size_t smem,
                             cudaStream_t stream)
{
    batch_trace_kernel<TPL><<<grid, threads, smem, stream>>>(p);
    count_launch(1);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_batch_stage(const float *raw, const long long *coff, const long long *soff,
                               const int *spad, int gran, int nsets, float *staged, int *snneg,
                               float *sqabs, cudaStream_t stream)
{
    batch_stage_kernel<<<nsets, 256, 0, stream>>>(raw, coff, soff, spad, gran, staged, snneg,
                                                  sqabs);
    count_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_batch_sort(const BatchQueues &q, const long long *line_off, int nsets,
                              int item_lines, cudaStream_t stream)
{
    batch_sort_kernel<<<1, 1024, 0, stream>>>(q, line_off, nsets, item_lines);
    count_launch(1);
    return cudaGetLastError();
}

cudaError_t prepare_batch_trace(size_t smem)
{
    cudaError_t e = cudaFuncSetAttribute(batch_trace_kernel<4>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_trace_kernel<8>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(batch_trace_kernel<16>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return e;
}

cudaError_t launch_batch_trace(const BatchParams &p, int tpl, int grid, int threads, size_t smem,
                               cudaStream_t stream)
{
    switch (tpl) {
    case 4: return launch_batch_one<4>(p, grid, threads, smem, stream);
    case 8: return launch_batch_one<8>(p, grid, threads, smem, stream);
    case 16: return launch_batch_one<16>(p, grid, threads, smem, stream);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace em
