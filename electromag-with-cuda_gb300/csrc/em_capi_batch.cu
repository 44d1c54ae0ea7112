// C ABI of the batched tracer (em_trace_batch_f32): planning of the work
// items, buffers, and the launch sequence (optionally a CUDA graph).
#include <algorithm>
#include <chrono>
#include <climits>
#include <mutex>
#include <numeric>
#include <vector>

#include "em_internal.h"
#include "em_plan.h"
#include "emgb300.h"

namespace em {
namespace {

struct Buf {
    size_t off = 0;
    size_t add(size_t bytes)
    {
        const size_t o = off;
        off += (bytes + 255) / 256 * 256;
        return o;
    }
};

int trace_batch(size_t nsets, const float *charges, const int64_t *charge_off, const float *sx,
                const float *sy, const float *sz, const int64_t *line_off,
                const int32_t *steps_per_line, int max_steps, float resolution,
                float term_radius, int store_rows, float *vx, float *vy, float *vz, float *lx,
                float *ly, float *lz, int32_t *len, int32_t *cls, const em_batch_options *opt,
                em_perf *perf)
{
    using clock = std::chrono::steady_clock;
    const auto t_start = clock::now();
    if (!nsets || !charge_off || !line_off)
        return EM_ERR_ARG;
    if (resolution == 0)
        return EM_ERR_RESOLUTION;
    if (max_steps < 1)
        return EM_ERR_STEPS;
    if (nsets > (size_t)INT_MAX / 4 || store_rows < 0)
        return EM_ERR_TOO_LARGE;
    const long long N = line_off[nsets], Pt = charge_off[nsets];
    if (N <= 0 || Pt <= 0 || line_off[0] != 0 || charge_off[0] != 0)
        return EM_ERR_ARG;
    if (!charges || !sx || !sy || !sz || !lx || !ly || !lz || !len || !cls)
        return EM_ERR_ARG;
    if (store_rows > 0 && (!vx || !vy || !vz))
        return EM_ERR_ARG;
    if (store_rows > max_steps)
        store_rows = max_steps;
    if (N > (long long)INT_MAX || (long long)store_rows * N > (LLONG_MAX / 16))
        return EM_ERR_TOO_LARGE;
    em_batch_options o{};
    if (opt)
        o = *opt;
    const int tpl = o.threads_per_line ? o.threads_per_line : 16;
    if (tpl != 4 && tpl != 8 && tpl != 16)
        return EM_ERR_ARG;
    // a tile beyond 65 536 records could never fit shared memory
    if (o.tile_charges < 0 || o.tile_charges > 65536)
        return EM_ERR_ARG;
    const int item_lines = o.lines_per_item > 0 ? o.lines_per_item : 512;
    // most lines of a set end within a few dozen steps while the few that
    // run to their limit carry most of the pairs: a short first phase hands
    // those on, grouped by set, before they can hold a CTA alone
    const int first_budget = o.first_budget > 0 ? o.first_budget : 64;
    const int phases = o.phases > 0 ? std::min(o.phases, 8) : 4;
    const int stages = o.stages > 0 ? std::min(o.stages, 8) : 4;
    if (o.device_ptrs && ((uintptr_t)charges & 15))
        return EM_ERR_ARG;
    for (size_t s = 0; s < nsets; ++s)
        if (charge_off[s + 1] <= charge_off[s] || line_off[s + 1] < line_off[s] ||
            charge_off[s + 1] - charge_off[s] > (int64_t)(INT_MAX / 64))
            return EM_ERR_ARG;
    if (perf)
        perf->progress = 0;

    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);

    // ---- plan ---------------------------------------------------------------
    const int gran = tpl;
    const size_t smem_cap = std::min<size_t>(c.smem_optin, 227 * 1024);
    const int resident_cap = (int)((smem_cap - 256) / 16);
    int tile = o.tile_charges > 0 ? o.tile_charges : 1024;
    tile = (tile + gran - 1) / gran * gran;
    if (256 + (size_t)stages * tile * 16 > smem_cap)
        return EM_ERR_ARG;
    std::vector<long long> soff(nsets), coff(nsets + 1), loff(nsets + 1);
    std::vector<int> spad(nsets);
    long long staged = 0;
    for (size_t s = 0; s < nsets; ++s) {
        const long long p = charge_off[s + 1] - charge_off[s];
        spad[s] = (int)(ceil_div(p, gran) * gran + gran);
        soff[s] = staged;
        staged += spad[s];
        coff[s] = charge_off[s];
        loff[s] = line_off[s];
    }
    coff[nsets] = charge_off[nsets];
    loff[nsets] = line_off[nsets];
    int max_pad = *std::max_element(spad.begin(), spad.end());
    const size_t smem = 256 + (size_t)std::max(std::min(max_pad, resident_cap), stages * tile) * 16;
    // phase-0 items: chunks of item_lines lines, largest work first
    std::vector<int4> items0;
    std::vector<double> work;
    for (size_t s = 0; s < nsets; ++s) {
        const long long a = line_off[s], b = line_off[s + 1];
        for (long long k = a; k < b; k += item_lines) {
            items0.push_back(make_int4((int)s, (int)k, (int)std::min(b, k + item_lines), 0));
            work.push_back((double)(charge_off[s + 1] - charge_off[s]) *
                           (double)(std::min(b, k + item_lines) - k));
        }
    }
    std::vector<size_t> order(items0.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t i, size_t j) { return work[i] > work[j]; });
    std::vector<int4> sorted_items(items0.size());
    for (size_t i = 0; i < order.size(); ++i)
        sorted_items[i] = items0[order[i]];
    const int nitems0 = (int)sorted_items.size();
    // continuation items: the lines one CTA holds at once (31 compute warps,
    // 32/tpl lines each); the lines still running after a phase are the long
    // ones, of near-equal length within a set, so such an item keeps every
    // warp busy to its end, and small items balance the CTAs
    const int cont_lines = 31 * (32 / tpl);
    const long long max_next_items = (long long)nsets + N / cont_lines + 1;
    std::vector<int> set_order(nsets);
    std::iota(set_order.begin(), set_order.end(), 0);
    std::stable_sort(set_order.begin(), set_order.end(), [&](int a, int b) {
        return charge_off[a + 1] - charge_off[a] > charge_off[b + 1] - charge_off[b];
    });

    // ---- device workspace ------------------------------------------------------
    Buf B;
    const size_t o_staged = B.add((size_t)staged * 16);
    const size_t o_soff = B.add(nsets * 8), o_spad = B.add(nsets * 4), o_snneg = B.add(nsets * 4),
                 o_sqabs = B.add(nsets * 4), o_coff = B.add((nsets + 1) * 8),
                 o_loff = B.add((nsets + 1) * 8);
    const size_t o_items0 = B.add((size_t)std::max(nitems0, 1) * 16);
    const size_t o_itemsn = B.add((size_t)max_next_items * 16);
    const size_t o_ctl = B.add(256); // counters
    const size_t o_st = B.add((size_t)N * 16);
    const size_t o_cont = B.add((size_t)N * 8), o_conts = B.add((size_t)N * 8);
    const size_t o_setq = B.add(nsets * 4 * 3 + nsets * 8 + 64);
    const size_t o_order = B.add(nsets * 4);
    size_t o_raw = 0, o_lines = 0, o_spl = 0, o_out = 0, o_rows = 0;
    const bool host = !o.device_ptrs;
    if (host) {
        o_raw = B.add((size_t)Pt * 16);
        o_lines = B.add((size_t)N * 12);
        if (steps_per_line)
            o_spl = B.add((size_t)N * 4);
        o_out = B.add((size_t)N * 20);
        if (store_rows > 0)
            o_rows = B.add((size_t)store_rows * N * 12);
    }
    if ((code = grow(&c.batch, &c.batch_cap, B.off)))
        return code;
    if ((code = grow(&c.errbuf, &c.errbuf_cap, 256)))
        return code;
    c.err = static_cast<int *>(c.errbuf);
    unsigned char *w = static_cast<unsigned char *>(c.batch);
    cudaStream_t st = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;

    const float *d_charges = charges, *d_sx = sx, *d_sy = sy, *d_sz = sz;
    const int32_t *d_spl = steps_per_line;
    float *d_vx = vx, *d_vy = vy, *d_vz = vz, *d_lx = lx, *d_ly = ly, *d_lz = lz;
    int32_t *d_len = len, *d_cls = cls;
    if (host) {
        d_charges = reinterpret_cast<float *>(w + o_raw);
        float *L = reinterpret_cast<float *>(w + o_lines);
        d_sx = L;
        d_sy = L + N;
        d_sz = L + 2 * N;
        if (steps_per_line)
            d_spl = reinterpret_cast<int32_t *>(w + o_spl);
        float *O = reinterpret_cast<float *>(w + o_out);
        d_lx = O;
        d_ly = O + N;
        d_lz = O + 2 * N;
        d_len = reinterpret_cast<int32_t *>(O + 3 * N);
        d_cls = d_len + N;
        if (store_rows > 0) {
            float *R = reinterpret_cast<float *>(w + o_rows);
            d_vx = R;
            d_vy = R + (size_t)store_rows * N;
            d_vz = R + 2 * (size_t)store_rows * N;
        }
    }
    // inputs (outside any graph: the graph replays only device work)
    cudaError_t e = cudaSuccess;
    auto H2D = [&](void *d, const void *h, size_t bytes) {
        if (e == cudaSuccess && bytes)
            e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
    };
    H2D(w + o_soff, soff.data(), nsets * 8);
    H2D(w + o_spad, spad.data(), nsets * 4);
    H2D(w + o_coff, coff.data(), (nsets + 1) * 8);
    H2D(w + o_loff, loff.data(), (nsets + 1) * 8);
    H2D(w + o_items0, sorted_items.data(), (size_t)nitems0 * 16);
    H2D(w + o_order, set_order.data(), nsets * 4);
    if (host) {
        H2D((void *)d_charges, charges, (size_t)Pt * 16);
        H2D((void *)d_sx, sx, (size_t)N * 4);
        H2D((void *)d_sy, sy, (size_t)N * 4);
        H2D((void *)d_sz, sz, (size_t)N * 4);
        if (steps_per_line)
            H2D((void *)d_spl, steps_per_line, (size_t)N * 4);
    }
    if (e != cudaSuccess)
        return map_cuda(e);
    if ((e = prepare_batch_trace(smem)) != cudaSuccess)
        return map_cuda(e);

    // control block: [0] nitems0, [4] item ctr 0, [8] next nitems, [12] next ctr,
    // [16] cont count (u64), [24] evals (u64)
    unsigned char *ctl = w + o_ctl;
    int *nitems0_d = reinterpret_cast<int *>(ctl);
    unsigned *ctr0 = reinterpret_cast<unsigned *>(ctl + 4);
    int *nitemsn = reinterpret_cast<int *>(ctl + 8);
    unsigned *ctrn = reinterpret_cast<unsigned *>(ctl + 12);
    unsigned long long *cont_count = reinterpret_cast<unsigned long long *>(ctl + 16);
    unsigned long long *evals = reinterpret_cast<unsigned long long *>(ctl + 24);

    BatchParams P{};
    P.staged = reinterpret_cast<const float4 *>(w + o_staged);
    P.soff = reinterpret_cast<const long long *>(w + o_soff);
    P.spad = reinterpret_cast<const int *>(w + o_spad);
    P.snneg = reinterpret_cast<const int *>(w + o_snneg);
    P.sqabs = reinterpret_cast<const float *>(w + o_sqabs);
    P.coff = reinterpret_cast<const long long *>(w + o_coff);
    P.sx = d_sx;
    P.sy = d_sy;
    P.sz = d_sz;
    P.steps_per_line = d_spl;
    P.max_steps = max_steps;
    P.nlines = N;
    P.cont_in = reinterpret_cast<const long long *>(w + o_conts);
    float *S = reinterpret_cast<float *>(w + o_st);
    P.st_x = S;
    P.st_y = S + N;
    P.st_z = S + 2 * N;
    P.st_s = reinterpret_cast<int *>(S + 3 * N);
    P.cont_out = reinterpret_cast<long long *>(w + o_cont);
    P.cont_count = cont_count;
    P.vx = d_vx;
    P.vy = d_vy;
    P.vz = d_vz;
    P.store_rows = store_rows;
    P.lx = d_lx;
    P.ly = d_ly;
    P.lz = d_lz;
    P.len = d_len;
    P.cls = d_cls;
    P.res = resolution;
    P.term_r2 = (double)term_radius * (double)term_radius;
    P.evals = evals;
    P.resident_cap = resident_cap;
    P.tile_recs = tile;
    P.stages = stages;
    P.regroup = o.deterministic ? 0 : 1;
    P.err = c.err;

    BatchQueues Q{};
    Q.cont = P.cont_out;
    Q.cont_count = cont_count;
    Q.cont_sorted = reinterpret_cast<long long *>(w + o_conts);
    int *sq = reinterpret_cast<int *>(w + o_setq);
    Q.set_count = sq;
    Q.set_fill = sq + nsets;
    Q.set_item_off = sq + 2 * nsets;
    Q.set_line_off = reinterpret_cast<long long *>(w + o_setq + ((nsets * 12 + 7) / 8) * 8);
    Q.next_items = reinterpret_cast<int4 *>(w + o_itemsn);
    Q.next_nitems = nitemsn;
    Q.next_item_ctr = ctrn;
    Q.set_order = reinterpret_cast<const int *>(w + o_order);

    const int threads = 1024; // 31 compute warps + 1 copy warp
    H2D(nitems0_d, &nitems0, 4);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st); // pageable sources are consumed before capture
    if (e != cudaSuccess)
        return map_cuda(e);
    auto enqueue = [&]() -> cudaError_t {
        // counters after nitems0 (which stays)
        cudaError_t r = cudaMemsetAsync(ctl + 4, 0, 60, st);
        if (r == cudaSuccess)
            r = cudaMemsetAsync(c.err, 0, sizeof(int), st);
        if (r == cudaSuccess)
            r = launch_batch_stage(d_charges, reinterpret_cast<const long long *>(w + o_coff),
                                   P.soff, P.spad, gran, (int)nsets,
                                   reinterpret_cast<float *>(w + o_staged),
                                   reinterpret_cast<int *>(w + o_snneg),
                                   reinterpret_cast<float *>(w + o_sqabs), st);
        int budget = first_budget;
        for (int ph = 0; ph < phases && r == cudaSuccess; ++ph) {
            BatchParams Pp = P;
            Pp.phase = ph;
            Pp.items = ph == 0 ? reinterpret_cast<const int4 *>(w + o_items0) : Q.next_items;
            Pp.nitems = ph == 0 ? nitems0_d : nitemsn;
            Pp.item_ctr = ph == 0 ? ctr0 : ctrn;
            Pp.budget = (ph == phases - 1 || budget >= max_steps) ? 0 : budget;
            r = launch_batch_trace(Pp, tpl, c.nsm, threads, smem, st);
            if (r == cudaSuccess && ph + 1 < phases)
                r = launch_batch_sort(Q, reinterpret_cast<const long long *>(w + o_loff),
                                      (int)nsets, cont_lines, st);
            budget = budget > INT_MAX / 4 ? INT_MAX : budget * 4;
        }
        return r;
    };

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    if (o.use_graph) {
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t r = enqueue();
            e = cudaStreamEndCapture(st, &graph);
            if (r != cudaSuccess)
                e = r;
        }
        if (e == cudaSuccess)
            e = cudaGraphInstantiate(&gexec, graph, 0);
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev0, st);
    if (e == cudaSuccess)
        e = o.use_graph ? cudaGraphLaunch(gexec, st) : enqueue();
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev1, st);
    if (e == cudaSuccess && host) {
        auto D2H = [&](void *h, const void *d, size_t bytes) {
            if (e == cudaSuccess && bytes)
                e = cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st);
        };
        D2H(lx, d_lx, (size_t)N * 4);
        D2H(ly, d_ly, (size_t)N * 4);
        D2H(lz, d_lz, (size_t)N * 4);
        D2H(len, d_len, (size_t)N * 4);
        D2H(cls, d_cls, (size_t)N * 4);
        if (store_rows > 0) {
            D2H(vx, d_vx, (size_t)store_rows * N * 4);
            D2H(vy, d_vy, (size_t)store_rows * N * 4);
            D2H(vz, d_vz, (size_t)store_rows * N * 4);
        }
    }
    unsigned long long ev = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&ev, evals, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) {
        int dev_err = 0;
        code = read_dev_err(c, st, &dev_err);
    } else {
        code = map_cuda(e);
    }
    if (gexec)
        cudaGraphExecDestroy(gexec);
    if (graph)
        cudaGraphDestroy(graph);
    if (code)
        return code;
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (perf) {
        perf->time = ms * 1e-3;
        perf->pairs = (double)ev;
        perf->performance = 0;
        perf->wall_time = std::chrono::duration<double>(clock::now() - t_start).count();
        perf->progress = 1.0;
    }
    return EM_OK;
}

} // namespace
} // namespace em

extern "C" int em_trace_batch_f32(size_t nsets, const float *charges, const int64_t *charge_off,
                                  const float *sx, const float *sy, const float *sz,
                                  const int64_t *line_off, const int32_t *steps_per_line,
                                  int max_steps, float resolution, float term_radius,
                                  int store_rows, float *vx, float *vy, float *vz, float *lx,
                                  float *ly, float *lz, int32_t *len, int32_t *cls,
                                  const em_batch_options *opt, em_perf *perf)
{
    return em::trace_batch(nsets, charges, charge_off, sx, sy, sz, line_off, steps_per_line,
                           max_steps, resolution, term_radius, store_rows, vx, vy, vz, lx, ly,
                           lz, len, cls, opt, perf);
}
