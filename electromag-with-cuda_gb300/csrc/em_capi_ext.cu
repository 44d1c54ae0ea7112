// C ABI of the extended tracer (em_trace_lines_*) and of the seeding helper.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>

#include "em_internal.h"
#include "em_plan.h"
#include "emgb300.h"

namespace em {
namespace {

// Layout of the per-device status block (DevCtx::errbuf, 256 B).
constexpr size_t kOffMeta = 16, kOffQabs = 20, kOffNext = 32, kOffEvals = 40,
                 kOffRefines = 48, kOffContCount = 56, kOffContNext = 64, kOffLive = 72,
                 kOffContCount2 = 80;

template <class T>
int trace_lines(T *x, T *y, T *z, size_t n, size_t max_steps, const int32_t *spl,
                const T *charges, size_t p, T resolution, T term_radius, int32_t *len,
                int32_t *cls, T *ex, T *ey, T *ez, const em_options *opt, em_perf *perf)
{
    using clock = std::chrono::steady_clock;
    const auto t_start = clock::now();
    if (!n)
        return EM_ERR_N_ZERO;
    if (resolution == 0)
        return EM_ERR_RESOLUTION;
    if (max_steps < 1)
        return EM_ERR_STEPS;
    if (!x || !y || !z || !len || !cls || (p && !charges))
        return EM_ERR_ARG;
    const bool want_field = ex || ey || ez;
    if (want_field && !(ex && ey && ez))
        return EM_ERR_ARG;
    em_options o{};
    if (opt)
        o = *opt;
    const int mode = o.precision == EM_PREC_MIXED  ? EXT_MIXED
                     : o.precision == EM_PREC_DF64 ? EXT_DF64
                                                   : EXT_FAST;
    if (o.precision != EM_PREC_FP32 && o.precision != EM_PREC_MIXED &&
        o.precision != EM_PREC_DF64)
        return EM_ERR_ARG;
    if (mode != EXT_FAST && sizeof(T) != 4)
        return EM_ERR_ARG;
    if (o.refine != EM_REFINE_FP64 && o.refine != EM_REFINE_DF64)
        return EM_ERR_ARG;
    if (!(term_radius >= 0) || !(o.null_frac >= 0) || !(o.refine_kappa >= 0))
        return EM_ERR_ARG;
    if (max_steps > (size_t)INT_MAX || p > (size_t)(INT_MAX / 64) ||
        n > (size_t)(LLONG_MAX / 64) / max_steps)
        return EM_ERR_TOO_LARGE;
    if (o.device_ptrs && ((uintptr_t)charges & 15))
        return EM_ERR_ARG;
    const int tpl = o.threads_per_line ? o.threads_per_line : 8;
    if (tpl != 4 && tpl != 8 && tpl != 16 && tpl != 32)
        return EM_ERR_ARG;
    // launch-shape overrides (0: the library's choice); a tile beyond 65 536
    // records could never fit shared memory
    if (o.warps_per_cta < 0 || o.warps_per_cta > 32 || o.tile_charges < 0 ||
        o.tile_charges > 65536)
        return EM_ERR_ARG;
    if (perf)
        perf->progress = 0;

    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);

    // ---- plan: one persistent CTA per SM, all charges resident if they fit
    const size_t rec = sizeof(T) * 4;
    const size_t smem_cap = std::min<size_t>(c.smem_optin, 227 * 1024);
    const int gran = tpl;
    const long long p_min = ceil_div((long long)p, gran) * gran + gran;
    LaunchCfg cfg{};
    cfg.tpl = tpl;
    cfg.kl = 1;
    cfg.grid = c.nsm;
    const int cta_warps = ext_cta_threads(mode) / 32;
    cfg.resident = !o.force_streamed && 128 + (size_t)p_min * rec <= smem_cap;
    int p_pad, n_tiles, tile;
    if (cfg.resident) {
        p_pad = (int)p_min;
        n_tiles = 1;
        tile = p_pad;
        cfg.stages = 1;
        cfg.warps = std::min(o.warps_per_cta ? o.warps_per_cta : 32, cta_warps);
        cfg.smem = 128 + (size_t)p_pad * rec;
    } else {
        tile = o.tile_charges ? o.tile_charges : (rec == 16 ? 1024 : 512);
        tile = (tile + gran - 1) / gran * gran;
        cfg.stages = 4;
        while (cfg.stages > 2 && 128 + (size_t)cfg.stages * tile * rec > smem_cap)
            --cfg.stages;
        if (128 + (size_t)cfg.stages * tile * rec > smem_cap)
            return EM_ERR_ARG;
        n_tiles = (int)ceil_div(p_min, tile);
        if (!o.tile_charges) {
            // the same number of tiles, evened out: no nearly empty last
            // tile of pad records (p = 16384 would pay 6 % more pairs)
            tile = (int)(ceil_div(ceil_div(p_min, n_tiles), gran) * gran);
        }
        p_pad = n_tiles * tile;
        cfg.warps = std::min(o.warps_per_cta ? o.warps_per_cta : 31, cta_warps - 1);
        cfg.smem = 128 + (size_t)cfg.stages * tile * rec;
    }
    cfg.tile_recs = tile;

    // ---- buffers
    if ((code = grow(&c.charges, &c.charges_cap, (size_t)p_pad * rec)))
        return code;
    if ((code = grow(&c.charges_raw, &c.charges_raw_cap, p * rec + 16)))
        return code;
    if ((code = grow(&c.errbuf, &c.errbuf_cap, 256)))
        return code;
    c.err = static_cast<int *>(c.errbuf);
    unsigned char *status = static_cast<unsigned char *>(c.errbuf);
    cudaStream_t s = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;

    const size_t elems = n * max_steps;
    T *dx = x, *dy = y, *dz = z, *dex = ex, *dey = ey, *dez = ez;
    int32_t *dlen = len, *dcls = cls;
    const int32_t *dspl = spl;
    if (!o.device_ptrs) {
        if ((code = grow(&c.lines, &c.lines_cap, 3 * elems * sizeof(T))))
            return code;
        dx = static_cast<T *>(c.lines);
        dy = dx + elems;
        dz = dy + elems;
        const size_t meta_bytes = (3 * n * sizeof(int32_t) + 255) / 256 * 256;
        const size_t need = meta_bytes + (want_field ? 3 * elems * sizeof(T) : 0);
        if ((code = grow(&c.scratch, &c.scratch_cap, need)))
            return code;
        unsigned char *b = static_cast<unsigned char *>(c.scratch);
        dlen = reinterpret_cast<int32_t *>(b);
        dcls = dlen + n;
        dspl = spl ? dcls + n : nullptr;
        if (want_field) {
            dex = reinterpret_cast<T *>(b + meta_bytes);
            dey = dex + elems;
            dez = dey + elems;
        }
    }
    // tail hand-off (not in deterministic mode: the tail kernels sum a
    // line's charges in another grouping): the lines left once at most half
    // the warp slots would hold one each go to the tail kernels.  With
    // streamed tiles every warp of a CTA waits on every tile, so a few long
    // lines on a few warps hold whole SMs; spread over many warps they use
    // them.  With resident charges a lone line gains from more warps as
    // long as each warp keeps enough pairs per row (w_cap below).
    LaunchCfg wcfg = cfg;
    wcfg.warps = kExtWideThreads / 32 - (cfg.resident ? 0 : 1);
    int wide_tiles = n_tiles;
    if (!cfg.resident) {
        // streamed: a wide group splits every tile W ways, so its warps
        // take the staged tiles up to four at a time (the last one
        // shorter), in as many stages (2..4) as fit beside the static slots:
        // fewer waits and loop set-ups per pair
        const size_t room = smem_cap > kExtWideSlots + 128 ? smem_cap - kExtWideSlots - 128 : 0;
        for (int m = 4; m >= 1; m >>= 1) {
            const size_t tb = (size_t)tile * m * rec;
            if (2 * tb <= room) {
                wcfg.tile_recs = tile * m;
                wcfg.stages = (int)std::min<size_t>(4, room / tb);
                wcfg.smem = 128 + (size_t)wcfg.stages * tb;
                wide_tiles = (int)ceil_div(n_tiles, m);
                break;
            }
        }
    }
    // with resident charges a warp's share of a row must outweigh the
    // per-row reductions, the barrier and the step, which every warp of a
    // group runs (FP32) or waits for: at least 16 FP32 pairs per lane
    // (about 14 instructions each), 12 mixed, 6 double-float, 1 FP64
    // (measured on the GPU-scale set with termination, resident-charge tail
    // kernel: 8 / 6 pairs per lane (16 warps for a lone line) gave 8.9 /
    // 15.7 ms for FP32 / mixed, 16 / 12 (8 warps) 8.8 / 15.3, 32 / 24 (4
    // warps) 9.0 / 15.5; double-float at 6 pairs: 44.3 ms); below two warps
    // per line the lane-group kernel's regrouping (a warp per line) serves
    // the tail better.  Streamed rows also wait on the tile ring, so there
    // the count alone sets W.
    int w_cap = wcfg.warps;
    if (cfg.resident) {
        const long long per_lane = sizeof(T) == 8       ? 1
                                   : mode == EXT_DF64  ? 6
                                   : mode == EXT_MIXED ? 12
                                                       : 16;
        w_cap = (int)std::min<long long>(wcfg.warps, p_pad / (32LL * per_lane));
    }
    const bool tail = !o.deterministic && !o.warps_per_cta && w_cap >= 2 &&
                      wcfg.smem + kExtWideSlots <= c.smem_optin;
    const long long tail_lines = tail ? (long long)c.nsm * wcfg.warps / 2 : 0;
    if (tail && (code = grow(&c.tail, &c.tail_cap, 2 * n * sizeof(ExtCont<T>))))
        return code;
    cudaError_t e = cudaMemsetAsync(c.errbuf, 0, 88, s);
    const unsigned long long n_live = n;
    if (e == cudaSuccess && tail)
        e = cudaMemcpyAsync(status + kOffLive, &n_live, sizeof(n_live), cudaMemcpyHostToDevice,
                            s);
    const cudaMemcpyKind kin = o.device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (e == cudaSuccess && p)
        e = cudaMemcpyAsync(c.charges_raw, charges, p * rec, kin, s);
    if (e == cudaSuccess)
        e = launch_ext_stage<T>(c.charges_raw, (int)p, c.charges, p_pad, gran,
                                mode == EXT_MIXED ? tile : 0,
                                reinterpret_cast<int *>(status + kOffMeta),
                                reinterpret_cast<float *>(status + kOffQabs), s);
    if (e == cudaSuccess && !o.device_ptrs) {
        e = cudaMemcpyAsync(dx, x, n * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dy, y, n * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dz, z, n * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && spl)
            e = cudaMemcpyAsync(const_cast<int32_t *>(dspl), spl, n * sizeof(int32_t),
                                cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess)
        return map_cuda(e);

    ExtParams<T> prm{};
    prm.x = dx;
    prm.y = dy;
    prm.z = dz;
    prm.ex = dex;
    prm.ey = dey;
    prm.ez = dez;
    prm.charges = c.charges;
    prm.meta = reinterpret_cast<const int *>(status + kOffMeta);
    prm.qabs = reinterpret_cast<const float *>(status + kOffQabs);
    prm.n = (long long)n;
    prm.max_steps = (int)max_steps;
    prm.steps_per_line = dspl;
    prm.resolution = (double)resolution;
    prm.term_r2 = (double)term_radius * (double)term_radius;
    prm.null_frac = o.null_frac;
    {
        const double kappa = mix_kappa(o);
        prm.kappa2 = kappa * kappa;
    }
    prm.len = dlen;
    prm.cls = dcls;
    prm.next_line = reinterpret_cast<unsigned long long *>(status + kOffNext);
    prm.evals = reinterpret_cast<unsigned long long *>(status + kOffEvals);
    prm.refines = reinterpret_cast<unsigned long long *>(status + kOffRefines);
    prm.p_pad = p_pad;
    prm.n_tiles = n_tiles;
    prm.tile_recs = tile;
    prm.stage_recs = tile;
    prm.stages = cfg.stages;
    prm.resident = cfg.resident;
    prm.regroup = o.deterministic ? 0 : 1;
    prm.refine_fp64 = o.refine == EM_REFINE_FP64 ? 1 : 0;
    prm.err = c.err;
    prm.cont = c.tail;
    prm.cont_count = reinterpret_cast<unsigned long long *>(status + kOffContCount);
    prm.cont_next = reinterpret_cast<unsigned long long *>(status + kOffContNext);
    prm.live_count = reinterpret_cast<unsigned long long *>(status + kOffLive);
    prm.tail_lines = tail_lines;

    e = cudaEventRecord(c.ev0, s);
    if (e == cudaSuccess)
        e = launch_ext_trace<T>(prm, cfg, mode, s);
    if (e == cudaSuccess && tail) {
        // the handed-off lines, in rounds: each round gives a line as many
        // warps as fill the SMs, and hands its lines on to the next (wider)
        // round once few enough are left
        unsigned char *buf[2] = {static_cast<unsigned char *>(c.tail),
                                 static_cast<unsigned char *>(c.tail) + n * sizeof(ExtCont<T>)};
        unsigned long long *cnt[2] = {
            reinterpret_cast<unsigned long long *>(status + kOffContCount),
            reinterpret_cast<unsigned long long *>(status + kOffContCount2)};
        const int ncw = wcfg.warps;
        for (int round = 0; e == cudaSuccess && round < 64; ++round) {
            const int in = round & 1, out = in ^ 1;
            unsigned long long handed = 0;
            e = cudaMemcpyAsync(&handed, cnt[in], sizeof(handed), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(s);
            if (e != cudaSuccess || handed == 0)
                break;
            int w = 1, w_next = 0;
            for (int d = w_cap; d >= 1; --d) {
                if (ncw % d == 0 &&
                    (unsigned long long)c.nsm * (unsigned long long)(ncw / d) >= handed) {
                    w = d;
                    break;
                }
            }
            for (int d = w + 1; d <= w_cap; ++d) {
                if (ncw % d == 0) {
                    w_next = d;
                    break;
                }
            }
            const unsigned long long zero[2] = {0, 0};
            e = cudaMemcpyAsync(cnt[out], zero, sizeof(zero[0]), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(prm.cont_next, zero, sizeof(zero[0]),
                                    cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(prm.live_count, &handed, sizeof(handed),
                                    cudaMemcpyHostToDevice, s);
            prm.cont_in = buf[in];
            prm.cont_in_count = cnt[in];
            prm.cont = buf[out];
            prm.cont_count = cnt[out];
            prm.tail_lines = w_next ? (long long)c.nsm * (ncw / w_next) : 0;
            prm.wide = w;
            ExtParams<T> wp = prm;
            wp.n_tiles = wide_tiles;
            wp.tile_recs = wcfg.tile_recs;
            wp.stages = wcfg.stages;
            if (e == cudaSuccess)
                e = launch_ext_wide<T>(wp, wcfg, mode, s);
        }
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev1, s);
    if (e == cudaSuccess && !o.device_ptrs) {
        e = cudaMemcpyAsync(x, dx, elems * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(y, dy, elems * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(z, dz, elems * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(len, dlen, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(cls, dcls, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && want_field) {
            e = cudaMemcpyAsync(ex, dex, elems * sizeof(T), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ey, dey, elems * sizeof(T), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(ez, dez, elems * sizeof(T), cudaMemcpyDeviceToHost, s);
        }
    }
    unsigned long long cnt[3] = {0, 0, 0};
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(cnt, status + kOffNext, sizeof(cnt), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess)
        return map_cuda(e);
    int dev_err = 0;
    code = read_dev_err(c, s, &dev_err);
    if (code)
        return code;
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    if (perf) {
        const double tk = ms * 1e-3;
        perf->time = tk;
        perf->pairs = (double)cnt[1] * (double)p;
        perf->performance = tk > 0 ? (double)cnt[1] * (18.0 * (double)p + 13.0) / tk / 1e9 : 0;
        perf->fp64_refines = (double)cnt[2];
        perf->wall_time = std::chrono::duration<double>(clock::now() - t_start).count();
        perf->progress = 1.0;
    }
    return EM_OK;
}

} // namespace
} // namespace em

extern "C" {

int em_trace_lines_f32(float *x, float *y, float *z, size_t n, size_t max_steps,
                       const int32_t *steps_per_line, const float *charges, size_t p,
                       float resolution, float term_radius, int32_t *len, int32_t *cls,
                       float *ex, float *ey, float *ez, const em_options *opt, em_perf *perf)
{
    return em::trace_lines<float>(x, y, z, n, max_steps, steps_per_line, charges, p,
                                  resolution, term_radius, len, cls, ex, ey, ez, opt, perf);
}

int em_trace_lines_f64(double *x, double *y, double *z, size_t n, size_t max_steps,
                       const int32_t *steps_per_line, const double *charges, size_t p,
                       double resolution, double term_radius, int32_t *len, int32_t *cls,
                       double *ex, double *ey, double *ez, const em_options *opt,
                       em_perf *perf)
{
    return em::trace_lines<double>(x, y, z, n, max_steps, steps_per_line, charges, p,
                                   resolution, term_radius, len, cls, ex, ey, ez, opt, perf);
}

int em_seed_fibonacci_f32(const float *charges, size_t p, size_t lines_per_charge,
                          float radius, float *sx, float *sy, float *sz, size_t cap,
                          size_t *count)
{
    if ((p && !charges) || !count || (cap && (!sx || !sy || !sz)))
        return EM_ERR_ARG;
    const double ga = M_PI * (3.0 - std::sqrt(5.0)); // golden angle
    size_t w = 0;
    for (size_t j = 0; j < p && w < cap; ++j) {
        if (!(charges[4 * j + 3] > 0))
            continue;
        for (size_t i = 0; i < lines_per_charge && w < cap; ++i) {
            const double zz = 1.0 - (2.0 * (double)i + 1.0) / (double)lines_per_charge;
            const double rr = std::sqrt(1.0 - zz * zz);
            const double ph = ga * (double)i;
            sx[w] = (float)((double)charges[4 * j + 0] + radius * rr * std::cos(ph));
            sy[w] = (float)((double)charges[4 * j + 1] + radius * rr * std::sin(ph));
            sz[w] = (float)((double)charges[4 * j + 2] + radius * zz);
            ++w;
        }
    }
    *count = w;
    return EM_OK;
}

} // extern "C"
