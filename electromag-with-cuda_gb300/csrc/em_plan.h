// Per-device state and launch planning for the tracer kernels.
#pragma once

#include <algorithm>
#include <cstddef>
#include <mutex>

#include "em_internal.h"
#include "emgb300.h"

namespace em {

constexpr int kMaxDevices = 64;

// Mixed arithmetic on the reference-layout tracer: a vertex's field is
// re-evaluated in double-float where the terms' size, sqrt(sum_j |t_j|^2),
// exceeds this multiple of |E| (the FP32 sum's error grows with it).
constexpr double kMixKappaDefault = 2.5;

// The conditioning bound of a call: refine_kappa when given, else
// 1/null_frac when given (re-evaluate where |E| is below that fraction of
// the terms' size), else the default.
inline double mix_kappa(const em_options &o)
{
    if (o.refine_kappa > 0)
        return o.refine_kappa;
    if (o.null_frac > 0)
        return 1.0 / o.null_frac;
    return kMixKappaDefault;
}

// Cached per-device state.  `mu` serialises calls on one device; buffers
// only grow and are released by em_release().
struct DevCtx {
    std::mutex init_mu, mu;
    bool ready = false;
    int device = 0;
    int nsm = 0;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr; // device-to-host copies overlapped with tracing
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_chunk = nullptr;
    cudaEvent_t ev_rows[8] = {}; // end of each row chunk's trace (progress)
    void *charges = nullptr; // staged (padded, possibly paired) charges
    size_t charges_cap = 0;
    void *charges_raw = nullptr; // the caller's records, copied as given
    size_t charges_raw_cap = 0;
    void *lines = nullptr;
    size_t lines_cap = 0;
    void *errbuf = nullptr;
    size_t errbuf_cap = 0;
    void *scratch = nullptr; // field-at-points / extended / adjoint staging
    size_t scratch_cap = 0;
    void *adj = nullptr;     // adjoint workspace
    size_t adj_cap = 0;
    void *batch = nullptr;   // batched-tracer workspace
    size_t batch_cap = 0;
    void *tail = nullptr;    // extended tracer: handed-off lines
    size_t tail_cap = 0;
    int *err = nullptr;
};

DevCtx *get_ctx(int *code);
int grow(void **buf, size_t *cap, size_t need);
int map_cuda(cudaError_t e);
int read_dev_err(DevCtx &c, cudaStream_t s, int *dev_err_host);

struct Plan {
    LaunchCfg cfg{};
    int arith = ARITH_FAST; // resolved kernel arithmetic (Arith)
    long long n_groups = 0;
    int p_pad = 0;
    int n_tiles = 0;
};

inline long long ceil_div(long long a, long long b) { return (a + b - 1) / b; }

// Staged charge layout for a kernel arithmetic (stage_kernel's `paired`).
inline int stage_layout(int arith)
{
    return arith == ARITH_FAST2 || arith == ARITH_MIXED ? 1 : 0;
}

// Relative cost of one line-group step for `tpl` threads per line and `kl`
// lines per lane: pair work per lane (one charge load per kl pairs) plus
// the butterfly and the per-vertex step.
inline double group_step_cost(long long p, int tpl, int kl)
{
    int lg = 0;
    for (int t = tpl; t > 1; t >>= 1)
        ++lg;
    return kl * ((double)ceil_div(p, tpl) * (13.0 + 1.0 / kl) + 18.0 * lg + 120.0);
}

// Issue efficiency with w warps on the busiest SM sub-partition: too few
// warps cannot hide the FP32-pipe and MUFU latencies.  Fitted to measured
// traces of 16 384 lines x 1024 charges over every (tpl, kl) shape.
inline double smsp_efficiency(long long w)
{
    return w >= 4 ? 1.0 : w == 3 ? 0.95 : w == 2 ? 0.87 : 0.68;
}

// Group-steps on the busiest SM sub-partition (4 per SM) when w warps of
// one CTA run gpc line groups: full rounds of w warps, then a last round
// of the groups left over, each round at the issue efficiency of the warps
// it keeps busy (a short last round runs latency-bound).
inline double sm_rounds_cost(long long gpc, long long w)
{
    const long long rounds = ceil_div(gpc, w);
    const long long last = gpc - (rounds - 1) * w;
    const long long full = ceil_div(w, 4), tail = ceil_div(last, 4);
    return (double)(rounds - 1) * (double)full / smsp_efficiency(full) +
           (double)tail / smsp_efficiency(tail);
}

// Picks threads per line, lines per lane, compute warps per CTA and the
// grid for n lines and p charges on a device with nsm SMs (one persistent
// CTA per SM).  fixed_tpl / fixed_kl of 0 are searched, and so is the warp
// count up to max_warps (fewer warps can balance the rounds better: 54
// groups per SM at 24 warps leave a last round of 6).  Shapes are tried
// from (8, 2) down, most warps first, and a later one must be 2 % cheaper
// to replace an earlier one.
inline void choose_shape(long long n, long long p, int nsm, int max_warps, int fixed_tpl,
                         int fixed_kl, int *tpl_out, int *kl_out, int *warps_out)
{
    double best = 0;
    int bt = 1, bk = 1, bw = 1;
    for (int kl = 2; kl >= 1; --kl) {
        if (fixed_kl && kl != fixed_kl)
            continue;
        for (int tpl = 8; tpl >= 1; tpl >>= 1) {
            if (fixed_tpl && tpl != fixed_tpl)
                continue;
            const long long lpw = kl * 32 / tpl;
            const long long groups = ceil_div(n, lpw);
            const long long grid = std::min<long long>(nsm, groups);
            const long long gpc = ceil_div(groups, grid);
            const int wmax = (int)std::min<long long>(max_warps, gpc);
            const double step = group_step_cost(p, tpl, kl);
            for (int warps = wmax; warps >= 1; --warps) {
                const double t = sm_rounds_cost(gpc, warps) * step;
                if (best == 0 || t < best * 0.98) {
                    best = t;
                    bt = tpl;
                    bk = kl;
                    bw = warps;
                }
            }
        }
    }
    *tpl_out = bt;
    *kl_out = bk;
    *warps_out = bw;
}

template <class T>
int make_plan(const DevCtx &c, size_t n, size_t p, const em_options &o, Plan *pl)
{
    const size_t rec = sizeof(T) * 4;
    const int fixed_tpl = o.arith == EM_ARITH_EXACT
                              ? (sizeof(T) == 4 ? exact_tpl_f32((long long)n, c.nsm) : 1)
                              : o.threads_per_line;
    if (fixed_tpl != 0 && fixed_tpl != 1 && fixed_tpl != 2 && fixed_tpl != 4 && fixed_tpl != 8)
        return EM_ERR_ARG;
    // tile overrides beyond 65 536 records could never fit shared memory and
    // would overflow the granule rounding below
    if (o.warps_per_cta < 0 || o.warps_per_cta > 32 || o.tile_charges < 0 ||
        o.tile_charges > 65536)
        return EM_ERR_ARG;
    if (o.pack < EM_PACK_AUTO || o.pack > EM_PACK_PAIRS)
        return EM_ERR_ARG;
    if (o.arith == EM_ARITH_MIXED && sizeof(T) != 4)
        return EM_ERR_ARG;
    int arith = o.arith == EM_ARITH_EXACT   ? ARITH_EXACT
                : o.arith == EM_ARITH_MIXED ? ARITH_MIXED
                                            : ARITH_FAST;
    // packed pairs only on request: each .f32x2 FMA holds the FMA pipe for
    // two cycles, so it saves issue slots but not pipe time
    if (arith == ARITH_FAST && sizeof(T) == 4 && o.pack == EM_PACK_PAIRS)
        arith = ARITH_FAST2;
    if (o.lines_per_thread < 0 || o.lines_per_thread > 2)
        return EM_ERR_ARG;
    // lines per lane: searched for the fast scalar form when the caller does
    // not say (two lines share each charge load, one line doubles the warps
    // for small line counts); 2 for packed pairs, 1 for exact arithmetic
    // (mixed: 2 unless asked, in CTAs of at most 512 threads, whose 128
    // registers hold two lines' packed chunk sums, compensated sums and
    // FP64 positions)
    int fixed_kl = 1;
    if (arith == ARITH_FAST)
        fixed_kl = o.lines_per_thread;
    else if (arith == ARITH_MIXED)
        fixed_kl = o.lines_per_thread ? o.lines_per_thread : 2;
    else if (arith == ARITH_FAST2)
        fixed_kl = o.lines_per_thread ? o.lines_per_thread : 2;
    // the exact arithmetic with several lanes per line keeps each warp's
    // terms in shared memory beside the charges (up to a full CTA's warps)
    const size_t term_bytes = arith == ARITH_EXACT && fixed_tpl >= kExactSmemTpl
                                  ? (size_t)(exact_max_threads(fixed_tpl) / 32) *
                                        kExactTermBytesPerWarp
                                  : 0;
    const size_t smem_cap = std::min<size_t>(c.smem_optin, 227 * 1024) - term_bytes;
    int tpl = 1, kl = 1, warps = 1;
    // resident if the padded set fits next to the barrier block
    const size_t gran_max = 16 * kUnroll;
    const size_t p_res = (p + gran_max - 1) / gran_max * gran_max;
    const bool resident = !o.force_streamed && 128 + p_res * rec <= smem_cap;
    // the mixed form's per-line sums need more than 64 registers: at most
    // 512 threads (128 registers) per CTA
    const int max_warps = (arith == ARITH_MIXED   ? 16
                           : arith == ARITH_EXACT ? exact_max_threads(fixed_tpl) / 32
                                                  : 32) -
                          (resident ? 0 : 1);
    if (arith == ARITH_MIXED) {
        // the mixed form takes its groups from a queue, so rounds need no
        // balancing: 8 lanes x 2 lines (unless asked otherwise) and every
        // warp the groups can keep busy (on 32 736 lines x 4096 charges
        // 1971 Gpair/s, against 1826 with one line per lane and 1732 with
        // 4 lanes per line)
        tpl = fixed_tpl ? fixed_tpl : 8;
        kl = fixed_kl;
        const long long groups = ceil_div((long long)n, kl * 32 / tpl);
        warps = (int)std::min<long long>(max_warps, ceil_div(groups, c.nsm));
    } else {
        choose_shape((long long)n, (long long)p, c.nsm, max_warps, fixed_tpl, fixed_kl, &tpl,
                     &kl, &warps);
    }
    if (o.warps_per_cta)
        warps = std::min(o.warps_per_cta, max_warps);
    // records per padding granule: every lane gets whole unrolled groups
    const int gran = tpl * kUnroll * (stage_layout(arith) ? 2 : 1);
    Plan r;
    r.arith = arith;
    r.n_groups = ceil_div((long long)n, kl * 32 / tpl);
    r.cfg.tpl = tpl;
    r.cfg.kl = kl;
    r.cfg.warps = warps;
    r.cfg.grid = (int)std::min<long long>(c.nsm, r.n_groups);
    r.cfg.resident = resident ? 1 : 0;
    if (resident) {
        // at least one granule of pad records: a call without charges traces
        // a zero field (the reference then steps by 0/0 into NaN, code 0)
        r.p_pad = (int)((std::max<size_t>(p, 1) + gran - 1) / gran * gran);
        r.n_tiles = 1;
        r.cfg.stages = 1;
        r.cfg.tile_recs = r.p_pad;
        r.cfg.smem = 128 + (size_t)r.p_pad * rec + term_bytes;
    } else {
        int tile = o.tile_charges ? o.tile_charges : (rec == 16 ? 1024 : 512);
        tile = (tile + gran - 1) / gran * gran;
        r.cfg.stages = 4;
        while (r.cfg.stages > 2 && 128 + (size_t)r.cfg.stages * tile * rec > smem_cap)
            --r.cfg.stages;
        if (128 + (size_t)r.cfg.stages * tile * rec > smem_cap)
            return EM_ERR_ARG;
        r.n_tiles = (int)ceil_div((long long)p, tile);
        if (r.n_tiles == 0)
            r.n_tiles = 1;
        r.p_pad = r.n_tiles * tile;
        r.cfg.tile_recs = tile;
        r.cfg.smem = 128 + (size_t)r.cfg.stages * tile * rec + term_bytes;
    }
    *pl = r;
    return EM_OK;
}

} // namespace em
