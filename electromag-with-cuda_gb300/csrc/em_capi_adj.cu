// C ABI of the adjoint (em_adjoint_f32): forward trace, loss, backward.
#include <algorithm>
#include <chrono>
#include <climits>
#include <mutex>

#include "em_internal.h"
#include "em_plan.h"
#include "emgb300.h"

namespace em {
namespace {

constexpr int kSeg = 64; // rows per backward segment (line-state checkpoints)

int adjoint(float *x, float *y, float *z, size_t n, size_t rows, const float *charges,
            size_t p, float resolution, int use_curvature, const float *tx, const float *ty,
            const float *tz, double *loss, double *grad, const em_options *opt, em_perf *fwd,
            em_perf *bwd)
{
    using clock = std::chrono::steady_clock;
    const auto t_start = clock::now();
    if (!n)
        return EM_ERR_N_ZERO;
    if (resolution == 0)
        return EM_ERR_RESOLUTION;
    if (rows < 2)
        return EM_ERR_STEPS;
    if (!x || !y || !z || !charges || !p || !tx || !ty || !tz || !loss || !grad)
        return EM_ERR_ARG;
    em_options o{};
    if (opt)
        o = *opt;
    if (rows > (size_t)INT_MAX || p > 14000 || n > (size_t)(LLONG_MAX / 64) / rows)
        return EM_ERR_TOO_LARGE;
    if (o.device_ptrs && ((uintptr_t)charges & 15))
        return EM_ERR_ARG;

    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);

    AdjFused af{};
    const bool fused = adjoint_fused_plan((int)p, c.nsm, &af) != 0;
    const bool stored = fused && !o.adjoint_checkpoint;
    // forward shape: 8 lanes per line, one line per lane, scalar pairs, in
    // both modes (the order the field recompute repeats bit for bit, so the
    // two modes trace the same vertices)
    em_options fo{};
    fo.threads_per_line = 8;
    fo.lines_per_thread = 1;
    fo.pack = EM_PACK_SCALAR;
    Plan pl;
    if ((code = make_plan<float>(c, n, p, fo, &pl)))
        return code;
    if (!pl.cfg.resident && !stored)
        return EM_ERR_TOO_LARGE;
    const size_t elems = n * rows;
    cudaStream_t s = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;
    const int p_stage = fused ? std::max(pl.p_pad, af.p_bwd) : pl.p_pad;

    // the fused backward's lane-pair copy of the records follows the plain ones
    if ((code = grow(&c.charges, &c.charges_cap,
                     (size_t)(p_stage + (fused ? af.p_bwd : 0)) * 16)))
        return code;
    if ((code = grow(&c.charges_raw, &c.charges_raw_cap, p * 16 + 16)))
        return code;
    if ((code = grow(&c.errbuf, &c.errbuf_cap, 256)))
        return code;
    c.err = static_cast<int *>(c.errbuf);
    const long long recs = (long long)kSeg * (long long)n;
    int slices;
    if (fused) {
        slices = (int)std::min<long long>(64, af.teams);
    } else {
        const int cb = adjoint_charge_blocks((int)p);
        slices = (int)std::max<long long>(
            1, std::min<long long>(std::max(1, 4 * c.nsm / cb), (recs + 2047) / 2048));
    }
    // adjoint workspace: abar (3n f32); records (6 * seg * n f32, two-pass)
    // or the field (3 * rows * n f32 stored, 3 * 2 seg * n f32 recomputed) and
    // the team partials (teams * 4 * p_bwd float2, fused); slice partials
    // (slices * p * 4 f64); the loss and its per-CTA partials, then grad (4p f64)
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t field_rows = stored ? rows : 2 * (size_t)kSeg; // two halves when recomputed
    const size_t off_rec = up(3 * n * 4);
    const size_t rec_bytes = fused ? 3 * field_rows * n * 4 : 6 * (size_t)recs * 4;
    const size_t off_tpart = off_rec + up(rec_bytes);
    const size_t tpart_bytes = fused ? (size_t)af.teams * 4 * (size_t)af.p_bwd * 8 : 0;
    const size_t off_part = off_tpart + up(tpart_bytes);
    const size_t off_loss = off_part + up((size_t)slices * p * 4 * 8);
    const size_t off_grad = off_loss + up(8 * (1 + (size_t)adjoint_loss_parts(c.nsm)));
    const size_t need = off_grad + 4 * p * 8;
    if ((code = grow(&c.adj, &c.adj_cap, need)))
        return code;
    unsigned char *ws = static_cast<unsigned char *>(c.adj);

    float *dx = x, *dy = y, *dz = z;
    const float *dtx = tx, *dty = ty, *dtz = tz;
    if (!o.device_ptrs) {
        if ((code = grow(&c.lines, &c.lines_cap, 3 * elems * 4)))
            return code;
        if ((code = grow(&c.scratch, &c.scratch_cap, 3 * elems * 4)))
            return code;
        dx = static_cast<float *>(c.lines);
        dy = dx + elems;
        dz = dy + elems;
        float *t = static_cast<float *>(c.scratch);
        dtx = t;
        dty = t + elems;
        dtz = t + 2 * elems;
    }
    cudaError_t e = cudaMemsetAsync(c.err, 0, sizeof(int), s);
    const cudaMemcpyKind kin = o.device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(c.charges_raw, charges, p * 16, kin, s);
    if (e == cudaSuccess)
        e = launch_stage_charges<float>(c.charges_raw, (int)p, c.charges, p_stage, 0,
                                        pl.cfg.tile_recs, s);
    void *paired = static_cast<float4 *>(c.charges) + p_stage;
    if (e == cudaSuccess && fused)
        e = launch_adjoint_pair_stage(c.charges, af.p_bwd, af.team_warps, paired, s);
    if (e == cudaSuccess && !o.device_ptrs) {
        const float *src[6] = {x, y, z, tx, ty, tz};
        float *dst[6] = {dx, dy, dz, const_cast<float *>(dtx), const_cast<float *>(dty),
                         const_cast<float *>(dtz)};
        for (int k = 0; k < 6 && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(dst[k], src[k], (k < 3 ? n : elems) * 4,
                                cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess)
        e = cudaMemsetAsync(ws + off_tpart, 0, off_grad - off_tpart, s);
    if (e != cudaSuccess)
        return map_cuda(e);

    RefTraceParams<float> prm{};
    prm.x = dx;
    prm.y = dy;
    prm.z = dz;
    prm.charges = c.charges;
    prm.n = (long long)n;
    prm.n_groups = pl.n_groups;
    prm.total_steps = (int)rows;
    prm.p_pad = pl.p_pad;
    prm.n_tiles = pl.n_tiles;
    prm.tile_recs = pl.cfg.tile_recs;
    prm.stages = pl.cfg.stages;
    prm.resident = pl.cfg.resident;
    prm.rule = use_curvature ? RULE_SSE : RULE_FIXED;
    prm.resolution = resolution;
    prm.err = c.err;
    float *fbuf = reinterpret_cast<float *>(ws + off_rec);
    const size_t fstride = field_rows * n;
    if (stored) {
        prm.fx = fbuf;
        prm.fy = fbuf + fstride;
        prm.fz = fbuf + 2 * fstride;
    }

    AdjParams ap{};
    ap.x = dx;
    ap.y = dy;
    ap.z = dz;
    ap.tx = dtx;
    ap.ty = dty;
    ap.tz = dtz;
    ap.charges = c.charges;
    ap.raw = static_cast<const float *>(c.charges_raw);
    ap.p = (int)p;
    ap.p_pad = pl.p_pad;
    ap.n = (long long)n;
    ap.rows = (int)rows;
    ap.seg = kSeg;
    ap.resolution = resolution;
    ap.curvature = use_curvature ? 1 : 0;
    ap.abar = reinterpret_cast<float *>(ws);
    ap.rec = reinterpret_cast<float *>(ws + off_rec);
    ap.rec_stride = (size_t)recs;
    ap.gpart = reinterpret_cast<double *>(ws + off_part);
    ap.slices = slices;
    ap.err = c.err;
    if (fused) {
        ap.fx = fbuf;
        ap.fy = fbuf + fstride;
        ap.fz = fbuf + 2 * fstride;
        ap.f_row0 = 0;
        ap.stored = stored ? 1 : 0;
        ap.tpart = reinterpret_cast<float2 *>(ws + off_tpart);
        ap.p_bwd = af.p_bwd;
        ap.charges_bwd = paired;
        ap.team_warps = af.team_warps;
        ap.teams = af.teams;
    }
    double *dloss = reinterpret_cast<double *>(ws + off_loss);
    double *dgrad = reinterpret_cast<double *>(ws + off_grad);

    cudaEvent_t ev2 = nullptr;
    e = cudaEventCreate(&ev2);
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev0, s);
    if (e == cudaSuccess)
        e = launch_ref_trace<float>(prm, pl.cfg, pl.arith, s);
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev1, s);
    if (e == cudaSuccess)
        e = launch_adjoint_backward(ap, fused ? &af : nullptr, c.nsm,
                                    128 + (size_t)pl.p_pad * 16, dloss, dgrad, s, c.copy_stream,
                                    (size_t)kSeg * n);
    if (e == cudaSuccess)
        e = cudaEventRecord(ev2, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(loss, dloss, 8, o.device_ptrs ? cudaMemcpyDeviceToDevice
                                                         : cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(grad, dgrad, 4 * p * 8,
                            o.device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            s);
    if (e == cudaSuccess && !o.device_ptrs) {
        e = cudaMemcpyAsync(x + n, dx + n, (elems - n) * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(y + n, dy + n, (elems - n) * 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(z + n, dz + n, (elems - n) * 4, cudaMemcpyDeviceToHost, s);
    }
    int dev_err = 0;
    if (e == cudaSuccess)
        code = read_dev_err(c, s, &dev_err);
    else
        code = map_cuda(e);
    float ms_f = 0, ms_b = 0;
    if (code == EM_OK) {
        cudaEventElapsedTime(&ms_f, c.ev0, c.ev1);
        cudaEventElapsedTime(&ms_b, c.ev1, ev2);
    }
    if (ev2)
        cudaEventDestroy(ev2);
    if (code)
        return code;
    const double pairs = (double)n * (double)(rows - 1) * (double)p;
    const double wall = std::chrono::duration<double>(clock::now() - t_start).count();
    if (fwd) {
        fwd->time = ms_f * 1e-3;
        fwd->pairs = pairs;
        fwd->performance = fwd->time > 0 ? pairs * 20.0 / fwd->time / 1e9 : 0;
        fwd->wall_time = wall;
        fwd->progress = 1.0;
    }
    if (bwd) {
        bwd->time = ms_b * 1e-3;
        // pair passes: fused (1), plus the field recompute (2), or the
        // recompute, Jacobian-vector and charge passes (3)
        bwd->pairs = (stored ? 1 : fused ? 2 : 3) * pairs;
        bwd->performance = 0;
        bwd->wall_time = wall;
        bwd->progress = 1.0;
    }
    return EM_OK;
}

} // namespace
} // namespace em

extern "C" int em_adjoint_f32(float *x, float *y, float *z, size_t n, size_t rows,
                              const float *charges, size_t p, float resolution, int use_curvature,
                              const float *tx, const float *ty, const float *tz, double *loss,
                              double *grad, const em_options *opt, em_perf *fwd, em_perf *bwd)
{
    return em::adjoint(x, y, z, n, rows, charges, p, resolution, use_curvature, tx, ty, tz, loss,
                       grad, opt, fwd, bwd);
}
