// C ABI of libemgb300.so: argument checks in the reference's order, device
// buffers cached per device, launch planning, host<->device staging.
//
// Return codes 1/2/3/5 and their order follow CPU_Implement.cpp:213-230.
// The _f32/_f64 entry points take host pointers and return when the result
// is in the caller's arrays, like CalcField_CPU<T> (CPU_Implement.cpp:501).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdlib>
#include <climits>
#include <cstring>
#include <mutex>

#include "em_internal.h"
#include "emgb300.h"
#include "em_plan.h"

namespace em {

DevCtx *get_ctx(int *code)
{
    static DevCtx ctxs[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        *code = EM_ERR_NO_DEVICE;
        return nullptr;
    }
    DevCtx &c = ctxs[dev];
    std::lock_guard<std::mutex> g(c.init_mu);
    if (!c.ready) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
            cudaGetLastError();
            *code = EM_ERR_NO_DEVICE;
            return nullptr;
        }
        c.device = dev;
        c.nsm = prop.multiProcessorCount;
        c.smem_optin = prop.sharedMemPerBlockOptin;
        if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&c.ev0) != cudaSuccess || cudaEventCreate(&c.ev1) != cudaSuccess ||
            cudaEventCreateWithFlags(&c.ev_chunk, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            *code = EM_ERR_CUDA;
            return nullptr;
        }
        for (cudaEvent_t &ev : c.ev_rows)
            if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                *code = EM_ERR_CUDA;
                return nullptr;
            }
        c.ready = true;
    }
    *code = EM_OK;
    return &c;
}

// Host-side fault injection for tests: EM_INJECT_ALLOC_FAIL=<k> makes the
// k-th device allocation of the process fail (counting from 1).
static bool inject_alloc_failure()
{
    static long long target = [] {
        const char *v = std::getenv("EM_INJECT_ALLOC_FAIL");
        return v ? std::atoll(v) : 0LL;
    }();
    static std::atomic<long long> count{0};
    return target > 0 && ++count == target;
}

int grow(void **buf, size_t *cap, size_t need)
{
    if (need <= *cap && *buf)
        return EM_OK;
    if (inject_alloc_failure())
        return EM_ERR_NOMEM;
    if (*buf) {
        cudaFree(*buf);
        *buf = nullptr;
        *cap = 0;
    }
    const size_t want = std::max<size_t>(need, 256);
    if (cudaMalloc(buf, want) != cudaSuccess) {
        cudaGetLastError();
        *buf = nullptr;
        return EM_ERR_NOMEM;
    }
    *cap = want;
    return EM_OK;
}

int map_cuda(cudaError_t e)
{
    if (e == cudaSuccess)
        return EM_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? EM_ERR_NOMEM : EM_ERR_CUDA;
}

int read_dev_err(DevCtx &c, cudaStream_t s, int *dev_err_host)
{
    int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, c.err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return map_cuda(e);
    *dev_err_host = v;
    return v == EM_DEVERR_TIMEOUT ? EM_ERR_TIMEOUT : (v ? EM_ERR_CUDA : EM_OK);
}

namespace {

// Traces lines [line0, line0 + nl) of the caller's arrays (n lines per row;
// nl = n: all of them).  A partial range needs host arrays: its row-0 seeds
// go in as one contiguous slice and rows 1.. come back as a pitched copy.
template <class T>
int calc_field(T *x, T *y, T *z, size_t n, size_t total_steps, const T *charges, size_t p,
               T resolution, int use_curvature, const em_options *opt, bool plain,
               em_perf *perf, size_t line0 = 0, size_t nl = 0)
{
    using clock = std::chrono::steady_clock;
    const auto t_start = clock::now();
    // Reference order of checks: CPU_Implement.cpp:213-230.
    if (!n)
        return EM_ERR_N_ZERO;
    if (resolution == 0)
        return EM_ERR_RESOLUTION;
    const bool req64 = plain ? true : (opt && opt->require_n64);
    if (use_curvature && req64 && (n & 63))
        return EM_ERR_N_ALIGN;
    if (total_steps < 2)
        return EM_ERR_STEPS;
    if (!x || !y || !z || (p && !charges))
        return EM_ERR_ARG;
    em_options o{};
    if (opt)
        o = *opt;
    if (o.arith != EM_ARITH_FAST && o.arith != EM_ARITH_EXACT &&
        !(o.arith == EM_ARITH_MIXED && sizeof(T) == 4))
        return EM_ERR_ARG;
    if (o.rule != EM_RULE_SSE && o.rule != EM_RULE_GENERIC)
        return EM_ERR_ARG;
    if (!(o.null_frac >= 0) || !(o.refine_kappa >= 0))
        return EM_ERR_ARG;
    if (total_steps > (size_t)INT_MAX || p > (size_t)(INT_MAX / 64) ||
        n > (size_t)(LLONG_MAX / 64) / total_steps)
        return EM_ERR_TOO_LARGE;
    if (o.device_ptrs && ((uintptr_t)charges & 15))
        return EM_ERR_ARG;
    if (o.field_out && !o.device_ptrs)
        return EM_ERR_ARG;
    if (!nl)
        nl = n;
    if (line0 > n || nl > n - line0 || (nl != n && o.device_ptrs))
        return EM_ERR_ARG;
    if (perf)
        perf->progress = 0;

    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);

    Plan pl;
    code = make_plan<T>(c, nl, p, o, &pl);
    if (code)
        return code;
    const size_t rec = sizeof(T) * 4;
    cudaStream_t s = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;

    if ((code = grow(&c.charges, &c.charges_cap, (size_t)pl.p_pad * rec)))
        return code;
    if ((code = grow(&c.charges_raw, &c.charges_raw_cap, (size_t)p * rec + 16)))
        return code;
    if ((code = grow(&c.errbuf, &c.errbuf_cap, 256)))
        return code;
    c.err = static_cast<int *>(c.errbuf);

    T *dx = x, *dy = y, *dz = z;
    const size_t elems = nl * total_steps;
    if (!o.device_ptrs) {
        if ((code = grow(&c.lines, &c.lines_cap, 3 * elems * sizeof(T))))
            return code;
        dx = static_cast<T *>(c.lines);
        dy = dx + elems;
        dz = dy + elems;
    }
    cudaError_t e = cudaSuccess;
    const cudaMemcpyKind kin = o.device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (p)
        e = cudaMemcpyAsync(c.charges_raw, charges, p * rec, kin, s);
    if (e == cudaSuccess)
        e = launch_stage_charges<T>(c.charges_raw, (int)p, c.charges, pl.p_pad,
                                    stage_layout(pl.arith), pl.cfg.tile_recs, s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c.errbuf, 0, 64, s);
    // mixed: the count of re-evaluated vertices (status word at byte 32)
    unsigned long long *refines = reinterpret_cast<unsigned long long *>(
        static_cast<unsigned char *>(c.errbuf) + 32);
    if (e == cudaSuccess && !o.device_ptrs) {
        e = cudaMemcpyAsync(dx, x + line0, nl * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dy, y + line0, nl * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dz, z + line0, nl * sizeof(T), cudaMemcpyHostToDevice, s);
    }
    if (e != cudaSuccess)
        return map_cuda(e);

    RefTraceParams<T> prm{};
    prm.x = dx;
    prm.y = dy;
    prm.z = dz;
    prm.charges = c.charges;
    prm.n = (long long)nl;
    prm.n_groups = pl.n_groups;
    prm.total_steps = (int)total_steps;
    prm.p_pad = pl.p_pad;
    prm.n_tiles = pl.n_tiles;
    prm.tile_recs = pl.cfg.tile_recs;
    prm.stages = pl.cfg.stages;
    prm.resident = pl.cfg.resident;
    prm.rule = use_curvature ? o.rule : RULE_FIXED;
    prm.resolution = resolution;
    prm.err = c.err;
    const double kappa = mix_kappa(o);
    prm.kappa2 = kappa * kappa;
    prm.refines = refines;
    if (pl.arith == ARITH_EXACT && sizeof(T) == 4)
        prm.exact_nb = exact_nb_verified(s) ? 1 : 0;
    // the mixed form's groups come from a queue (status word at byte 40)
    if (pl.arith == ARITH_MIXED)
        prm.group_ctr = reinterpret_cast<unsigned long long *>(
            static_cast<unsigned char *>(c.errbuf) + 40);
    // field output: the mixed form stores its final field itself; the fast
    // and exact forms use their stored-field slot (the sum before the fast
    // form's Coulomb factor, which a small kernel applies afterwards)
    T *fout = static_cast<T *>(o.field_out);
    const size_t fcount = n * (total_steps - 1);
    if (fout && pl.arith == ARITH_MIXED) {
        prm.ox = fout;
        prm.oy = fout + fcount;
        prm.oz = fout + 2 * fcount;
    } else if (fout) {
        prm.fx = fout;
        prm.fy = fout + fcount;
        prm.fz = fout + 2 * fcount;
    }

    // Host arrays, all lines: trace in row chunks and copy each finished
    // chunk to the host on the copy stream while the next one is traced
    // (rows are contiguous blocks of n values; a chunk resumes from the last
    // row of the one before, so the result is the one-launch result; not in
    // the mixed form, whose FP64 position a stored FP32 row would round).
    const bool chunked = !o.device_ptrs && nl == n && elems * sizeof(T) * 3 >= (64u << 20) &&
                         total_steps >= 64 && pl.arith != ARITH_MIXED;
    const int nchunks = chunked ? 8 : 1;
    // first row of chunk k (chunk k holds rows [row_of(k), row_of(k + 1)))
    auto row_of = [&](int k) {
        return 1 + (int)(((long long)(total_steps - 1) * k) / nchunks);
    };
    auto launch_chunk = [&](int k) {
        const int r0 = row_of(k), r1 = row_of(k + 1);
        // rows [r0, r1) from row r0 - 1: the arrays seen from row r0 - 1
        RefTraceParams<T> q = prm;
        const size_t base = (size_t)(r0 - 1) * n;
        q.x = dx + base;
        q.y = dy + base;
        q.z = dz + base;
        q.seed_x = dx;
        q.seed_y = dy;
        q.seed_z = dz;
        q.total_steps = r1 - r0 + 1;
        cudaError_t le = launch_ref_trace<T>(q, pl.cfg, pl.arith, s);
        // the kernel time ends with the last chunk, before any copy waits
        if (le == cudaSuccess && k == nchunks - 1)
            le = cudaEventRecord(c.ev1, s);
        if (le == cudaSuccess && chunked)
            le = cudaEventRecord(c.ev_rows[k], s);
        return le;
    };
    e = cudaEventRecord(c.ev0, s);
    if (e == cudaSuccess)
        e = launch_chunk(0);
    for (int k = 0; k < nchunks && e == cudaSuccess; ++k) {
        // The copies of chunk k wait for chunk k alone, and chunk k + 1 is
        // queued before them: a copy into pageable host memory returns only
        // once it is done, and the next chunk then already runs beside it.
        if (chunked) {
            e = cudaEventRecord(c.ev_chunk, s);
            if (e == cudaSuccess)
                e = cudaStreamWaitEvent(c.copy_stream, c.ev_chunk, 0);
        }
        if (e == cudaSuccess && k + 1 < nchunks)
            e = launch_chunk(k + 1);
        if (e == cudaSuccess && chunked) {
            const size_t off = (size_t)row_of(k) * n;
            const size_t cnt = (size_t)(row_of(k + 1) - row_of(k)) * n;
            T *dst[3] = {x, y, z};
            const T *src[3] = {dx, dy, dz};
            for (int d = 0; d < 3 && e == cudaSuccess; ++d)
                e = cudaMemcpyAsync(dst[d] + off, src[d] + off, cnt * sizeof(T),
                                    cudaMemcpyDeviceToHost, c.copy_stream);
        }
    }
    if (e == cudaSuccess && chunked) {
        // the call's stream waits for the last copies, so it completes as one
        e = cudaEventRecord(c.ev_chunk, c.copy_stream);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(s, c.ev_chunk, 0);
    }
    if (e == cudaSuccess && fout && pl.arith != ARITH_MIXED && pl.arith != ARITH_EXACT)
        e = launch_scale_coulomb<T>(fout, 3 * fcount, s);
    if (e != cudaSuccess)
        return map_cuda(e);
    if (chunked) {
        // copies already enqueued
    } else if (!o.device_ptrs && nl == n) {
        const size_t rest = elems - n;
        e = cudaMemcpyAsync(x + n, dx + n, rest * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(y + n, dy + n, rest * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(z + n, dz + n, rest * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess)
            return map_cuda(e);
    } else if (!o.device_ptrs) {
        // rows 1.. of the range: nl values per row into a row pitch of n
        T *dst[3] = {x, y, z};
        const T *src[3] = {dx, dy, dz};
        for (int k = 0; k < 3 && e == cudaSuccess; ++k)
            e = cudaMemcpy2DAsync(dst[k] + n + line0, n * sizeof(T), src[k] + nl,
                                  nl * sizeof(T), nl * sizeof(T), total_steps - 1,
                                  cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess)
            return map_cuda(e);
    }
    // Progress while the chunks run, for a thread that polls perf->progress
    // as the reference's monitor does ("Electromag utils.h":133-156; the
    // reference adds each finished block's share, CPU_Implement.cpp:340-342):
    // the share of rows traced, raised as each chunk's trace completes.
    if (chunked && perf) {
        for (int k = 0; k + 1 < nchunks; ++k) {
            if (cudaEventSynchronize(c.ev_rows[k]) != cudaSuccess)
                break; // the stream's error is reported below
            perf->progress = (double)(row_of(k + 1) - 1) / (double)(total_steps - 1);
        }
    }
    int dev_err = 0;
    code = read_dev_err(c, s, &dev_err);
    if (code)
        return code;
    float ms = 0;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    unsigned long long nref = 0;
    if (perf && pl.arith == ARITH_MIXED &&
        cudaMemcpy(&nref, refines, sizeof(nref), cudaMemcpyDeviceToHost) != cudaSuccess)
        return map_cuda(cudaGetLastError());
    if (perf) {
        perf->fp64_refines = (double)nref;
        const double tk = ms * 1e-3;
        perf->time = tk;
        perf->pairs = (double)nl * (double)(total_steps - 1) * (double)p;
        perf->performance =
            tk > 0 ? (double)nl * (double)(total_steps - 1) * (18.0 * (double)p + 13.0) / tk / 1e9
                   : 0;
        perf->wall_time = std::chrono::duration<double>(clock::now() - t_start).count();
        perf->progress = 1.0;
    }
    return EM_OK;
}

template <class T>
int field_at(const T *px, const T *py, const T *pz, size_t m, const T *charges, size_t p,
             T *ex, T *ey, T *ez, const em_options *opt)
{
    if (!m)
        return EM_OK;
    if (!px || !py || !pz || !ex || !ey || !ez || (p && !charges))
        return EM_ERR_ARG;
    // one 256-thread block per 256 points: at most 2^31 - 1 blocks
    if (p > (size_t)INT_MAX / 4 || m > (size_t)INT_MAX * 256)
        return EM_ERR_TOO_LARGE;
    em_options o{};
    if (opt)
        o = *opt;
    if (o.arith != EM_ARITH_FAST && o.arith != EM_ARITH_EXACT)
        return EM_ERR_ARG;
    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);
    cudaStream_t s = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;
    const T *dpx = px, *dpy = py, *dpz = pz, *dch = charges;
    T *dex = ex, *dey = ey, *dez = ez;
    cudaError_t e = cudaSuccess;
    if (!o.device_ptrs) {
        if ((code = grow(&c.scratch, &c.scratch_cap, (6 * m + 4 * p + 64) * sizeof(T))))
            return code;
        T *b = static_cast<T *>(c.scratch);
        T *bpx = b, *bpy = b + m, *bpz = b + 2 * m, *bch = b + 3 * m;
        dex = bch + 4 * p + 32;
        dey = dex + m;
        dez = dey + m;
        e = cudaMemcpyAsync(bpx, px, m * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(bpy, py, m * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(bpz, pz, m * sizeof(T), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && p)
            e = cudaMemcpyAsync(bch, charges, 4 * p * sizeof(T), cudaMemcpyHostToDevice, s);
        dpx = bpx;
        dpy = bpy;
        dpz = bpz;
        dch = bch;
    }
    if (e == cudaSuccess)
        e = launch_field<T>(dpx, dpy, dpz, (long long)m, dch, (int)p, o.arith,
                            o.rule == EM_RULE_SSE, dex, dey, dez, s);
    if (e == cudaSuccess && !o.device_ptrs) {
        e = cudaMemcpyAsync(ex, dex, m * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ey, dey, m * sizeof(T), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ez, dez, m * sizeof(T), cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    return map_cuda(e);
}

} // namespace
} // namespace em

extern "C" {

int em_field_f32(const float *px, const float *py, const float *pz, size_t m,
                 const float *charges, size_t p, float *ex, float *ey, float *ez,
                 const em_options *opt)
{
    return em::field_at<float>(px, py, pz, m, charges, p, ex, ey, ez, opt);
}

int em_field_f64(const double *px, const double *py, const double *pz, size_t m,
                 const double *charges, size_t p, double *ex, double *ey, double *ez,
                 const em_options *opt)
{
    return em::field_at<double>(px, py, pz, m, charges, p, ex, ey, ez, opt);
}

} // extern "C"

namespace em {
namespace {

// Runs one line range on `device` from whichever host thread calls it; the
// caller's current device is restored afterwards.
template <class T>
int calc_field_part(int device, T *x, T *y, T *z, size_t n, size_t total_steps, size_t line0,
                    size_t nlines, const T *charges, size_t p, T resolution, int use_curvature,
                    const em_options *opt, em_perf *perf)
{
    if (!nlines)
        return EM_ERR_N_ZERO;
    if (opt && opt->device_ptrs)
        return EM_ERR_ARG;
    int ndev = 0, prev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    const int code = calc_field<T>(x, y, z, n, total_steps, charges, p, resolution,
                                   use_curvature, opt, false, perf, line0, nlines);
    cudaSetDevice(prev);
    return code;
}

} // namespace
} // namespace em

extern "C" {

int em_calc_field_part_f32(int device, float *x, float *y, float *z, size_t n,
                           size_t total_steps, size_t line0, size_t nlines,
                           const float *charges, size_t p, float resolution, int use_curvature,
                           const em_options *opt, em_perf *perf)
{
    return em::calc_field_part<float>(device, x, y, z, n, total_steps, line0, nlines, charges,
                                      p, resolution, use_curvature, opt, perf);
}

int em_calc_field_part_f64(int device, double *x, double *y, double *z, size_t n,
                           size_t total_steps, size_t line0, size_t nlines,
                           const double *charges, size_t p, double resolution,
                           int use_curvature, const em_options *opt, em_perf *perf)
{
    return em::calc_field_part<double>(device, x, y, z, n, total_steps, line0, nlines, charges,
                                       p, resolution, use_curvature, opt, perf);
}

int em_calc_field_f32(float *x, float *y, float *z, size_t n, size_t total_steps,
                      const float *charges, size_t p, float resolution, int use_curvature,
                      em_perf *perf)
{
    return em::calc_field<float>(x, y, z, n, total_steps, charges, p, resolution,
                                 use_curvature, nullptr, true, perf);
}

int em_calc_field_f64(double *x, double *y, double *z, size_t n, size_t total_steps,
                      const double *charges, size_t p, double resolution, int use_curvature,
                      em_perf *perf)
{
    return em::calc_field<double>(x, y, z, n, total_steps, charges, p, resolution,
                                  use_curvature, nullptr, true, perf);
}

int em_calc_field_ex_f32(float *x, float *y, float *z, size_t n, size_t total_steps,
                         const float *charges, size_t p, float resolution, int use_curvature,
                         const em_options *opt, em_perf *perf)
{
    return em::calc_field<float>(x, y, z, n, total_steps, charges, p, resolution,
                                 use_curvature, opt, false, perf);
}

int em_calc_field_ex_f64(double *x, double *y, double *z, size_t n, size_t total_steps,
                         const double *charges, size_t p, double resolution,
                         int use_curvature, const em_options *opt, em_perf *perf)
{
    return em::calc_field<double>(x, y, z, n, total_steps, charges, p, resolution,
                                  use_curvature, opt, false, perf);
}

int em_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int em_release_device(int device)
{
    int prev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return EM_ERR_NO_DEVICE;
    }
    const int code = em_release();
    cudaSetDevice(prev);
    return code;
}

int em_release(void)
{
    int code = EM_OK;
    em::DevCtx *c = em::get_ctx(&code);
    if (!c)
        return code;
    std::lock_guard<std::mutex> g(c->mu);
    for (auto pr : {std::make_pair(&c->charges, &c->charges_cap),
                    std::make_pair(&c->charges_raw, &c->charges_raw_cap),
                    std::make_pair(&c->lines, &c->lines_cap),
                    std::make_pair(&c->scratch, &c->scratch_cap),
                    std::make_pair(&c->adj, &c->adj_cap),
                    std::make_pair(&c->batch, &c->batch_cap),
                    std::make_pair(&c->tail, &c->tail_cap),
                    std::make_pair(&c->errbuf, &c->errbuf_cap)}) {
        if (*pr.first)
            cudaFree(*pr.first);
        *pr.first = nullptr;
        *pr.second = 0;
    }
    c->err = nullptr;
    return EM_OK;
}

const char *em_strerror(int code)
{
    switch (code) {
    case EM_OK: return "success";
    case EM_ERR_N_ZERO: return "n == 0";
    case EM_ERR_RESOLUTION: return "resolution == 0";
    case EM_ERR_STEPS: return "total_steps < 2";
    case EM_ERR_ARG: return "invalid argument";
    case EM_ERR_N_ALIGN: return "n is not a multiple of 64";
    case EM_ERR_CUDA: return "CUDA runtime error";
    case EM_ERR_NOMEM: return "device memory allocation failed";
    case EM_ERR_TIMEOUT: return "device-side wait timed out";
    case EM_ERR_NO_DEVICE: return "no usable CUDA device";
    case EM_ERR_TOO_LARGE: return "size beyond this entry point's limit";
    case EM_ERR_IO: return "file could not be opened or written";
    default: return "unknown error";
    }
}

const char *em_version(void) { return "0.1.0"; }

} // extern "C"
