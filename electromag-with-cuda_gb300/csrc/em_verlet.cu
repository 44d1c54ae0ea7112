// One velocity-Verlet step of moving point charges in the field of the
// static charges and of each other (emgVerletStep, ElectroMag/src/
// Particle_System.cpp:109-190, with BoundToBox :28-66 and emgFieldsAdd
// :72-102).  The reference never instantiates it (magneto_k is defined with
// a trailing semicolon, Magnetics.h:25, and Vector3 has no arithmetic
// operators) and drops the updated particle; this is the step it describes:
//
//   v' = v + a dt/2,  r' = r + v' dt
//   E  = K sum_static q r/|r|^3 + K sum_{j != i} q_j r/|r|^3   (r = r' - c_j)
//   B  = magneto_k sum_{j != i} q_j v_j x r/|r|^3
//   a'' = (q E + q v' x B) / m,  v'' = v' + a'' dt/2,  then reflection off
//   the box walls (position mirrored, velocity component negated)
//
// Every particle sees the others' start-of-step states, exactly as the
// reference's loop does (it reads dynCharges[j], which it never updates), so
// particles are independent: 1, 2 or 4 lanes per particle (enough to fill
// the SMs), charges and particles staged through shared memory in tiles (the
// all-pairs pattern of the field tracer).  The tile that holds a block's
// particles runs the loop that skips j = i; every other tile runs without
// the test.
#include <chrono>
#include <climits>
#include <cstdint>
#include <mutex>

#include "em_device.cuh"
#include "em_internal.h"
#include "em_math.cuh"
#include "em_plan.h"
#include "emgb300.h"

namespace em {
namespace {

constexpr double kMagnetoK = 1E-7; // magneto_k, include/Magnetics.h:25
constexpr int kVerletBlock = 128;

template <class T> struct alignas(sizeof(T) * 4) Dyn {
    T x, y, z, q, vx, vy, vz, m; // dynamicPointCharge<T> (Electrodynamics.h:29-34)
};
template <class T> struct alignas(sizeof(T) * 4) Q4 {
    T x, y, z, q; // pointCharge<T>
};

template <class T> __device__ __forceinline__ T inv_len3(T r2);
template <> __device__ __forceinline__ float inv_len3<float>(float r2)
{
    const float inv = rsqrt_fast(r2);
    return inv * inv * inv;
}
template <> __device__ __forceinline__ double inv_len3<double>(double r2)
{
    const double inv = 1.0 / sqrt(r2);
    return inv * inv * inv;
}

template <class T> struct VerletArgs {
    const Dyn<T> *in;
    Dyn<T> *out;
    T *accel;            // n * 3, a(t) in, a(t + dt) out
    const T *charges;    // p * 4 static
    long long n;
    int p;
    T lo[3], hi[3];
    T dt;
};

// Particles per thread: each source record read from shared memory feeds
// kParts pairs (one per particle the thread holds), a quarter of the shared
// loads per pair of one particle per thread (the first form, shared-memory
// bound at 982 Gpair/s; two particles 1154, four 1279 on 65 536 moving and
// 4096 static charges).  Each particle's sums run in the same order as with
// one particle per thread, so the bits do not depend on kParts.
constexpr int kParts = 4;
constexpr int kTile = 512; // records per shared-memory tile

// Pairs of the moving sources tile[0, count) with the kParts particles of
// this thread (lane t of TPP); in the tile that holds them (SELF), each
// particle skips its own record self[k].
template <class T, int TPP, bool SELF>
__device__ __forceinline__ void dyn_tile(const Dyn<T> *tile, int count, const int (&self)[kParts],
                                         int t, const T (&rx)[kParts], const T (&ry)[kParts],
                                         const T (&rz)[kParts], T (&ex)[kParts], T (&ey)[kParts],
                                         T (&ez)[kParts], T (&bx)[kParts], T (&by)[kParts],
                                         T (&bz)[kParts])
{
#pragma unroll 2
    for (int j = t; j < count; j += TPP) {
        const Dyn<T> d = tile[j];
#pragma unroll
        for (int k = 0; k < kParts; ++k) {
            if (SELF && j == self[k])
                continue;
            const T dx = rx[k] - d.x, dy = ry[k] - d.y, dz = rz[k] - d.z;
            const T r2 = fma(dz, dz, fma(dy, dy, dx * dx));
            const T w = d.q * inv_len3<T>(r2);
            ex[k] = fma(w, dx, ex[k]);
            ey[k] = fma(w, dy, ey[k]);
            ez[k] = fma(w, dz, ez[k]);
            // v_j x r
            const T cx = fma(d.vy, dz, -d.vz * dy);
            const T cy = fma(d.vz, dx, -d.vx * dz);
            const T cz = fma(d.vx, dy, -d.vy * dx);
            bx[k] = fma(w, cx, bx[k]);
            by[k] = fma(w, cy, by[k]);
            bz[k] = fma(w, cz, bz[k]);
        }
    }
}

template <int TPP, class T> __device__ __forceinline__ T lanes_sum(T v)
{
#pragma unroll
    for (int o = TPP / 2; o >= 1; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// TPP lanes share a particle and split its sums (j = t, t + TPP, ...), so a
// modest particle count still fills the SMs; a thread holds kParts
// particles (slot s of the block: particles s, s + S, s + 2S, ... with
// S = kVerletBlock/TPP), a block kParts S particles, all in one
// kTile-record tile.
template <class T, int TPP>
__global__ void __launch_bounds__(kVerletBlock) verlet_kernel(const VerletArgs<T> A)
{
    __shared__ Dyn<T> dtile[kTile];
    __shared__ Q4<T> stile[kTile];
    constexpr int S = kVerletBlock / TPP; // particle slots per block
    constexpr int PPB = kParts * S;       // particles per block
    static_assert(kTile % PPB == 0 && kTile % TPP == 0, "tile holds whole blocks");
    const int t = threadIdx.x % TPP;
    const int slot = threadIdx.x / TPP;
    const long long base = blockIdx.x * (long long)PPB;
    long long i[kParts];
    bool own[kParts];
    T q[kParts], mass[kParts];
    T rx[kParts], ry[kParts], rz[kParts], vx[kParts], vy[kParts], vz[kParts];
    const T dt2 = A.dt / T(2);
#pragma unroll
    for (int k = 0; k < kParts; ++k) {
        i[k] = base + slot + (long long)k * S;
        own[k] = i[k] < A.n;
        Dyn<T> me{};
        T ax = 0, ay = 0, az = 0;
        if (own[k]) {
            me = A.in[i[k]];
            ax = A.accel[3 * i[k]];
            ay = A.accel[3 * i[k] + 1];
            az = A.accel[3 * i[k] + 2];
        }
        q[k] = me.q;
        mass[k] = me.m;
        // v(t + dt/2) = v(t) + a(t) dt/2;  r(t + dt) = r(t) + v(t + dt/2) dt
        vx[k] = me.vx + ax * dt2;
        vy[k] = me.vy + ay * dt2;
        vz[k] = me.vz + az * dt2;
        rx[k] = me.x + vx[k] * A.dt;
        ry[k] = me.y + vy[k] * A.dt;
        rz[k] = me.z + vz[k] * A.dt;
    }

    T ex[kParts], ey[kParts], ez[kParts], bx[kParts], by[kParts], bz[kParts];
#pragma unroll
    for (int k = 0; k < kParts; ++k)
        ex[k] = ey[k] = ez[k] = bx[k] = by[k] = bz[k] = 0;
    for (int t0 = 0; t0 < A.p; t0 += kTile) {
        const int cnt = min(kTile, A.p - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kVerletBlock)
            stile[k] = reinterpret_cast<const Q4<T> *>(A.charges)[t0 + k];
        __syncthreads();
#pragma unroll 2
        for (int j = t; j < cnt; j += TPP) {
            const Q4<T> c = stile[j];
#pragma unroll
            for (int k = 0; k < kParts; ++k) {
                const T dx = rx[k] - c.x, dy = ry[k] - c.y, dz = rz[k] - c.z;
                const T r2 = fma(dz, dz, fma(dy, dy, dx * dx));
                const T w = c.q * inv_len3<T>(r2);
                ex[k] = fma(w, dx, ex[k]);
                ey[k] = fma(w, dy, ey[k]);
                ez[k] = fma(w, dz, ez[k]);
            }
        }
    }
    const long long mine = base / kTile * kTile; // the tile holding this block
    int self[kParts];
#pragma unroll
    for (int k = 0; k < kParts; ++k)
        self[k] = (int)(i[k] - mine);
    for (long long t0 = 0; t0 < A.n; t0 += kTile) {
        const int cnt = (int)min((long long)kTile, A.n - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kVerletBlock)
            dtile[k] = A.in[t0 + k];
        __syncthreads();
        if (t0 == mine)
            dyn_tile<T, TPP, true>(dtile, cnt, self, t, rx, ry, rz, ex, ey, ez, bx, by, bz);
        else
            dyn_tile<T, TPP, false>(dtile, cnt, self, t, rx, ry, rz, ex, ey, ez, bx, by, bz);
    }
    const T K = (T)kElectroK, MK = (T)kMagnetoK;
#pragma unroll
    for (int k = 0; k < kParts; ++k) {
        T Ex = lanes_sum<TPP>(ex[k]), Ey = lanes_sum<TPP>(ey[k]), Ez = lanes_sum<TPP>(ez[k]);
        T Bx = lanes_sum<TPP>(bx[k]), By = lanes_sum<TPP>(by[k]), Bz = lanes_sum<TPP>(bz[k]);
        if (!own[k] || t != 0)
            continue;
        Ex *= K;
        Ey *= K;
        Ez *= K;
        Bx *= MK;
        By *= MK;
        Bz *= MK;
        T vxk = vx[k], vyk = vy[k], vzk = vz[k];
        T rxk = rx[k], ryk = ry[k], rzk = rz[k];
        // a = (q E + q v x B) / m
        const T fx = q[k] * Ex + q[k] * (vyk * Bz - vzk * By);
        const T fy = q[k] * Ey + q[k] * (vzk * Bx - vxk * Bz);
        const T fz = q[k] * Ez + q[k] * (vxk * By - vyk * Bx);
        const T axk = fx / mass[k], ayk = fy / mass[k], azk = fz / mass[k];
        vxk += axk * dt2;
        vyk += ayk * dt2;
        vzk += azk * dt2;
        // BoundToBox (Particle_System.cpp:28-66): upper walls, then lower walls
        T *r[3] = {&rxk, &ryk, &rzk}, *v[3] = {&vxk, &vyk, &vzk};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (*r[c] > A.hi[c]) {
                *r[c] = T(2) * A.hi[c] - *r[c];
                *v[c] = -*v[c];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (*r[c] < A.lo[c]) {
                *r[c] = T(2) * A.lo[c] - *r[c];
                *v[c] = -*v[c];
            }
        }
        Dyn<T> o;
        o.q = q[k];
        o.m = mass[k];
        o.x = rxk;
        o.y = ryk;
        o.z = rzk;
        o.vx = vxk;
        o.vy = vyk;
        o.vz = vzk;
        A.out[i[k]] = o;
        A.accel[3 * i[k]] = axk;
        A.accel[3 * i[k] + 1] = ayk;
        A.accel[3 * i[k] + 2] = azk;
    }
}

template <class T>
int verlet(T *dyn, T *accel, size_t n, const T *charges, size_t p, const T *box_min,
           const T *box_max, T dt, size_t steps, const em_options *opt, em_perf *perf)
{
    using clock = std::chrono::steady_clock;
    const auto t_start = clock::now();
    if (!n)
        return 1; // emgVerletStep's only check
    if (!dyn || !accel || (p && !charges) || !box_min || !box_max || !steps)
        return EM_ERR_ARG;
    if (n > (size_t)(LLONG_MAX / 64) || p > (size_t)INT_MAX / 4)
        return EM_ERR_TOO_LARGE;
    em_options o{};
    if (opt)
        o = *opt;
    if (o.device_ptrs && (((uintptr_t)dyn % alignof(Dyn<T>)) ||
                          ((uintptr_t)charges % alignof(Q4<T>)) ||
                          ((uintptr_t)accel % sizeof(T))))
        return EM_ERR_ARG;
    int code = EM_OK;
    DevCtx *cp = get_ctx(&code);
    if (!cp)
        return code;
    DevCtx &c = *cp;
    std::lock_guard<std::mutex> guard(c.mu);
    cudaStream_t s = (o.device_ptrs && o.stream) ? (cudaStream_t)o.stream : c.stream;
    const size_t dbytes = n * sizeof(Dyn<T>), abytes = n * 3 * sizeof(T);
    const size_t cbytes = p * 4 * sizeof(T);
    // scratch: two particle buffers (ping-pong); host calls also stage the
    // accelerations and the charges
    const size_t off_acc = 2 * ((dbytes + 255) / 256 * 256);
    const size_t off_ch = off_acc + (abytes + 255) / 256 * 256;
    if ((code = grow(&c.scratch, &c.scratch_cap, off_ch + cbytes + 256)))
        return code;
    unsigned char *ws = static_cast<unsigned char *>(c.scratch);
    Dyn<T> *buf[2] = {reinterpret_cast<Dyn<T> *>(ws),
                      reinterpret_cast<Dyn<T> *>(ws + off_acc / 2)};
    T *dacc = accel;
    const T *dch = charges;
    cudaError_t e = cudaSuccess;
    const cudaMemcpyKind kin = o.device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    e = cudaMemcpyAsync(buf[0], dyn, dbytes, kin, s);
    if (!o.device_ptrs) {
        dacc = reinterpret_cast<T *>(ws + off_acc);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(dacc, accel, abytes, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess && p) {
            T *hc = reinterpret_cast<T *>(ws + off_ch);
            e = cudaMemcpyAsync(hc, charges, cbytes, cudaMemcpyHostToDevice, s);
            dch = hc;
        }
    }
    VerletArgs<T> A{};
    A.accel = dacc;
    A.charges = dch;
    A.n = (long long)n;
    A.p = (int)p;
    for (int k = 0; k < 3; ++k) {
        A.lo[k] = box_min[k];
        A.hi[k] = box_max[k];
    }
    A.dt = dt;
    // lanes per particle: the caller's (opt->threads_per_line), else the
    // fewest that give about 24 warps per SM (kParts particles per thread)
    const size_t want = (size_t)c.nsm * 24 * 32;
    int tpp = 8;
    for (int cand = 1; cand <= 4; cand *= 2)
        if (n * cand / kParts >= want) {
            tpp = cand;
            break;
        }
    if (o.threads_per_line)
        tpp = o.threads_per_line;
    if (tpp != 1 && tpp != 2 && tpp != 4 && tpp != 8)
        return EM_ERR_ARG;
    const size_t ppb = (size_t)kParts * kVerletBlock / tpp; // particles per block
    const unsigned grid = (unsigned)((n + ppb - 1) / ppb);
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev0, s);
    for (size_t k = 0; k < steps && e == cudaSuccess; ++k) {
        A.in = buf[k & 1];
        A.out = buf[(k + 1) & 1];
        if (tpp == 8)
            verlet_kernel<T, 8><<<grid, kVerletBlock, 0, s>>>(A);
        else if (tpp == 4)
            verlet_kernel<T, 4><<<grid, kVerletBlock, 0, s>>>(A);
        else if (tpp == 2)
            verlet_kernel<T, 2><<<grid, kVerletBlock, 0, s>>>(A);
        else
            verlet_kernel<T, 1><<<grid, kVerletBlock, 0, s>>>(A);
        count_launch(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(c.ev1, s);
    const cudaMemcpyKind kout = o.device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dyn, buf[steps & 1], dbytes, kout, s);
    if (e == cudaSuccess && !o.device_ptrs)
        e = cudaMemcpyAsync(accel, dacc, abytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess)
        return map_cuda(e);
    if (perf) {
        float ms = 0;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        perf->time = ms * 1e-3;
        perf->pairs = (double)steps * (double)n * ((double)p + (double)n - 1.0);
        perf->performance = 0;
        perf->wall_time = std::chrono::duration<double>(clock::now() - t_start).count();
        perf->progress = 1.0;
    }
    return EM_OK;
}

} // namespace
} // namespace em

extern "C" {

int em_verlet_step_f32(float *dyn, float *accel, size_t n, const float *charges, size_t p,
                       const float *box_min, const float *box_max, float dt, size_t steps,
                       const em_options *opt, em_perf *perf)
{
    return em::verlet<float>(dyn, accel, n, charges, p, box_min, box_max, dt, steps, opt, perf);
}

int em_verlet_step_f64(double *dyn, double *accel, size_t n, const double *charges, size_t p,
                       const double *box_min, const double *box_max, double dt, size_t steps,
                       const em_options *opt, em_perf *perf)
{
    return em::verlet<double>(dyn, accel, n, charges, p, box_min, box_max, dt, steps, opt,
                              perf);
}

} // extern "C"
