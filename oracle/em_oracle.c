/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * Portable-C restatement of the ElectroMag field-line tracer (reference:
 * ElectroMag/src/CPU_Implement.cpp, include/Electrostatics.h,
 * include/Vector.h).  The oracle: used only by the tests, by the smoke
 * check and as bench.py's CPU baseline.  Compile with -ffp-contract=off and
 * without -ffast-math: the operation sequence below is the reference's, one
 * IEEE-754 rounding per operation, so that the results are bit-identical to
 * the reference's SSE build (checked against tests/golden/).
 *
 * Lines are processed in blocks of 16 (the SSE path's LINES_WIDTH,
 * CPU_Implement.cpp:200-204).  The innermost loops run across the lines of a
 * block, which lets the compiler use SIMD lanes without reordering any
 * per-line arithmetic.
 */
#include "em_oracle.h"

#include <math.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* include/Electrostatics.h:27 */
#define ORC_ELECTRO_K 8.987551787E9

#define OB 16

#ifdef _OPENMP
static void orc_set_threads(int nthreads)
{
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
}
#else
static void orc_set_threads(int nthreads) { (void)nthreads; }
#endif

static int orc_validate(size_t n, double resolution, size_t total_steps,
                        int variant)
{
    /* CPU_Implement.cpp:213-230 (SSE float), :372-388 (SSE2 double),
     * :110-127 (generic), :43-52 (fixed step). */
    if (!n)
        return 1;
    if (resolution == 0)
        return 2;
    if (variant == ORC_CURV_SSE && (n & 63))
        return 5;
    if (total_steps < 2)
        return 3;
    return 0;
}

/* The same body is instantiated for float and double. */
#define ORC_DEFINE_CALC(SUFFIX, T, SQRT)                                       \
    int orc_calc_field_##SUFFIX(T *x, T *y, T *z, size_t n,                    \
                                size_t total_steps, const T *charges,          \
                                size_t p, T resolution, int variant,           \
                                size_t line0, size_t nlines, int nthreads)     \
    {                                                                          \
        int rc = orc_validate(n, (double)resolution, total_steps, variant);    \
        if (rc)                                                                \
            return rc;                                                         \
        if (variant < ORC_CURV_SSE || variant > ORC_FIXED)                     \
            return 4;                                                          \
        if (nlines == 0)                                                       \
            nlines = n;                                                        \
        if (line0 >= n || nlines > n - line0)                                  \
            return 4;                                                          \
        orc_set_threads(nthreads);                                             \
        const T K = (T)ORC_ELECTRO_K;                                          \
        const long nblocks = (long)((nlines + OB - 1) / OB);                   \
        _Pragma("omp parallel for schedule(dynamic, 1)")                       \
        for (long b = 0; b < nblocks; ++b) {                                   \
            const size_t first = line0 + (size_t)b * OB;                       \
            const size_t end = line0 + nlines;                                 \
            const int cnt = (int)((end - first) < OB ? (end - first) : OB);    \
            T px[OB], py[OB], pz[OB]; /* current point */                     \
            T rx0[OB], ry0[OB], rz0[OB]; /* curvature reference vector */     \
            T ax[OB], ay[OB], az[OB];                                          \
            for (int i = 0; i < OB; ++i) {                                     \
                const size_t l = first + (size_t)(i < cnt ? i : 0);            \
                px[i] = rx0[i] = x[l];                                         \
                py[i] = ry0[i] = y[l];                                         \
                pz[i] = rz0[i] = z[l];                                         \
            }                                                                  \
            for (size_t step = 1; step < total_steps; ++step) {                \
                if (variant == ORC_CURV_GENERIC) {                             \
                    /* prevVec = previous point, CPU_Implement.cpp:148-153 */  \
                    for (int i = 0; i < OB; ++i) {                             \
                        rx0[i] = px[i];                                        \
                        ry0[i] = py[i];                                        \
                        rz0[i] = pz[i];                                        \
                    }                                                          \
                }                                                              \
                for (int i = 0; i < OB; ++i)                                   \
                    ax[i] = ay[i] = az[i] = 0;                                 \
                for (size_t j = 0; j < p; ++j) {                               \
                    const T cx = charges[4 * j + 0];                           \
                    const T cy = charges[4 * j + 1];                           \
                    const T cz = charges[4 * j + 2];                           \
                    const T q = charges[4 * j + 3];                            \
                    if (variant == ORC_CURV_SSE) {                             \
                        /* PartField(charge, point, k):                        \
                         * r*k*q / (r2*sqrt(r2)), Electrostatics.h:38-51 */    \
                        for (int i = 0; i < OB; ++i) {                         \
                            const T rx = px[i] - cx;                           \
                            const T ry = py[i] - cy;                           \
                            const T rz = pz[i] - cz;                           \
                            T l2 = rx * rx;                                    \
                            l2 = l2 + ry * ry;                                 \
                            l2 = l2 + rz * rz;                                 \
                            const T d = l2 * SQRT(l2);                         \
                            ax[i] += ((rx * K) * q) / d;                       \
                            ay[i] += ((ry * K) * q) / d;                       \
                            az[i] += ((rz * K) * q) / d;                       \
                        }                                                      \
                    } else {                                                   \
                        /* PartField(charge, point): r * (k*q/(r2*sqrt(r2))),  \
                         * Electrostatics.h:53-60 */                           \
                        const T kq = K * q;                                    \
                        for (int i = 0; i < OB; ++i) {                         \
                            const T rx = px[i] - cx;                           \
                            const T ry = py[i] - cy;                           \
                            const T rz = pz[i] - cz;                           \
                            T l2 = rx * rx;                                    \
                            l2 = l2 + ry * ry;                                 \
                            l2 = l2 + rz * rz;                                 \
                            const T s = kq / (l2 * SQRT(l2));                  \
                            ax[i] += rx * s;                                   \
                            ay[i] += ry * s;                                   \
                            az[i] += rz * s;                                   \
                        }                                                      \
                    }                                                          \
                }                                                              \
                for (int i = 0; i < OB; ++i) {                                 \
                    T scale;                                                   \
                    if (variant == ORC_FIXED) {                                \
                        scale = resolution; /* CPU_Implement.cpp:89-90 */      \
                    } else {                                                   \
                        /* k = |(E - P0) x P0| / (|E|^2 sqrt|E|^2),            \
                         * CPU_Implement.cpp:327-329 / :163-165 */             \
                        T k2 = ax[i] * ax[i];                                  \
                        k2 = k2 + ay[i] * ay[i];                               \
                        k2 = k2 + az[i] * az[i];                               \
                        const T ix = ax[i] - rx0[i];                           \
                        const T iy = ay[i] - ry0[i];                           \
                        const T iz = az[i] - rz0[i];                           \
                        const T cx = iy * rz0[i] - iz * ry0[i];                \
                        const T cy = iz * rx0[i] - ix * rz0[i];                \
                        const T cz = ix * ry0[i] - iy * rx0[i];                \
                        T c2 = cx * cx;                                        \
                        c2 = c2 + cy * cy;                                     \
                        c2 = c2 + cz * cz;                                     \
                        const T kc = SQRT(c2) / (k2 * SQRT(k2));               \
                        scale = (kc + (T)1) * resolution;                      \
                    }                                                          \
                    /* vec3SetInvLen, include/Vector.h:157-164 */              \
                    T e2 = ax[i] * ax[i];                                      \
                    e2 = e2 + ay[i] * ay[i];                                   \
                    e2 = e2 + az[i] * az[i];                                   \
                    const T s = scale * SQRT(e2);                              \
                    px[i] = px[i] + ax[i] / s;                                 \
                    py[i] = py[i] + ay[i] / s;                                 \
                    pz[i] = pz[i] + az[i] / s;                                 \
                }                                                              \
                const size_t row = n * step;                                   \
                for (int i = 0; i < cnt; ++i) {                                \
                    x[row + first + (size_t)i] = px[i];                        \
                    y[row + first + (size_t)i] = py[i];                        \
                    z[row + first + (size_t)i] = pz[i];                        \
                }                                                              \
            }                                                                  \
        }                                                                      \
        return 0;                                                              \
    }

ORC_DEFINE_CALC(f32, float, sqrtf)
ORC_DEFINE_CALC(f64, double, sqrt)

void orc_field_f32(const float *px, const float *py, const float *pz, size_t m,
                   const float *charges, size_t p, int three_arg, float *ex,
                   float *ey, float *ez)
{
    const float K = (float)ORC_ELECTRO_K;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)m; ++i) {
        float ax = 0, ay = 0, az = 0;
        for (size_t j = 0; j < p; ++j) {
            const float rx = px[i] - charges[4 * j + 0];
            const float ry = py[i] - charges[4 * j + 1];
            const float rz = pz[i] - charges[4 * j + 2];
            const float q = charges[4 * j + 3];
            float l2 = rx * rx;
            l2 = l2 + ry * ry;
            l2 = l2 + rz * rz;
            const float d = l2 * sqrtf(l2);
            if (three_arg) {
                ax += ((rx * K) * q) / d;
                ay += ((ry * K) * q) / d;
                az += ((rz * K) * q) / d;
            } else {
                const float s = (K * q) / d;
                ax += rx * s;
                ay += ry * s;
                az += rz * s;
            }
        }
        ex[i] = ax;
        ey[i] = ay;
        ez[i] = az;
    }
}

void orc_field_f64(const double *px, const double *py, const double *pz,
                   size_t m, const double *charges, size_t p, double *ex,
                   double *ey, double *ez, double *maxc, int nthreads)
{
    orc_set_threads(nthreads);
    const double K = ORC_ELECTRO_K;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)m; ++i) {
        double ax = 0, ay = 0, az = 0, mc = 0;
        for (size_t j = 0; j < p; ++j) {
            const double rx = px[i] - charges[4 * j + 0];
            const double ry = py[i] - charges[4 * j + 1];
            const double rz = pz[i] - charges[4 * j + 2];
            const double q = charges[4 * j + 3];
            double l2 = rx * rx;
            l2 = l2 + ry * ry;
            l2 = l2 + rz * rz;
            const double d = l2 * sqrt(l2);
            ax += ((rx * K) * q) / d;
            ay += ((ry * K) * q) / d;
            az += ((rz * K) * q) / d;
            const double c = fabs(K * q) / l2;
            if (c > mc)
                mc = c;
        }
        ex[i] = ax;
        ey[i] = ay;
        ez[i] = az;
        if (maxc)
            maxc[i] = mc;
    }
}

int orc_trace_lines_f64(const double *charges, size_t p, double *x, double *y,
                        double *z, size_t n, size_t max_steps,
                        const int32_t *max_steps_per_line, double resolution,
                        double term_radius, int32_t *len, int32_t *cls,
                        int nthreads)
{
    if (!n)
        return 1;
    if (resolution == 0)
        return 2;
    if (max_steps < 1)
        return 3;
    orc_set_threads(nthreads);
    const double K = ORC_ELECTRO_K;
    const double r2term = term_radius * term_radius;
#pragma omp parallel for schedule(dynamic, 4)
    for (long l = 0; l < (long)n; ++l) {
        size_t lim = max_steps;
        if (max_steps_per_line) {
            const int32_t v = max_steps_per_line[l];
            lim = v < 1 ? 1 : ((size_t)v < max_steps ? (size_t)v : max_steps);
        }
        double px = x[l], py = y[l], pz = z[l];
        const double p0x = px, p0y = py, p0z = pz;
        int32_t c = ORC_TERM_STEPS;
        size_t s;
        for (s = 1; s < lim; ++s) {
            double ax = 0, ay = 0, az = 0, dmin = INFINITY;
            for (size_t j = 0; j < p; ++j) {
                const double rx = px - charges[4 * j + 0];
                const double ry = py - charges[4 * j + 1];
                const double rz = pz - charges[4 * j + 2];
                const double q = charges[4 * j + 3];
                double l2 = rx * rx;
                l2 = l2 + ry * ry;
                l2 = l2 + rz * rz;
                const double d = l2 * sqrt(l2);
                ax += ((rx * K) * q) / d;
                ay += ((ry * K) * q) / d;
                az += ((rz * K) * q) / d;
                if (q < 0 && l2 < dmin)
                    dmin = l2;
            }
            if (dmin < r2term) {
                c = ORC_TERM_CHARGE;
                break;
            }
            double k2 = ax * ax;
            k2 = k2 + ay * ay;
            k2 = k2 + az * az;
            const double ix = ax - p0x, iy = ay - p0y, iz = az - p0z;
            const double cx = iy * p0z - iz * p0y;
            const double cy = iz * p0x - ix * p0z;
            const double cz = ix * p0y - iy * p0x;
            double c2 = cx * cx;
            c2 = c2 + cy * cy;
            c2 = c2 + cz * cz;
            const double kc = sqrt(c2) / (k2 * sqrt(k2));
            const double sc = ((kc + 1.0) * resolution) * sqrt(k2);
            const double nx = px + ax / sc, ny = py + ay / sc,
                         nz = pz + az / sc;
            if (!(k2 > 0) || !isfinite(nx) || !isfinite(ny) || !isfinite(nz)) {
                c = ORC_TERM_NULL;
                break;
            }
            px = nx;
            py = ny;
            pz = nz;
            x[s * n + (size_t)l] = px;
            y[s * n + (size_t)l] = py;
            z[s * n + (size_t)l] = pz;
        }
        len[l] = (int32_t)s;
        cls[l] = c;
    }
    return 0;
}

size_t orc_seed_fibonacci_f64(const double *charges, size_t p,
                              size_t lines_per_charge, double radius,
                              double *sx, double *sy, double *sz, size_t cap)
{
    const double ga = M_PI * (3.0 - sqrt(5.0)); /* golden angle */
    size_t w = 0;
    for (size_t j = 0; j < p; ++j) {
        if (!(charges[4 * j + 3] > 0))
            continue;
        for (size_t i = 0; i < lines_per_charge; ++i) {
            if (w >= cap)
                return w;
            const double zz = 1.0 - (2.0 * (double)i + 1.0) /
                                        (double)lines_per_charge;
            const double rr = sqrt(1.0 - zz * zz);
            const double ph = ga * (double)i;
            sx[w] = charges[4 * j + 0] + radius * rr * cos(ph);
            sy[w] = charges[4 * j + 1] + radius * rr * sin(ph);
            sz[w] = charges[4 * j + 2] + radius * zz;
            ++w;
        }
    }
    return w;
}

/* ---------------------------------------------------------------------------
 * Adjoint checks: the frozen-step map, its complex-step derivative and its
 * discrete adjoint, all in FP64 (test infrastructure).
 */
#include <complex.h>
#include <stdlib.h>

/* E' = sum_j q_j r / |r|^3 (the Coulomb constant factored out). */
static void field_prime(const double *ch, size_t p, double x, double y,
                        double z, double *e)
{
    double ax = 0, ay = 0, az = 0;
    for (size_t j = 0; j < p; ++j) {
        const double rx = x - ch[4 * j], ry = y - ch[4 * j + 1],
                     rz = z - ch[4 * j + 2], q = ch[4 * j + 3];
        const double r2 = rx * rx + ry * ry + rz * rz;
        const double s = q / (r2 * sqrt(r2));
        ax += s * rx;
        ay += s * ry;
        az += s * rz;
    }
    e[0] = ax;
    e[1] = ay;
    e[2] = az;
}

/* lam = 1/((k+1) res) with k = |(E - P0) x P0| / |E|^3, E = K E'. */
static double frozen_lambda(const double *ep, const double *p0, double res)
{
    const double K = ORC_ELECTRO_K;
    const double ex = K * ep[0], ey = K * ep[1], ez = K * ep[2];
    const double k2 = ex * ex + ey * ey + ez * ez;
    const double ix = ex - p0[0], iy = ey - p0[1], iz = ez - p0[2];
    const double cx = iy * p0[2] - iz * p0[1], cy = iz * p0[0] - ix * p0[2],
                 cz = ix * p0[1] - iy * p0[0];
    const double kc = sqrt(cx * cx + cy * cy + cz * cz) / (k2 * sqrt(k2));
    return 1.0 / ((kc + 1.0) * res);
}

/* lam as the FP32 trace steps: the reference's single-precision sequence
 * (CPU_Implement.cpp:322-331) from E = K E' rounded to FP32 (the field an
 * FP32 forward stepped with), curvature against the FP32 seed; each
 * operation rounded once (the oracle is built without contraction). */
static double frozen_lambda_f32(const double *ep, const double *p0, double res)
{
    const double K = ORC_ELECTRO_K;
    const float ex = (float)(K * ep[0]), ey = (float)(K * ep[1]), ez = (float)(K * ep[2]);
    const float px = (float)p0[0], py = (float)p0[1], pz = (float)p0[2];
    float k2 = ex * ex;
    k2 = k2 + ey * ey;
    k2 = k2 + ez * ez;
    const float ix = ex - px, iy = ey - py, iz = ez - pz;
    const float cx = iy * pz - iz * py, cy = iz * px - ix * pz, cz = ix * py - iy * px;
    float c2 = cx * cx;
    c2 = c2 + cy * cy;
    c2 = c2 + cz * cz;
    const float kc = sqrtf(c2) / (k2 * sqrtf(k2));
    return (double)(1.0f / ((kc + 1.0f) * (float)res));
}

double orc_frozen_loss_f64(const double *charges, size_t p, const double *sx,
                           const double *sy, const double *sz, size_t n,
                           size_t S, double res, const double *tx,
                           const double *ty, const double *tz,
                           const double *lam_in, double *lam_out, double *vx,
                           double *vy, double *vz)
{
    double L = 0;
    for (size_t l = 0; l < n; ++l) {
        double v[3] = {sx[l], sy[l], sz[l]};
        const double p0[3] = {sx[l], sy[l], sz[l]};
        for (size_t s = 0; s < S; ++s) {
            const size_t i = s * n + l;
            const double dx = v[0] - tx[i], dy = v[1] - ty[i], dz = v[2] - tz[i];
            L += dx * dx + dy * dy + dz * dz;
            if (vx) {
                vx[i] = v[0];
                vy[i] = v[1];
                vz[i] = v[2];
            }
            if (s + 1 == S)
                break;
            double e[3];
            field_prime(charges, p, v[0], v[1], v[2], e);
            const double lam = lam_in ? lam_in[i] : frozen_lambda(e, p0, res);
            if (lam_out)
                lam_out[i] = lam;
            const double en = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            for (int c = 0; c < 3; ++c)
                v[c] += lam * e[c] / en;
        }
    }
    return L;
}

double orc_frozen_loss_cs_f64(const double *charges, size_t p, const double *sx,
                              const double *sy, const double *sz, size_t n,
                              size_t S, double res, const double *tx,
                              const double *ty, const double *tz,
                              const double *lam_in, size_t j, int c, double h)
{
    (void)res;
    double complex *ch = malloc(sizeof(double complex) * 4 * p);
    for (size_t k = 0; k < 4 * p; ++k)
        ch[k] = charges[k];
    ch[4 * j + (size_t)c] += I * h;
    double complex L = 0;
    for (size_t l = 0; l < n; ++l) {
        double complex v[3] = {sx[l], sy[l], sz[l]};
        for (size_t s = 0; s < S; ++s) {
            const size_t i = s * n + l;
            const double complex dx = v[0] - tx[i], dy = v[1] - ty[i],
                                 dz = v[2] - tz[i];
            L += dx * dx + dy * dy + dz * dz;
            if (s + 1 == S)
                break;
            double complex e[3] = {0, 0, 0};
            for (size_t k = 0; k < p; ++k) {
                const double complex rx = v[0] - ch[4 * k], ry = v[1] - ch[4 * k + 1],
                                     rz = v[2] - ch[4 * k + 2];
                const double complex r2 = rx * rx + ry * ry + rz * rz;
                const double complex sc = ch[4 * k + 3] / (r2 * csqrt(r2));
                e[0] += sc * rx;
                e[1] += sc * ry;
                e[2] += sc * rz;
            }
            const double complex en = csqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            for (int d = 0; d < 3; ++d)
                v[d] += lam_in[i] * e[d] / en;
        }
    }
    free(ch);
    return cimag(L) / h;
}

/* Backward sweep of the frozen map along the trajectory vx, vy, vz (S rows
 * of n lines): the discrete adjoint of CPU_Implement.cpp:322-338's step with
 * lam_s from lam_in, or, when lam_in is NULL, from the curvature of the
 * field at the given vertex against the line's row-0 vertex (curvature 0:
 * lam_s = 1/res).  Adds dL/d(charges) into grad. */
static void adjoint_sweep(const double *charges, size_t p, const double *vx,
                          const double *vy, const double *vz, size_t n, size_t S,
                          double res, int curvature, const double *tx,
                          const double *ty, const double *tz, const double *lam_in,
                          const double *const *fe, int lam_fp32, double *grad)
{
    for (size_t l = 0; l < n; ++l) {
        const size_t last = (S - 1) * n + l;
        const double p0[3] = {vx[l], vy[l], vz[l]};
        double a[3] = {2 * (vx[last] - tx[last]), 2 * (vy[last] - ty[last]),
                       2 * (vz[last] - tz[last])};
        for (size_t s = S - 1; s-- > 0;) {
            const size_t i = s * n + l;
            const double v[3] = {vx[i], vy[i], vz[i]};
            double e[3];
            if (fe) {
                e[0] = fe[0][i];
                e[1] = fe[1][i];
                e[2] = fe[2][i];
            } else {
                field_prime(charges, p, v[0], v[1], v[2], e);
            }
            const double lam = lam_in     ? lam_in[i]
                               : !curvature ? 1.0 / res
                               : lam_fp32   ? frozen_lambda_f32(e, p0, res)
                                            : frozen_lambda(e, p0, res);
            const double en = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
            const double u[3] = {e[0] / en, e[1] / en, e[2] / en};
            const double ua = u[0] * a[0] + u[1] * a[1] + u[2] * a[2];
            double mu[3];
            for (int c = 0; c < 3; ++c)
                mu[c] = lam * (a[c] - u[c] * ua) / en;
            double jm[3] = {0, 0, 0};
            for (size_t j = 0; j < p; ++j) {
                const double r[3] = {v[0] - charges[4 * j], v[1] - charges[4 * j + 1],
                                     v[2] - charges[4 * j + 2]};
                const double q = charges[4 * j + 3];
                const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
                const double i3 = 1.0 / (r2 * sqrt(r2));
                const double d = r[0] * mu[0] + r[1] * mu[1] + r[2] * mu[2];
                for (int c = 0; c < 3; ++c) {
                    const double g = mu[c] * i3 - 3.0 * r[c] * d * i3 / r2;
                    jm[c] += q * g;
                    grad[4 * j + (size_t)c] -= q * g;
                }
                grad[4 * j + 3] += d * i3;
            }
            for (int c = 0; c < 3; ++c)
                a[c] = 2 * (v[c] - (c == 0 ? tx[i] : c == 1 ? ty[i] : tz[i])) + a[c] + jm[c];
        }
    }
}

double orc_frozen_grad_f64(const double *charges, size_t p, const double *sx,
                           const double *sy, const double *sz, size_t n,
                           size_t S, double res, const double *tx,
                           const double *ty, const double *tz,
                           const double *lam_in, double *grad)
{
    double *vx = malloc(sizeof(double) * S * n), *vy = malloc(sizeof(double) * S * n),
           *vz = malloc(sizeof(double) * S * n);
    const double L = orc_frozen_loss_f64(charges, p, sx, sy, sz, n, S, res, tx, ty,
                                         tz, lam_in, NULL, vx, vy, vz);
    for (size_t k = 0; k < 4 * p; ++k)
        grad[k] = 0;
    adjoint_sweep(charges, p, vx, vy, vz, n, S, res, 1, tx, ty, tz, lam_in, NULL, 0, grad);
    free(vx);
    free(vy);
    free(vz);
    return L;
}

double orc_adjoint_at_f64(const double *charges, size_t p, const double *vx,
                          const double *vy, const double *vz, size_t n, size_t S,
                          double res, int curvature, const double *tx,
                          const double *ty, const double *tz, double *grad)
{
    double L = 0;
    for (size_t i = 0; i < S * n; ++i) {
        const double dx = vx[i] - tx[i], dy = vy[i] - ty[i], dz = vz[i] - tz[i];
        L += dx * dx + dy * dy + dz * dz;
    }
    for (size_t k = 0; k < 4 * p; ++k)
        grad[k] = 0;
    adjoint_sweep(charges, p, vx, vy, vz, n, S, res, curvature, tx, ty, tz, NULL, NULL, 0,
                  grad);
    return L;
}

double orc_adjoint_at_field_f64(const double *charges, size_t p, const double *vx,
                                const double *vy, const double *vz, size_t n, size_t S,
                                double res, int curvature, const double *tx,
                                const double *ty, const double *tz, const double *fx,
                                const double *fy, const double *fz, int lam_fp32,
                                double *grad)
{
    double L = 0;
    for (size_t i = 0; i < S * n; ++i) {
        const double dx = vx[i] - tx[i], dy = vy[i] - ty[i], dz = vz[i] - tz[i];
        L += dx * dx + dy * dy + dz * dz;
    }
    for (size_t k = 0; k < 4 * p; ++k)
        grad[k] = 0;
    const double *fe[3] = {fx, fy, fz};
    adjoint_sweep(charges, p, vx, vy, vz, n, S, res, curvature, tx, ty, tz, NULL, fe, lam_fp32,
                  grad);
    return L;
}
