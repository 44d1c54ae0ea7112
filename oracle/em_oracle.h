/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * CPU oracle for the ElectroMag field-line tracer.  Only the tests, the smoke
 * check and bench.py's CPU-baseline leg call into liboracle.so; the CUDA
 * library never links or loads it.
 *
 * Every function restates the reference algorithm in portable C (no SIMD
 * intrinsics, no FMA contraction, no fast-math), so that its results are the
 * IEEE-754 results of the reference's own operation sequence.  The restatement
 * is pinned bit-for-bit against the reference compiled here from its own
 * sources (oracle/build_ref.sh -> oracle/_ref/, fixtures in tests/golden/).
 */
#ifndef EM_ORACLE_H
#define EM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Stepping variants of the reference tracer. */
enum {
    /* CalcField_CPU_T_Curvature<float/double> SSE specialisations,
     * ElectroMag/src/CPU_Implement.cpp:207-351 and :366-498 (x86 builds).
     * PartField with explicit k (include/Electrostatics.h:38-51); the
     * curvature reference vector is the seed point, loaded once (:254-256)
     * and never updated; n must be a multiple of 64 (:223-224, rc 5). */
    ORC_CURV_SSE = 0,
    /* Generic CalcField_CPU_T_Curvature<T>, CPU_Implement.cpp:104-191, which
     * is what a build without __SSE__ (e.g. aarch64) runs: two-argument
     * PartField (Electrostatics.h:53-60) and the curvature reference vector
     * reset to the previous point every step (:148-153). */
    ORC_CURV_GENERIC = 1,
    /* Fixed-step CalcField_CPU_T<T>, CPU_Implement.cpp:38-102. */
    ORC_FIXED = 2
};

/* Termination classes of the extended tracer. */
enum { ORC_TERM_STEPS = 0, ORC_TERM_CHARGE = 1, ORC_TERM_NULL = 2 };

/*
 * Traces lines [line0, line0+nlines) of an n-line field-line array laid out
 * like the reference's Vector3<Array<T>>: component arrays x, y, z of
 * n*total_steps elements, vertex (line, step) at index step*n + line, row 0
 * holding the seeds.  charges: p records {x, y, z, q} (pointCharge<T>,
 * Electrostatics.h:30-35).  nlines == 0 means all n lines.
 * Returns the reference's codes: 0 ok, 1 n == 0, 2 resolution == 0,
 * 3 total_steps < 2, 5 n not a multiple of 64 (ORC_CURV_SSE only).
 * nthreads <= 0 uses the OpenMP default.
 */
int orc_calc_field_f32(float *x, float *y, float *z, size_t n,
                       size_t total_steps, const float *charges, size_t p,
                       float resolution, int variant, size_t line0,
                       size_t nlines, int nthreads);
int orc_calc_field_f64(double *x, double *y, double *z, size_t n,
                       size_t total_steps, const double *charges, size_t p,
                       double resolution, int variant, size_t line0,
                       size_t nlines, int nthreads);

/*
 * Field at m points: sequential sum over charges 0..p-1 (the reference's
 * charge order, CPU_Implement.cpp:274).  The f32 form repeats the reference's
 * float PartField arithmetic (three_arg != 0: Electrostatics.h:38-51 as the
 * SSE path calls it; 0: :53-60).  The f64 form is the FP64 oracle; when maxc
 * is non-null it also returns the largest single-charge contribution |E_j|.
 */
void orc_field_f32(const float *px, const float *py, const float *pz, size_t m,
                   const float *charges, size_t p, int three_arg, float *ex,
                   float *ey, float *ez);
void orc_field_f64(const double *px, const double *py, const double *pz,
                   size_t m, const double *charges, size_t p, double *ex,
                   double *ey, double *ez, double *maxc, int nthreads);

/*
 * Extended method (seeded lines, termination near negative charges, step
 * limit), FP64 throughout.  It reuses the SSE stepping rule of
 * CPU_Implement.cpp:322-338 (curvature vector = the line's seed).
 * For s = 1..max_steps-1 the field and the nearest negative charge are
 * evaluated at vertex s-1; the line stops with class ORC_TERM_CHARGE when
 * that vertex lies strictly within term_radius of a negative charge, with
 * ORC_TERM_NULL when the field is zero or the step is not finite, and with
 * ORC_TERM_STEPS after max_steps vertices.  len[l] counts valid vertices
 * (seed included); rows at and after len[l] are not written.
 * max_steps_per_line, when non-null, overrides max_steps per line.
 */
int orc_trace_lines_f64(const double *charges, size_t p, double *x, double *y,
                        double *z, size_t n, size_t max_steps,
                        const int32_t *max_steps_per_line, double resolution,
                        double term_radius, int32_t *len, int32_t *cls,
                        int nthreads);

/* Fibonacci-sphere seeds: lines_per_charge points at distance radius around
 * every positive charge, in charge order.  Returns the number written
 * (at most cap). */
size_t orc_seed_fibonacci_f64(const double *charges, size_t p,
                              size_t lines_per_charge, double radius,
                              double *sx, double *sy, double *sz, size_t cap);

#ifdef __cplusplus
}
#endif
#endif

#ifdef __cplusplus
extern "C" {
#endif
/*
 * Adjoint checks (FP64).  The frozen-step map of the reference rule:
 *   v_{s+1} = v_s + lam_s * E(v_s) / |E(v_s)|,
 *   lam_s = 1 / ((k_s + 1) * res), k_s the curvature of CPU_Implement.cpp:
 *   327-329 against the seed, computed on the unperturbed trajectory.
 * Loss L = sum over lines and rows s = 0..S-1 of |v_s - t_s|^2.
 * Layout: seeds sx/sy/sz (n), targets and vertices s*n + line (S rows).
 * lam (n*(S-1), s*n + line): written when lam_out is non-null; the map
 * uses lam_in when it is non-null, else its own lam.
 */
double orc_frozen_loss_f64(const double *charges, size_t p, const double *sx,
                           const double *sy, const double *sz, size_t n,
                           size_t S, double res, const double *tx,
                           const double *ty, const double *tz,
                           const double *lam_in, double *lam_out, double *vx,
                           double *vy, double *vz);
/* Complex-step derivative of the frozen loss (lam_in required) with respect
 * to charge j's component c (0..2 position, 3 magnitude): Im L(x + ih) / h. */
double orc_frozen_loss_cs_f64(const double *charges, size_t p, const double *sx,
                              const double *sy, const double *sz, size_t n,
                              size_t S, double res, const double *tx,
                              const double *ty, const double *tz,
                              const double *lam_in, size_t j, int c, double h);
/* Discrete adjoint of the frozen map in FP64: grad[4j+c] = dL/d(charge j,
 * component c) (c: x, y, z, q).  Returns L. */
double orc_frozen_grad_f64(const double *charges, size_t p, const double *sx,
                           const double *sy, const double *sz, size_t n,
                           size_t S, double res, const double *tx,
                           const double *ty, const double *tz,
                           const double *lam_in, double *grad);
/* The same discrete adjoint linearised at a given trajectory (vx, vy, vz:
 * S rows of n lines, e.g. a GPU forward's vertices in FP64), with lam_s
 * computed from the FP64 field at each given vertex (curvature against the
 * row-0 vertex; curvature 0: 1/res).  Returns L at that trajectory. */
double orc_adjoint_at_f64(const double *charges, size_t p, const double *vx,
                          const double *vy, const double *vz, size_t n, size_t S,
                          double res, int curvature, const double *tx,
                          const double *ty, const double *tz, double *grad);
/* The same with the field E' = E/K at each vertex given (fx, fy, fz: the
 * S-1 rows the steps used, e.g. a GPU forward's own field) instead of
 * recomputed in FP64: the step lengths, directions and |E'| of the frozen
 * map are those of the given field, the Jacobian products stay FP64 sums.
 * lam_fp32: the step lengths by the reference's FP32 step sequence from the
 * field rounded to FP32 (exactly those an FP32 forward took); 0: in FP64. */
double orc_adjoint_at_field_f64(const double *charges, size_t p, const double *vx,
                                const double *vy, const double *vz, size_t n, size_t S,
                                double res, int curvature, const double *tx,
                                const double *ty, const double *tz, const double *fx,
                                const double *fy, const double *fz, int lam_fp32,
                                double *grad);
#ifdef __cplusplus
}
#endif
