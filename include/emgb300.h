/*
 * emgb300.h — C ABI of the GB300 field-line tracer (libemgb300.so).
 *
 * Drop-in for ElectroMag's calc-field entry points:
 *   int CalcField_CPU<T>(Vector3<Array<T>>& fieldLines,
 *                        Array<pointCharge<T>>& pointCharges, size_t n,
 *                        T resolution, perfPacket& perfData,
 *                        bool useCurvature)
 *       ElectroMag/src/"CPU Implement.h":25-30, CPU_Implement.cpp:501-527
 *   int CalcField(Array<Vector3<T>>&, Array<pointCharge<T>>&, size_t n,
 *                 T resolution, perfPacket&, bool useCurvature)
 *       GPGPU_Segment/src/Electrostatics.cpp:28-42 (stubs returning -1)
 *
 * Layout contract (the reference's, include/SOA_utils.hpp:31-112):
 *   field lines  three component arrays x, y, z of n*total_steps elements;
 *                vertex (line, step) at index step*n + line; row 0 holds
 *                the seeds, rows 1..total_steps-1 are written.
 *   charges      p records {x, y, z, q} of the element type (16 B for
 *                float, 32 B for double; pointCharge<T>,
 *                include/Electrostatics.h:30-35), 16-B aligned.
 * The caller owns every buffer.  Calls are synchronous unless a stream is
 * given through em_options with device pointers.  No call aborts: every
 * failure is a return code.
 */
#ifndef EMGB300_H
#define EMGB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define EM_API __attribute__((visibility("default")))
#else
#define EM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- return codes -------------------------------------------------------
 * 0..5 are the reference's (CPU_Implement.cpp:213-230); the rest are new. */
#define EM_OK 0
#define EM_ERR_N_ZERO 1        /* n == 0                                  */
#define EM_ERR_RESOLUTION 2    /* resolution == 0                         */
#define EM_ERR_STEPS 3         /* total_steps < 2                         */
#define EM_ERR_ARG 4           /* null pointer, misaligned or bad option  */
#define EM_ERR_N_ALIGN 5       /* n % 64 != 0 while reproducing the SSE
                                  path's restriction (CPU_Implement.cpp:223) */
#define EM_ERR_CUDA 10         /* a CUDA runtime call failed               */
#define EM_ERR_NOMEM 11        /* device allocation failed                 */
#define EM_ERR_TIMEOUT 12      /* a device-side wait hit its time limit    */
#define EM_ERR_NO_DEVICE 13    /* no CUDA device / library not usable      */
#define EM_ERR_TOO_LARGE 14    /* sizes beyond what the entry point takes  */
#define EM_ERR_IO 15           /* a file could not be opened or written    */

/* ---- arithmetic of the pair sum ------------------------------------------ */
#define EM_ARITH_FAST 0   /* FP32 (or FP64 for _f64) rsqrt + FMA             */
#define EM_ARITH_EXACT 1  /* the reference's IEEE operation sequence:
                             bit-identical to its strict x86 build          */
#define EM_ARITH_MIXED 2  /* _f32 only: FP32 pairs (two charges per packed
                             instruction) with a Newton-corrected inv^3,
                             compensated chunk sums, the line position in
                             FP64, and the field re-evaluated in
                             double-float where the sum is ill-conditioned
                             (sqrt(sum |t_j|^2) > refine_kappa |E|)        */

/* ---- stepping rule (which reference routine to reproduce) ---------------- */
#define EM_RULE_SSE 0      /* CalcField_CPU_T_Curvature<float/double> SSE
                              specialisations, CPU_Implement.cpp:207-498: the
                              curvature vector is the line's seed           */
#define EM_RULE_GENERIC 1  /* the generic template, CPU_Implement.cpp:104-191
                              (non-SSE builds): previous point              */

/* Performance record; the fields of perfPacket ("Data Structures.h":221-236)
 * plus the work counted by this library. */
typedef struct em_perf {
    double performance;  /* GFLOP/s, reference accounting:
                            n*(steps-1)*(18*p+13)/time (CPU_Implement.cpp:348) */
    double time;         /* seconds of device execution (CUDA events)        */
    volatile double progress; /* 0 before the call, 1.0 when complete        */
    double pairs;        /* pair interactions evaluated                      */
    double wall_time;    /* seconds of the whole call (copies included)      */
    double fp64_refines; /* vertices whose field was re-evaluated at higher
                            precision (mixed arithmetic)                     */
} em_perf;

/* Options for the _ex entry points.  Zero-initialise and set what you need. */
typedef struct em_options {
    int arith;        /* EM_ARITH_*                                          */
    int rule;         /* EM_RULE_* (curvature runs only)                     */
    int require_n64;  /* 1: return EM_ERR_N_ALIGN for n % 64 like the SSE
                         path; 0: any n                                      */
    int device_ptrs;  /* 1: x, y, z and charges are device pointers          */
    void *stream;     /* cudaStream_t for device_ptrs calls (NULL: the
                         library's stream, call returns when done)           */
    int threads_per_line; /* 0: automatic; else 1, 2, 4 or 8 (the exact
                             arithmetic sets its own: 4 or 8 lanes per line
                             in FP32, adding the terms in the reference's
                             order, 1 in FP64)                              */
    int warps_per_cta;    /* 0: automatic; else 1..32                        */
    int tile_charges;     /* 0: automatic; streamed-charge tile size         */
    int force_streamed;   /* 1: stream charge tiles even if they fit          */
    int pack;             /* EM_PACK_*: pair loop form for fast FP32         */
    int lines_per_thread; /* 0: automatic; 1 or 2 (fast arithmetic only)     */
    int precision;        /* em_trace_lines_f32: EM_PREC_FP32, EM_PREC_MIXED
                             or EM_PREC_DF64                                 */
    double null_frac;     /* mixed (both tracers), when refine_kappa is 0:
                             re-evaluate the field where |E| is below this
                             fraction of the terms' size sqrt(sum |t_j|^2),
                             i.e. refine_kappa = 1/null_frac (0: the
                             default 2.5 of refine_kappa)                    */
    int deterministic;    /* extended tracer: 1 keeps every line on its
                             initial lane group, so results repeat bit for
                             bit; 0 (default) lets warps widen the groups of
                             their last lines once no lines are left to hand
                             out, and hands the last lines to several warps
                             each (faster tails, last-bit differences)       */
    int adjoint_checkpoint; /* em_adjoint_f32: 0 (default) keeps the forward's
                             field at every vertex (12 more bytes per vertex);
                             1 keeps only the vertices and recomputes the
                             field per 64-row segment                        */
    int refine;           /* em_trace_lines_f32, mixed precision:
                             EM_REFINE_DF64 (default) or EM_REFINE_FP64, the
                             arithmetic of the re-evaluated field            */
    void *field_out;      /* em_calc_field_ex_* with device_ptrs only
                             (NULL: none): the field each step uses, as the
                             arrays' type, Coulomb constant applied; three
                             arrays of n*(total_steps-1) values back to back
                             (x, then y, then z), the field at vertex s of
                             line l at s*n + l                               */
    double refine_kappa;  /* mixed arithmetic (EM_ARITH_MIXED on the
                             reference loop, EM_PREC_MIXED in the extended
                             tracer): a vertex's field is re-evaluated where
                             the terms' size sqrt(sum_j |t_j|^2) exceeds
                             refine_kappa * |E| (0: see null_frac)           */
} em_options;

/* ---- precision of the extended tracer (em_trace_lines_f32) ---------------- */
#define EM_PREC_FP32 0    /* FP32 pairs and positions                        */
#define EM_PREC_MIXED 1   /* FP32 pairs with a Newton-corrected inv^3,
                             compensated sums, FP64 positions, the field
                             re-evaluated where the sum is ill-conditioned   */
#define EM_PREC_DF64 2    /* double-float pairs (two FP32 words, ~48 bits) on
                             the FP32 pipes, FP64 field, step and positions:
                             FP64-class fields at several times the native
                             FP64 rate of GB300                              */
#define EM_REFINE_DF64 0  /* mixed: re-evaluate in double-float (default)    */
#define EM_REFINE_FP64 1  /* mixed: re-evaluate in FP64                      */

/* ---- termination classes of the extended tracer --------------------------- */
#define EM_TERM_STEPS 0   /* reached its step limit                          */
#define EM_TERM_CHARGE 1  /* came within term_radius of a negative charge    */
#define EM_TERM_NULL 2    /* zero or non-finite field / step                 */

/* ---- pair loop form (fast FP32 only) -------------------------------------- */
#define EM_PACK_AUTO 0    /* library's choice                                */
#define EM_PACK_SCALAR 1  /* one charge per FP32 instruction                 */
#define EM_PACK_PAIRS 2   /* two charges per packed .f32x2 instruction       */

/* Reference-compatible entry points (host pointers, synchronous).
 * Replace CalcField_CPU<float>/<double> (CPU_Implement.cpp:501-527): same
 * layout, same codes in the same order (n == 0 -> 1, resolution == 0 -> 2,
 * curvature with n % 64 -> 5, total_steps < 2 -> 3).  total_steps is the
 * reference's fieldLines.GetSize()/n (CPU_Implement.cpp:219).  The arrays
 * may be ordinary (pageable) memory: above 64 MB of vertices the trace runs
 * in 8 row chunks and each chunk's copy back overlaps the next chunk, with
 * pageable and page-locked buffers alike. */
EM_API int em_calc_field_f32(float *x, float *y, float *z, size_t n, size_t total_steps,
                      const float *charges, size_t p, float resolution,
                      int use_curvature, em_perf *perf);
EM_API int em_calc_field_f64(double *x, double *y, double *z, size_t n,
                      size_t total_steps, const double *charges, size_t p,
                      double resolution, int use_curvature, em_perf *perf);

/* The same with options: device pointers, streams, arithmetic, stepping
 * rule, the n % 64 restriction lifted (require_n64 = 0). */
EM_API int em_calc_field_ex_f32(float *x, float *y, float *z, size_t n,
                         size_t total_steps, const float *charges, size_t p,
                         float resolution, int use_curvature,
                         const em_options *opt, em_perf *perf);
EM_API int em_calc_field_ex_f64(double *x, double *y, double *z, size_t n,
                         size_t total_steps, const double *charges, size_t p,
                         double resolution, int use_curvature,
                         const em_options *opt, em_perf *perf);

/* Tracing without any device allocation by the library.  This entry point
 * has no counterpart in the reference (whose calc-field paths allocate and
 * own their buffers).  It is for callers that cannot let a library call
 * cudaMalloc: applications whose own pool holds the whole GPU, and loops
 * that cannot take the device-wide synchronisation an allocation may cause.
 * x, y, z (n*total_steps each, reference layout) and charges
 * (p records {x,y,z,q}, 16-B aligned) are DEVICE pointers; the work runs on
 * `stream` (NULL: the default stream) and the call returns when it is done.
 * Default options: fast FP32, the SSE stepping rule, any n.
 * Its scratch is one static device array per GPU, held until exit, sized
 * for at most EM_NOALLOC_MAX_CHARGES charges; larger sets return
 * EM_ERR_TOO_LARGE.  The first call on a device performs a one-time set-up
 * (make it before any stream capture).  Every call synchronises `stream`
 * before it returns (it reads the kernel's error word back).  All calls on a
 * device share the array: calls that overlap on the GPU race, so order them. */
#define EM_NOALLOC_MAX_CHARGES 16384
EM_API int em_calc_field_noalloc_f32(float *x, float *y, float *z, size_t n,
                                     size_t total_steps, const float *charges,
                                     size_t p, float resolution,
                                     int use_curvature, void *stream);

/* Extended method: field lines seeded around charges (em_seed_fibonacci_*),
 * traced with the reference's stepping rule (CPU_Implement.cpp:322-338:
 * curvature against the line's seed) until, for s = 1.., the field at
 * vertex s-1 is evaluated and that vertex lies strictly within term_radius
 * of a negative charge (EM_TERM_CHARGE), the field or the step is zero or
 * non-finite (EM_TERM_NULL), or the line has max_steps vertices (or
 * steps_per_line[line], when given) (EM_TERM_STEPS).  The reference stops
 * only at the step limit; seeding and termination are additions.
 * Layout as the reference's: x, y, z of n*max_steps, vertex (line, s) at
 * s*n + line, row 0 = seeds.  len[line] = vertices written (seed included),
 * cls[line] = EM_TERM_*; rows at and after len[line] are unspecified.
 * ex, ey, ez (optional, n*max_steps): the field evaluated at vertex s, at
 * row s, for every evaluated vertex.  opt->precision selects FP32 or mixed
 * precision (_f32); _f64 runs FP64 throughout.  Host pointers unless
 * opt->device_ptrs.  perf->pairs counts field evaluations x p. */
EM_API int em_trace_lines_f32(float *x, float *y, float *z, size_t n,
                              size_t max_steps, const int32_t *steps_per_line,
                              const float *charges, size_t p, float resolution,
                              float term_radius, int32_t *len, int32_t *cls,
                              float *ex, float *ey, float *ez,
                              const em_options *opt, em_perf *perf);
EM_API int em_trace_lines_f64(double *x, double *y, double *z, size_t n,
                              size_t max_steps, const int32_t *steps_per_line,
                              const double *charges, size_t p,
                              double resolution, double term_radius,
                              int32_t *len, int32_t *cls, double *ex,
                              double *ey, double *ez, const em_options *opt,
                              em_perf *perf);

/* Gradients of a vertex loss through the tracer (no counterpart in the
 * reference).  Runs the forward trace (fast FP32, the reference rule:
 * curvature against the seed when use_curvature, else the fixed step) on
 * x, y, z (row 0 = seeds in, rows 1..rows-1 written), then the adjoint of
 * the discrete map v_{s+1} = v_s + lam_s E_s/|E_s| with the step lengths
 * lam_s = 1/((k_s+1) res) held at their forward values:
 *   *loss = sum over lines and rows of |v - t|^2 (targets tx, ty, tz),
 *   grad[4j+c] = dL/d(charge j component c), c = x, y, z, q (FP64).
 * The backward walks each line from its last row to its first.  For
 * p <= 4096 one fused pass forms every (vertex, charge) term once and feeds
 * both the line's adjoint and the charge's gradient; it reads the field the
 * forward stored at every vertex, or, with opt->adjoint_checkpoint, the field
 * recomputed from the stored vertices per 64-row segment.  Larger sets run
 * two passes per 64-row segment (the field recompute with the line adjoint,
 * then the charge gradients).  Charges must fit in shared memory
 * (p <= 14000, else EM_ERR_TOO_LARGE).  fwd / bwd (optional) receive the
 * forward and the backward device times (time) and pair evaluations.  Host
 * pointers unless opt->device_ptrs. */
EM_API int em_adjoint_f32(float *x, float *y, float *z, size_t n, size_t rows,
                          const float *charges, size_t p, float resolution,
                          int use_curvature, const float *tx, const float *ty,
                          const float *tz, double *loss, double *grad,
                          const em_options *opt, em_perf *fwd, em_perf *bwd);

/* Batched tracing of many independent charge sets (the extended method) in
 * persistent launches fed by a device work queue (no counterpart in the
 * reference, which traces one set per call).  Set s owns charge records
 * [charge_off[s], charge_off[s+1]) and lines [line_off[s], line_off[s+1])
 * (global line ids; charge_off and line_off are HOST arrays of nsets+1).
 * Seeds sx/sy/sz, optional steps_per_line and the outputs are indexed by
 * global line id: len, cls, the last vertex lx/ly/lz, and the first
 * store_rows rows of every line in vx/vy/vz (row * nlines + line; may be
 * NULL when store_rows == 0).  Host pointers unless opt->device_ptrs.
 * perf->pairs counts field evaluations x the set's charge count. */
typedef struct em_batch_options {
    int threads_per_line; /* 0: 16; else 4, 8 or 16 (lanes per line)        */
    int lines_per_item;   /* 0: 512 lines per phase-0 work item; later
                             phases' items hold the lines of one set that a
                             CTA traces at once (31 * 32 / threads_per_line),
                             largest sets first                              */
    int first_budget;     /* 0: 64 field evaluations per line in phase 0;
                             each later phase has four times more, the last
                             is unlimited                                    */
    int phases;           /* 0: 4                                            */
    int tile_charges;     /* 0: 1024; tile of sets too large for shared
                             memory                                          */
    int stages;           /* 0: 4; ring depth for those sets                 */
    int use_graph;        /* 1: capture the launches into a CUDA graph and
                             replay it                                       */
    int deterministic;    /* 1: no lane-group widening (bit-repeatable)      */
    int device_ptrs;
    void *stream;
} em_batch_options;
EM_API int em_trace_batch_f32(size_t nsets, const float *charges,
                              const int64_t *charge_off, const float *sx,
                              const float *sy, const float *sz,
                              const int64_t *line_off,
                              const int32_t *steps_per_line, int max_steps,
                              float resolution, float term_radius,
                              int store_rows, float *vx, float *vy, float *vz,
                              float *lx, float *ly, float *lz, int32_t *len,
                              int32_t *cls, const em_batch_options *opt,
                              em_perf *perf);

/* Seeds on a sphere of `radius` around every positive charge (q > 0), in
 * charge order: lines_per_charge golden-angle spiral directions
 * (z_i = 1 - (2i+1)/L, phi_i = i * pi (3 - sqrt 5)).  Writes at most cap
 * seeds to sx, sy, sz (host arrays) and their number to *count.  The
 * reference seeds from a grid or random points ("Electromag utils.h":29-70);
 * this seeding is the extended method's. */
EM_API int em_seed_fibonacci_f32(const float *charges, size_t p,
                                 size_t lines_per_charge, float radius,
                                 float *sx, float *sy, float *sz, size_t cap,
                                 size_t *count);

/* Field at m points, no stepping: E_i = sum_j PartField(charge_j, point_i)
 * summed in charge order (include/Electrostatics.h:38-60 as
 * CPU_Implement.cpp:274-320 sums it).  Points are SoA px/py/pz; the result
 * goes to ex/ey/ez.  Host pointers unless opt->device_ptrs.  With
 * EM_ARITH_EXACT, opt->rule picks the PartField form: EM_RULE_SSE the
 * three-argument one (:38-51), EM_RULE_GENERIC the two-argument one (:53-60).
 * opt may be NULL (fast arithmetic, host pointers).  m above 2^31 * 256 - 256
 * points or p above 2^29 charges: EM_ERR_TOO_LARGE. */
EM_API int em_field_f32(const float *px, const float *py, const float *pz,
                        size_t m, const float *charges, size_t p, float *ex,
                        float *ey, float *ez, const em_options *opt);
EM_API int em_field_f64(const double *px, const double *py, const double *pz,
                        size_t m, const double *charges, size_t p, double *ex,
                        double *ey, double *ez, const em_options *opt);

/* One range of lines, [line0, line0 + nlines), of the caller's host arrays
 * (reference layout, n lines per row) traced on CUDA device `device`, from
 * any host thread (the calling thread's current device is restored).  Row 0
 * of the range is read, rows 1..total_steps-1 of the range are written; the
 * rest of the arrays is untouched, so ranges on different devices may run
 * at the same time.  The per-device work of the reference's multi-device
 * functor (GPGPU_Segment/src/Abstract_Functor.cpp:29-160, MainFunctor of
 * ElectrostaticFunctor.hpp) with the rule and codes of em_calc_field_ex_*;
 * EM_ERR_NO_DEVICE for a device that does not exist.  Host pointers only. */
EM_API int em_calc_field_part_f32(int device, float *x, float *y, float *z,
                                  size_t n, size_t total_steps, size_t line0,
                                  size_t nlines, const float *charges, size_t p,
                                  float resolution, int use_curvature,
                                  const em_options *opt, em_perf *perf);
EM_API int em_calc_field_part_f64(int device, double *x, double *y, double *z,
                                  size_t n, size_t total_steps, size_t line0,
                                  size_t nlines, const double *charges,
                                  size_t p, double resolution, int use_curvature,
                                  const em_options *opt, em_perf *perf);

/* The whole trace split over several CUDA devices by the functor of
 * include/emgb300_functor.hpp (the reference's AbstractFunctor lifecycle
 * and remap policy, Abstract_Functor.cpp:29-160): one contiguous range of
 * lines per entry of devices[] (an ordinal may repeat), one host thread per
 * range; a range whose device fails moves to a device that has succeeded.
 * ran_on (optional, ndevices entries) gets the device each range completed
 * on, -1 if none; *nfailed (optional) the ranges that never completed.
 * Returns EM_OK when every range completed, else the last failing range's
 * code.  Host pointers only. */
EM_API int em_calc_field_multi_f32(const int *devices, size_t ndevices, float *x,
                                   float *y, float *z, size_t n,
                                   size_t total_steps, const float *charges,
                                   size_t p, float resolution, int use_curvature,
                                   const em_options *opt, em_perf *perf,
                                   size_t *nfailed, int *ran_on);
EM_API int em_calc_field_multi_f64(const int *devices, size_t ndevices,
                                   double *x, double *y, double *z, size_t n,
                                   size_t total_steps, const double *charges,
                                   size_t p, double resolution,
                                   int use_curvature, const em_options *opt,
                                   em_perf *perf, size_t *nfailed, int *ran_on);

/* One or more velocity-Verlet steps of moving point charges (emgVerletStep,
 * ElectroMag/src/Particle_System.cpp:109-190; no counterpart runs in the
 * reference, whose template is never instantiated).  dyn: n records
 * {x, y, z, q, vx, vy, vz, m} (dynamicPointCharge, Electrodynamics.h:29-34),
 * updated in place; accel: n x 3, a(t) in and a(t + dt) out.  Per step and
 * particle, from the start-of-step states of the others: v' = v + a dt/2,
 * r' = r + v' dt; E = K sum over the static charges (p records {x,y,z,q})
 * and the other particles of q r / |r|^3 at r'; B = 1e-7 sum over the other
 * particles of q v x r / |r|^3; a = q (E + v' x B) / m; v = v' + a dt/2;
 * then reflection off the walls of [box_min, box_max].  Returns 1 for n == 0
 * (the reference's check).  opt->threads_per_line, if set, is the number of
 * lanes that share a particle's sums (1, 2 or 4; default: enough to fill the
 * GPU).  Host pointers unless opt->device_ptrs. */
EM_API int em_verlet_step_f32(float *dyn, float *accel, size_t n,
                              const float *charges, size_t p,
                              const float *box_min, const float *box_max,
                              float dt, size_t steps, const em_options *opt,
                              em_perf *perf);
EM_API int em_verlet_step_f64(double *dyn, double *accel, size_t n,
                              const double *charges, size_t p,
                              const double *box_min, const double *box_max,
                              double dt, size_t steps, const em_options *opt,
                              em_perf *perf);

/* ---- the reference program's inputs and outputs (host code) --------------
 * Presets of ElectroMag.cpp:43-55 (SimulationParams: lines nx*ny*nz, static
 * charges, rows per line), selected there by --bogo, --micro, --enhanced,
 * --extreme, --insane, --fuckingInsane (default "normal"; "cpu" is defined
 * but unreachable from the command line).  Returns EM_ERR_ARG for an
 * unknown name. */
typedef struct em_preset_params {
    size_t nx, ny, nz;     /* line grid                                      */
    size_t p_static;       /* point charges                                  */
    size_t p_dynamic;      /* unused by the tracer (0 in every preset)       */
    size_t len;            /* rows per line, the seed row included           */
} em_preset_params;
EM_API int em_preset(const char *name, em_preset_params *out);

/* InitializePointChargeArray ("Electromag utils.h":91-111): per charge x, y,
 * z = (rand() - RAND_MAX/2) / RAND_MAX * 10000 and q = (rand() - RAND_MAX/10)
 * / RAND_MAX, in the reference's T arithmetic, from the C library's rand()
 * stream after srand(seed) (the reference: seed 1, or a timer with
 * --randseed).  The stream is this library's own restatement of the GNU C
 * library's additive generator, so results do not depend on the host's
 * libc and the caller's rand() state is untouched.  charges: p {x,y,z,q}. */
EM_API int em_init_charges_f32(float *charges, size_t p, unsigned seed);
EM_API int em_init_charges_f64(double *charges, size_t p, unsigned seed);
/* InitializeFieldLineArray ("Electromag utils.h":29-70) into the first
 * nx*ny*nz entries of x, y, z (row 0 of the line arrays).  Grid mode
 * (random = 0): 10 * (i - w/2 + 1e-5) per axis, line k*w*h + j*w + i; random
 * mode: (rand() - RAND_MAX/2) / RAND_MAX * 10000 per component after
 * srand(seed). */
EM_API int em_init_lines_f32(float *x, float *y, float *z, size_t nx, size_t ny,
                             size_t nz, int random, unsigned seed);
EM_API int em_init_lines_f64(double *x, double *y, double *z, size_t nx,
                             size_t ny, size_t nz, int random, unsigned seed);

/* The --save dump (ElectroMag.cpp:372-397): for each line, for each row,
 * " CPUL [line][row] x: X y: Y z: Z" from the a arrays, then the same with
 * "GPUL" from the b arrays; either set may be NULL (the reference writes
 * only the enabled paths).  Floats print like std::ostream's default (%g,
 * six significant digits).  Host pointers, reference layout (row*n + line). */
EM_API int em_save_lines_text_f32(const char *path, size_t n, size_t rows,
                                  const float *ax, const float *ay,
                                  const float *az, const float *bx,
                                  const float *by, const float *bz);
/* The --autoregress check (ElectroMag.cpp:400-453): per line, the first row
 * where |a - b| (FP32, the reference's vec3Len(vec3(a, b))) exceeds
 * threshold (the reference: 0.1).  first[line] gets that row or -1; when
 * path is not NULL the report is written in the reference's regression.txt
 * format (the previous row, the diverging row, their 3D offsets; row 0 is
 * reported alone).  *ndiverged (optional) counts the lines that diverge.
 * The scan runs on the GPU; with opt->device_ptrs all six arrays are device
 * pointers, else host arrays that are copied in.  first may be NULL. */
EM_API int em_autoregress_f32(const char *path, size_t n, size_t rows,
                              const float *ax, const float *ay,
                              const float *az, const float *bx,
                              const float *by, const float *bz,
                              float threshold, long long *first,
                              size_t *ndiverged, const em_options *opt);

/* Library state.  em_device_count: CUDA devices visible (0 when none).
 * em_release: frees the cached device buffers of the current device.
 * em_strerror: text for a return code. */
EM_API int em_device_count(void);
EM_API int em_release(void);
/* em_release for one device ordinal (the calling thread's device is kept). */
EM_API int em_release_device(int device);
EM_API const char *em_strerror(int code);
/* Diagnostics.  em_fp32_peak_tflops: measured FP32 FFMA throughput of the
 * current device (dense FMA chains, 2 FLOP per FMA), the denominator of the
 * tracer's FP32 roofline.  em_launch_count: kernels this library has
 * launched in this process. */
EM_API int em_fp32_peak_tflops(double *tflops, double *seconds);
/* Failure-path self-test: one warp waits on a device barrier that nothing
 * completes, bounded by limit_ms (1..5000).  Every device-side wait of the
 * tracer kernels is bounded the same way.  Returns EM_ERR_TIMEOUT when the
 * wait expired and the kernel returned as designed (the device stays
 * usable); *elapsed_ms gets the kernel's duration. */
EM_API int em_selftest_wait_timeout(int limit_ms, double *elapsed_ms);
/* Self-check of the exact arithmetic's branch-free correctly rounded
 * operations against the compiler's rounded ones, over the operand ranges
 * the exact tracer admits (other operands take the rounded operations):
 * every float in [2^-40, 2^40] for the square root, every float in
 * [2^-60, 2^60] for the reciprocal, and n_quotients seeded random quotients
 * of operands in [2^-60, 2^60].  mismatches[0..2]: root, reciprocal,
 * quotient mismatches (all zero when the operations agree bit for bit). */
EM_API int em_selftest_rounded_ops(unsigned long long n_quotients,
                                   unsigned long long *mismatches);
EM_API unsigned long long em_launch_count(void);
/* Library version, "major.minor.patch". */
EM_API const char *em_version(void);

#ifdef __cplusplus
}
#endif
#endif /* EMGB300_H */
