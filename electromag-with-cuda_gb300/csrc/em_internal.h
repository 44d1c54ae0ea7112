// Internal declarations shared by the kernels (.cu) and the C ABI layer.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace em {

// Device error word values (the kernel's status, read back by the host).
enum DevErr : int {
    EM_DEVERR_NONE = 0,
    EM_DEVERR_TIMEOUT = 1, // a bounded wait gave up
    EM_DEVERR_CONFIG = 2,  // launch parameters inconsistent (checked in-kernel)
};

// Stepping rules (which reference routine a run reproduces).
enum Rule : int {
    RULE_SSE = 0,     // CPU_Implement.cpp:207-351 / :366-498 (curvature, seed vector)
    RULE_GENERIC = 1, // CPU_Implement.cpp:104-191 (curvature, previous point)
    RULE_FIXED = 2,   // CPU_Implement.cpp:38-102 (fixed step)
};

// Per-pair arithmetic.
enum Arith : int {
    ARITH_FAST = 0,  // rsqrt + FMA, k applied once per vertex
    ARITH_EXACT = 1, // the reference's IEEE operation sequence, bit-exact
    ARITH_FAST2 = 2, // fast form on packed FP32 pairs (.f32x2), paired charge layout
    ARITH_MIXED = 3, // FP32 pairs + corrected inv^3 + compensation, FP64 position
};

// Charge record: pointCharge<T> of include/Electrostatics.h:30-35.
struct alignas(32) ChargeD {
    double x, y, z, q;
};
template <class T> struct ChargeRec;
template <> struct ChargeRec<float> {
    using type = float4;
};
template <> struct ChargeRec<double> {
    using type = ChargeD;
};

// Parameters of the reference-layout tracer (CalcField_CPU semantics).
template <class T> struct RefTraceParams {
    T *x, *y, *z;              // n*total_steps each; vertex (line, s) at s*n + line
    const void *charges;       // padded charge records, 16-B aligned
    long long n;               // number of lines (row stride)
    long long n_groups;        // ceil(n / lines_per_warp)
    int total_steps;           // rows, including the start row
    int p_pad;                 // padded charge count (resident: all; streamed: n_tiles*tile)
    int n_tiles;               // streamed: number of charge tiles
    int tile_recs;             // streamed: records per tile
    int stages;                // streamed: ring depth
    int resident;              // 1: all charges staged once
    int rule;                  // Rule
    T resolution;
    int *err;                  // device error word
    // optional: the charge sum E/K (fast arithmetic) at vertex s of each
    // line, stored at (s * n + line) for s < total_steps - 1 (null: none)
    T *fx, *fy, *fz;
    // the seeds the SSE rule's curvature reads (null: row 0 of x, y, z); a
    // launch that resumes a trace passes x, y, z from its start row
    const T *seed_x, *seed_y, *seed_z;
    // mixed arithmetic: the conditioning bound kappa^2 of the re-evaluation
    // test, and the count of re-evaluated vertices (null: not counted)
    double kappa2;
    unsigned long long *refines;
    // optional, mixed arithmetic: the field each step uses (Coulomb constant
    // applied, after any re-evaluation), stored like fx (null: none)
    T *ox, *oy, *oz;
    // optional (resident charges only): a zeroed counter from which warps
    // take line groups in order instead of the fixed round-robin deal
    unsigned long long *group_ctr;
    // exact arithmetic (FP32): 1 when the branch-free rounded operations
    // were verified on this device (exact_nb_verified), else 0 (the
    // compiler's rounded operations)
    int exact_nb;
};

// The exact arithmetic's branch-free rounded operations checked once per
// device and process against the compiler's rounded operations
// (em_probe.cu; every admitted root operand and divisor and 2^24 random
// quotients, a few milliseconds on stream s, no allocation): true when they
// agree bit for bit.
bool exact_nb_verified(cudaStream_t s);

// Extended tracer (em_trace_ext.cu).
enum ExtMode : int {
    EXT_FAST = 0,  // T arithmetic throughout (float, or double = the FP64 path)
    EXT_MIXED = 1, // FP32 pairs + corrected inv^3 + compensation, FP64 position
    EXT_DF64 = 2,  // double-float pairs (two FP32 words), FP64 position and step
};
// CTA size cap of the lane-group kernel: the mixed pass needs more than the
// 64 registers a 1024-thread CTA leaves a thread (it spilled there)
constexpr int ext_cta_threads(int mode) { return mode == EXT_MIXED ? 512 : 1024; }
// CTA size of the tail kernel in every mode: its rows are a latency chain
// (pairs, two reductions, the step), which the 128-register cap shortens
// (GPU-scale set with termination, FP32: 12.1 ms at 1024 threads, 9.9 at 512)
constexpr int kExtWideThreads = 512;
// termination classes written by the kernel (same values as EM_TERM_*)
constexpr int EM_TERM_STEPS_DEV = 0;
constexpr int EM_TERM_CHARGE_DEV = 1;
constexpr int EM_TERM_NULL_DEV = 2;

template <class T> struct ExtParams {
    T *x, *y, *z;                   // n*max_steps each; row 0 = seeds
    T *ex, *ey, *ez;                // optional: field at each evaluated vertex
    const void *charges;            // staged negatives-first, p_pad records
    const int *meta;                // [0] = padded negative block size
    const float *qabs;              // largest |q|
    long long n;
    int max_steps;
    const int *steps_per_line;      // optional per-line limits
    double resolution;
    double term_r2;
    double null_frac;               // (the call's option; the test uses kappa2)
    int *len, *cls;
    unsigned long long *next_line, *evals, *refines;
    int p_pad, n_tiles, tile_recs, stages, resident;
    int stage_recs;                 // staged tile (the mixed mode's paired blocks)
    int regroup;                    // widen lane groups once the queue is dry
    int refine_fp64;                // mixed: re-evaluate in FP64 (else double-float)
    double kappa2;                  // mixed: the conditioning test's kappa^2
    int *err;
    // Tail hand-off.  Once the queue is dry and at most tail_lines lines are
    // still being traced, a kernel saves each of them (ExtCont) and stops;
    // a tail kernel then traces them with `wide` warps per line, and hands
    // them on again (to a wider launch) once few enough are left.
    // tail_lines = 0 turns the hand-off off.
    void *cont;                              // ExtCont<T> records written here
    unsigned long long *cont_count;          // ... and their count
    const void *cont_in;                     // the tail kernel's lines
    const unsigned long long *cont_in_count; // ... and their count
    unsigned long long *cont_next;           // input lines taken
    unsigned long long *live_count;          // lines neither finished nor handed off
    long long tail_lines;
    int wide;
};

// A line handed from the lane-group kernel to a tail kernel: its next row
// and limit, the evaluation point and the FP64 position accumulator.
template <class T> struct ExtCont {
    long long line;
    int s, lim;
    T px, py, pz;
    double dx, dy, dz;
};

template <class T>
cudaError_t launch_ext_stage(const void *raw, int p, void *staged, int p_pad, int gran,
                             int block, int *meta, float *qabs, cudaStream_t stream);
template <class T>
cudaError_t launch_ext_trace(const ExtParams<T> &p, const struct LaunchCfg &cfg, int mode,
                             cudaStream_t stream);
// The tail kernels over the handed-off lines (p.wide warps per line).
template <class T>
cudaError_t launch_ext_wide(const ExtParams<T> &p, const struct LaunchCfg &cfg, int mode,
                            cudaStream_t stream);
constexpr size_t kExtWideSlots = 4096; // static shared memory of the tail kernels (bound)

// Adjoint of the frozen-step map (em_adjoint.cu).
struct AdjParams {
    const float *x, *y, *z;    // forward vertices, n*rows
    const float *tx, *ty, *tz; // targets, n*rows
    const void *charges;       // staged plain records, p_pad (padded)
    const float *raw;          // the caller's p records
    int p, p_pad;
    long long n;
    int rows, seg;
    float resolution;
    int curvature;
    float *abar;               // 3n: dL/dv of the current row (x, y, z blocks)
    float *rec;                // 6 blocks of rec_stride floats: v, mu per record
    size_t rec_stride;         // >= seg * n
    double *gpart;             // slices * p * 4 partial sums
    int slices;
    int *err;
    // field E/K at the vertices of rows [f_row0, ...) (row stride n): the
    // forward's own output (f_row0 = 0), or one segment recomputed from the
    // stored vertices (f_row0 = the segment's first row)
    float *fx, *fy, *fz;
    int f_row0;
    int stored;                // 1: the forward stored the field of every row
    // fused backward: per team, 4 blocks of p_bwd compensated (hi, lo) sums
    float2 *tpart;
    int p_bwd, team_warps;
    long long teams;
    const void *charges_bwd;   // fused backward: the records in lane pairs
};
// Shape of the fused backward (p up to kAdjFusedMaxCharges charges).
constexpr int kAdjFusedMaxCharges = 4096;
struct AdjFused {
    int cpl;          // charges per lane
    int team_warps;   // warps per line team
    int p_bwd;        // staged records the fused kernel reads (32 * team_warps * cpl)
    int grid;         // persistent CTAs
    long long teams;  // grid * teams per CTA
    size_t smem;
};
int adjoint_charge_blocks(int p);
// FP64 slots after the loss that hold its per-CTA partials
int adjoint_loss_parts(int nsm);
// Fills *f and returns 1 when the fused backward applies to p charges.
int adjoint_fused_plan(int p, int nsm, AdjFused *f);
// fused == nullptr: the two-pass backward (field recompute + Jacobian-vector
// kernel, then the charge-stationary kernel) per 64-row segment.
// Checkpoint mode (fused, field not stored): the field of segment k is
// recomputed on `side` into half k % 2 of a two-segment buffer (half_elems
// apart) while the fused kernel of segment k - 1 runs on `stream`.
// The fused backward's lane-pair layout of p_bwd staged plain records.
cudaError_t launch_adjoint_pair_stage(const void *plain, int p_bwd, int team_warps,
                                      void *paired, cudaStream_t stream);
cudaError_t launch_adjoint_backward(const AdjParams &P, const AdjFused *fused, int nsm,
                                    size_t smem, double *loss, double *grad,
                                    cudaStream_t stream, cudaStream_t side,
                                    size_t half_elems);

// Batched tracing (em_trace_batch.cu).
struct BatchParams {
    const float4 *staged;        // every set's staged charges
    const long long *soff;       // per set: first staged record
    const int *spad, *snneg;     // per set: staged records, padded negative block
    const float *sqabs;          // per set: largest |q|
    const long long *coff;       // per set: first charge record (nsets + 1)
    const float *sx, *sy, *sz;   // seeds of every line (global line ids)
    const int *steps_per_line;   // optional per-line limits
    int max_steps;
    long long nlines;
    const int4 *items;           // {set, begin, end, 0}; begin/end: line ids (phase 0)
                                 // or positions in cont_in (later phases)
    const int *nitems;
    unsigned *item_ctr;
    const long long *cont_in;    // later phases: line ids sorted by set
    float *st_x, *st_y, *st_z;   // saved state of deferred lines
    int *st_s;
    long long *cont_out;         // lines deferred by this phase
    unsigned long long *cont_count;
    int budget;                  // field evaluations per line in this phase (0: no limit)
    int phase;
    float *vx, *vy, *vz;         // rows < store_rows of every line: row * nlines + line
    int store_rows;
    float *lx, *ly, *lz;         // last vertex
    int *len, *cls;
    double res, term_r2;
    unsigned long long *evals;   // pair interactions evaluated
    int resident_cap, tile_recs, stages, regroup;
    int *err;
};
struct BatchQueues {
    const long long *cont;           // lines deferred by the finished phase
    unsigned long long *cont_count;  // their number (reset by the sort)
    long long *cont_sorted;          // the same ids grouped by set
    int *set_count, *set_fill, *set_item_off;
    long long *set_line_off;
    int4 *next_items;
    int *next_nitems;
    unsigned *next_item_ctr;
    const int *set_order;            // sets by descending charge count
};
cudaError_t launch_batch_stage(const float *raw, const long long *coff, const long long *soff,
                               const int *spad, int gran, int nsets, float *staged, int *snneg,
                               float *sqabs, cudaStream_t stream);
cudaError_t launch_batch_sort(const BatchQueues &q, const long long *line_off, int nsets,
                              int item_lines, cudaStream_t stream);
cudaError_t prepare_batch_trace(size_t smem);
cudaError_t launch_batch_trace(const BatchParams &p, int tpl, int grid, int threads, size_t smem,
                               cudaStream_t stream);

struct LaunchCfg {
    int tpl;     // threads per line (1, 2, 4, 8)
    int kl;      // lines per lane (1, 2; 2 only for the fast forms)
    int warps;   // compute warps per CTA
    int grid;    // CTAs
    int resident;
    int stages;
    int tile_recs;
    size_t smem; // dynamic shared memory bytes
};

// Charge padding granule per launch configuration (records).
constexpr int kUnroll = 8;
// The exact arithmetic: lanes per line in FP32 (their terms are added in
// the reference's charge order by every lane of the line; FP64 keeps one
// lane per line) — 8 while every line fits one round of 512-thread CTAs at
// 8 lanes, else 4 (the reference's default run, 16 384 lines: 137 ms at 4
// lanes, 169 at 8; 1088 lines: 17.8 ms at 4, 11.9 at 8) — and the CTA size
// cap for a shape: one lane per line (16 terms in flight) needs the
// registers of 256-thread CTAs, several lanes per line (8 in flight) fit 512
constexpr int exact_max_threads(int tpl) { return tpl == 1 ? 256 : 512; }
// 8 lanes per line pass each round's terms through shared memory (eight
// float4 per lane, after the charge tiles, every warp of a CTA); 4 lanes
// broadcast them by shuffles (measured: 8 lanes 11.9 -> 11.1 ms on the
// 256-charge configuration with the buffer, 4 lanes 136 -> 151 ms on the
// reference's default run)
constexpr int kExactSmemTpl = 8;
constexpr size_t kExactTermBytesPerWarp = 32 * 8 * 16;
inline int exact_tpl_f32(long long n, int nsm)
{
    return n <= (long long)nsm * (exact_max_threads(8) / 32) * (32 / 8) ? 8 : 4;
}

template <class T>
cudaError_t launch_ref_trace(const RefTraceParams<T> &p, const LaunchCfg &cfg, int arith,
                             cudaStream_t stream);
// v[0, m) *= the Coulomb constant, rounded as the tracer rounds it.
template <class T> cudaError_t launch_scale_coulomb(T *v, size_t m, cudaStream_t stream);

// Stages p raw charge records into p_pad records (pad record {1e15, 1e15,
// 1e15, 0}, whose contribution is exactly zero), plain (paired = 0) or in
// the packed form's two-plane blocks of `block` records (1).
template <class T>
cudaError_t launch_stage_charges(const void *raw, int p, void *staged, int p_pad, int paired,
                                 int block, cudaStream_t stream);

// Adds k to the process-wide count of kernels launched by this library.
void count_launch(unsigned long long k);

// Field at m points, one thread per point (em_field.cu).
template <class T>
cudaError_t launch_field(const T *px, const T *py, const T *pz, long long m, const T *charges,
                         int p, int arith, int three_arg, T *ex, T *ey, T *ez,
                         cudaStream_t stream);

} // namespace em
