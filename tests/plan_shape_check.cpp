// The launch planner (csrc/em_plan.h) on a model of a GB300 (152 SMs,
// 227 KB of opt-in shared memory): the shapes the measured sweeps chose.
// Compiled and run on the CPU by tests/test_plan_shapes.py.
#include <cstdio>

#include "em_plan.h"

using namespace em;

static int failures = 0;

static void expect(const char *what, bool ok)
{
    std::printf("%s %s\n", ok ? "ok" : "FAIL", what);
    if (!ok)
        ++failures;
}

int main()
{
    DevCtx c;
    c.nsm = 152;
    c.smem_optin = 232448;
    Plan p;
    em_options o{};

    // 32 736 lines x 4096 charges (the value workload): 8 lanes x 2 lines,
    // 27 warps, resident
    expect("gpu-scale fast", make_plan<float>(c, 32736, 4096, o, &p) == EM_OK &&
                                 p.cfg.tpl == 8 && p.cfg.kl == 2 && p.cfg.warps == 27 &&
                                 p.cfg.resident == 1 && p.arith == ARITH_FAST);
    // 16 384 lines x 1024 charges (the reference's default run): one line
    // per lane doubles the warps
    expect("16384x1024 fast", make_plan<float>(c, 16384, 1024, o, &p) == EM_OK &&
                                  p.cfg.tpl == 8 && p.cfg.kl == 1 && p.cfg.warps == 27);
    // the caller's lines per lane is kept
    o.lines_per_thread = 2;
    expect("16384x1024 kl forced", make_plan<float>(c, 16384, 1024, o, &p) == EM_OK &&
                                       p.cfg.kl == 2);
    o.lines_per_thread = 0;
    // exact arithmetic: FP32 with 4 lanes per line for many lines, 8 for
    // few (terms added in charge order by every lane), FP64 one lane per
    // line; one line per lane, CTAs within the exact form's cap
    o.arith = EM_ARITH_EXACT;
    expect("exact", make_plan<float>(c, 16384, 1024, o, &p) == EM_OK &&
                        p.cfg.tpl == exact_tpl_f32(16384, c.nsm) && p.cfg.kl == 1 &&
                        p.cfg.warps <= exact_max_threads(p.cfg.tpl) / 32 &&
                        p.arith == ARITH_EXACT);
    expect("exact few lines", make_plan<float>(c, 1088, 256, o, &p) == EM_OK &&
                                  p.cfg.tpl == exact_tpl_f32(1088, c.nsm));
    expect("exact f64", make_plan<double>(c, 16384, 1024, o, &p) == EM_OK && p.cfg.tpl == 1 &&
                            p.cfg.kl == 1 && p.cfg.warps <= exact_max_threads(1) / 32);
    // mixed: 8 lanes x 2 lines, every warp of a 512-thread CTA the groups
    // keep busy (groups come from a queue: no round balancing)
    o.arith = EM_ARITH_MIXED;
    expect("mixed", make_plan<float>(c, 32736, 4096, o, &p) == EM_OK && p.cfg.tpl == 8 &&
                        p.cfg.kl == 2 && p.cfg.warps == 16 && p.arith == ARITH_MIXED);
    // 16 384 lines: 2048 groups, 14 per SM
    expect("mixed 16384x1024", make_plan<float>(c, 16384, 1024, o, &p) == EM_OK &&
                                   p.cfg.tpl == 8 && p.cfg.kl == 2 && p.cfg.warps == 14);
    expect("mixed fp64 rejected", make_plan<double>(c, 32736, 4096, o, &p) == EM_ERR_ARG);
    o.arith = EM_ARITH_FAST;
    // 20 000 charges do not fit: streamed tiles, a producer warp's room left
    expect("streamed", make_plan<float>(c, 32768, 20000, o, &p) == EM_OK &&
                           p.cfg.resident == 0 && p.cfg.warps <= 31 && p.cfg.stages >= 2 &&
                           p.n_tiles * p.cfg.tile_recs >= 20000);
    // no charges: one granule of pad records (a zero field, as the reference)
    expect("zero charges", make_plan<float>(c, 1024, 0, o, &p) == EM_OK && p.p_pad > 0);
    // bad shapes are refused
    o.threads_per_line = 3;
    expect("bad lanes", make_plan<float>(c, 1024, 64, o, &p) == EM_ERR_ARG);
    return failures ? 1 : 0;
}
