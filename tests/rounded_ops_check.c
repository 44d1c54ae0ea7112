/* CPU check of the exact arithmetic's branch-free correctly rounded
 * operations (electromag-with-cuda_gb300/csrc/em_math.cuh: sqrt_rn_nb,
 * rcp_rn_nb, div_rn_nb — Markstein's FMA-residual corrections), restated
 * in C with fmaf and no contraction: the quotient step from a correctly
 * rounded reciprocal on random quotients, and the one-step reciprocal and
 * root from starts 0..2 ulp off the correctly rounded value.
 * The correctly rounded FP32 result is the double result rounded to float
 * (double rounding is innocuous for division and square root when the
 * wider format has at least 2p + 2 bits: 53 >= 50).  Test infrastructure. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static float rcp_step(float b, float y0) { return fmaf(fmaf(-b, y0, 1.0f), y0, y0); }
static float sqrt_step(float x, float y0)
{
    const float s = x * y0, h = 0.5f * y0;
    return fmaf(fmaf(-s, s, x), h, s);
}
static float div_step(float a, float b, float y)
{
    const float q0 = a * y;
    return fmaf(fmaf(-b, q0, a), y, q0);
}

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next(void)
{
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

int main(void)
{
    /* quotient step from the correctly rounded reciprocal (Markstein's
     * theorem: then q0 + r y rounds correctly): asserted */
    long long bad_q = 0;
    const long long nq = 200000000;
    for (long long i = 0; i < nq; ++i) {
        const uint64_t h = next();
        const uint32_t ma = (uint32_t)(h & 0x7fffff), mb = (uint32_t)((h >> 23) & 0x7fffff);
        const uint32_t ea = (uint32_t)((h >> 46) % 121) + 67u, eb = (uint32_t)((h >> 54) % 121) + 67u;
        const uint32_t sa = (uint32_t)(h >> 62) & 1u, sb = (uint32_t)(h >> 63) & 1u;
        const float a = f_of((sa << 31) | (ea << 23) | ma), b = f_of((sb << 31) | (eb << 23) | mb);
        const float y = (float)(1.0 / (double)b);
        bad_q += u_of(div_step(a, b, y)) != u_of((float)((double)a / (double)b));
    }
    printf("%s quotients from the rounded reciprocal (%lld random, operands in "
           "[2^-60, 2^60]): %lld mismatches\n", bad_q ? "FAIL" : "ok", nq, bad_q);
    /* one-step reciprocal and root from a start k ulp off the correctly
     * rounded value: exact for k = 0 (asserted); for other starts a few
     * significands round wrongly (reported), so exactness rests on the
     * device's own approximations, which the library verifies on the device
     * before it uses these operations (exact_nb_verified) */
    long long br[5] = {0}, bs[5] = {0};
    for (uint32_t m = 0; m < (1u << 23); ++m) {
        const float b = f_of(0x3f800000u | m);
        const float r = (float)(1.0 / (double)b);
        for (int k = -2; k <= 2; ++k)
            br[k + 2] += u_of(rcp_step(b, f_of(u_of(r) + k))) != u_of(r);
    }
    for (uint32_t u = 0x3f800000u; u < 0x40800000u; ++u) {
        const float x = f_of(u);
        const double sq = sqrt((double)x);
        const float s = (float)sq, y = (float)(1.0 / sq);
        for (int k = -2; k <= 2; ++k)
            bs[k + 2] += u_of(sqrt_step(x, f_of(u_of(y) + k))) != u_of(s);
    }
    printf("%s reciprocal and root from the correctly rounded start: %lld, %lld mismatches\n",
           (br[2] || bs[2]) ? "FAIL" : "ok", br[2], bs[2]);
    for (int k = -2; k <= 2; ++k)
        if (k)
            printf("info start %+d ulp: reciprocal %lld of 2^23, root %lld of 2^24 round wrongly\n",
                   k, br[k + 2], bs[k + 2]);
    return (bad_q || br[2] || bs[2]) ? 1 : 0;
}
