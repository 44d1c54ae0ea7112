// The reference program's inputs and outputs, host side: the presets of
// ElectroMag.cpp:43-55, the charge and line generators of
// "Electromag utils.h":29-111 (with the C library rand() stream they draw
// from) and the --save text dump of ElectroMag.cpp:372-397.
//
// Floating-point expressions follow the reference's C++ evaluation order and
// types operation by operation (T arithmetic, int -> T conversions where the
// reference converts); this file is compiled without contraction so each
// operation rounds once, as in the reference's x86 build.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "emgb300.h"

namespace em {
namespace {

constexpr int kRandMax = 2147483647; // RAND_MAX of the GNU C library

// rand() of the GNU C library (its default TYPE_3 generator), restated:
// state s_0 = seed (0 -> 1), s_i = 16807 s_{i-1} mod (2^31 - 1) for i < 31
// by Schrage's factorisation on signed 32-bit words; then the additive
// lagged-Fibonacci recurrence s_i += s_{i-31} over the 31-word ring with the
// partner 3 words ahead (mod 2^32), output (s >> 1); the first 310 outputs
// are discarded.
class CRand {
  public:
    explicit CRand(unsigned seed)
    {
        const int32_t s0 = static_cast<int32_t>(seed == 0 ? 1u : seed);
        ring_[0] = static_cast<uint32_t>(s0);
        long long w = s0;
        for (int i = 1; i < 31; ++i) {
            const long long hi = w / 127773, lo = w % 127773;
            w = 16807 * lo - 2836 * hi;
            if (w < 0)
                w += 2147483647;
            ring_[i] = static_cast<uint32_t>(w);
        }
        front_ = 3;
        rear_ = 0;
        for (int i = 0; i < 310; ++i)
            next();
    }
    int next()
    {
        ring_[front_] += ring_[rear_];
        const uint32_t v = ring_[front_] >> 1;
        front_ = front_ == 30 ? 0 : front_ + 1;
        rear_ = rear_ == 30 ? 0 : rear_ + 1;
        return static_cast<int>(v);
    }

  private:
    uint32_t ring_[31];
    int front_, rear_;
};

struct Preset {
    const char *name;
    em_preset_params v;
};

// SimulationParams of ElectroMag.cpp:43-55, by the command-line word that
// selects each one.
constexpr Preset kPresets[] = {
    {"normal", {128, 128, 1, 1024, 0, 2500}},
    {"enhanced", {256, 112, 1, 2048, 0, 5000}},
    {"extreme", {256, 256, 1, 2048, 0, 5000}},
    {"insane", {512, 512, 1, 2048, 0, 5000}},
    {"fuckingInsane", {1024, 1024, 1, 5120, 0, 10000}},
    {"cpu", {64, 64, 1, 1000, 0, 1000}},
    {"micro", {16, 16, 1, 1000, 0, 1000}},
    {"bogo", {16, 16, 1, 50, 0, 500}},
};

// (T)(rand() - (T)RAND_MAX/2) / RAND_MAX * 10000 and
// (T)(rand() - (T)RAND_MAX/10) / RAND_MAX ("Electromag utils.h":100-109)
template <class T> void init_charges(T *q, size_t p, unsigned seed)
{
    CRand r(seed);
    const T rm = static_cast<T>(kRandMax);
    for (size_t i = 0; i < p; ++i) {
        for (int c = 0; c < 3; ++c) {
            const T d = static_cast<T>(r.next()) - rm / T(2);
            q[4 * i + c] = d / rm * T(10000);
        }
        const T d = static_cast<T>(r.next()) - rm / T(10);
        q[4 * i + 3] = d / rm;
    }
}

// "Electromag utils.h":29-70
template <class T>
void init_lines(T *x, T *y, T *z, size_t w, size_t h, size_t d, int random, unsigned seed)
{
    const size_t n = w * h * d;
    if (random) {
        // (T)(rand() - RAND_MAX/2) / RAND_MAX * 10000, integer half
        CRand r(seed);
        const T rm = static_cast<T>(kRandMax);
        for (size_t i = 0; i < n; ++i) {
            x[i] = static_cast<T>(r.next() - kRandMax / 2) / rm * T(10000);
            y[i] = static_cast<T>(r.next() - kRandMax / 2) / rm * T(10000);
            z[i] = static_cast<T>(r.next() - kRandMax / 2) / rm * T(10000);
        }
        return;
    }
    // (T)(-((T)extent)/2 + 1E-5): the T quotient plus a double constant,
    // rounded back to T; each coordinate then steps by ++ in T
    auto start = [](size_t extent) {
        const T half = -static_cast<T>(extent) / T(2);
        return static_cast<T>(static_cast<double>(half) + 1E-5);
    };
    T zv = start(d);
    for (size_t k = 0; k < d; ++k, ++zv) {
        T yv = start(h);
        for (size_t j = 0; j < h; ++j, ++yv) {
            T xv = start(w);
            for (size_t i = 0; i < w; ++i, ++xv) {
                const size_t idx = k * w * h + j * w + i;
                x[idx] = T(10) * xv;
                y[idx] = T(10) * yv;
                z[idx] = T(10) * zv;
            }
        }
    }
}

// One dump line: std::ostream's default float output is printf's %g with
// six significant digits (the float widened to double first).
inline void put_vertex(std::string &out, const char *tag, size_t line, size_t row, float x,
                       float y, float z)
{
    char buf[160];
    const int len = std::snprintf(buf, sizeof buf, " %s [%zu][%zu] x: %g y: %g z: %g\n", tag,
                                  line, row, (double)x, (double)y, (double)z);
    out.append(buf, (size_t)len);
}

} // namespace
} // namespace em

extern "C" {

int em_preset(const char *name, em_preset_params *out)
{
    if (!name || !out)
        return EM_ERR_ARG;
    for (const auto &p : em::kPresets) {
        if (!std::strcmp(p.name, name)) {
            *out = p.v;
            return EM_OK;
        }
    }
    return EM_ERR_ARG;
}

int em_init_charges_f32(float *charges, size_t p, unsigned seed)
{
    if (!charges && p)
        return EM_ERR_ARG;
    em::init_charges<float>(charges, p, seed);
    return EM_OK;
}

int em_init_charges_f64(double *charges, size_t p, unsigned seed)
{
    if (!charges && p)
        return EM_ERR_ARG;
    em::init_charges<double>(charges, p, seed);
    return EM_OK;
}

int em_init_lines_f32(float *x, float *y, float *z, size_t nx, size_t ny, size_t nz,
                      int random, unsigned seed)
{
    if ((!x || !y || !z) && nx * ny * nz)
        return EM_ERR_ARG;
    em::init_lines<float>(x, y, z, nx, ny, nz, random, seed);
    return EM_OK;
}

int em_init_lines_f64(double *x, double *y, double *z, size_t nx, size_t ny, size_t nz,
                      int random, unsigned seed)
{
    if ((!x || !y || !z) && nx * ny * nz)
        return EM_ERR_ARG;
    em::init_lines<double>(x, y, z, nx, ny, nz, random, seed);
    return EM_OK;
}

int em_save_lines_text_f32(const char *path, size_t n, size_t rows, const float *ax,
                           const float *ay, const float *az, const float *bx, const float *by,
                           const float *bz)
{
    const bool a = ax && ay && az, b = bx && by && bz;
    if (!path || (!a && !b))
        return EM_ERR_ARG;
    std::FILE *f = std::fopen(path, "wb");
    if (!f)
        return EM_ERR_IO;
    // lines are formatted by all host threads in blocks and written in order
    const unsigned nt = std::max(1u, std::thread::hardware_concurrency());
    // at most about 8 MB of text per thread and block (a dump line is ~60
    // bytes), and every thread busy when the lines run out sooner
    const size_t line_bytes = (rows ? rows : 1) * 60 * ((a ? 1 : 0) + (b ? 1 : 0));
    const size_t per_block = std::max<size_t>(
        1, std::min((size_t(8) << 20) / line_bytes, (n + nt - 1) / nt));
    std::vector<std::string> part(nt);
    bool ok = true;
    for (size_t l0 = 0; l0 < n && ok; l0 += per_block * nt) {
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < nt; ++t) {
            pool.emplace_back([&, t] {
                std::string &out = part[t];
                out.clear();
                const size_t lo = l0 + t * per_block, hi = std::min(n, lo + per_block);
                for (size_t line = lo; line < hi; ++line) {
                    for (size_t row = 0; row < rows; ++row) {
                        const size_t i = row * n + line;
                        if (a)
                            em::put_vertex(out, "CPUL", line, row, ax[i], ay[i], az[i]);
                        if (b)
                            em::put_vertex(out, "GPUL", line, row, bx[i], by[i], bz[i]);
                    }
                }
            });
        }
        for (auto &th : pool)
            th.join();
        for (unsigned t = 0; t < nt && ok; ++t)
            ok = std::fwrite(part[t].data(), 1, part[t].size(), f) == part[t].size();
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? EM_OK : EM_ERR_IO;
}

} // extern "C"
