// Compile/link check of include/emgb300_dropin.hpp against containers shaped
// like the reference's (written here; they only mirror the member names the
// forwarding templates use).  Exit code 0 = every expectation held.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "emgb300_dropin.hpp"

template <class T> struct V3 {
    T x, y, z;
};
template <class T> struct Arr {
    std::vector<T> v;
    explicit Arr(size_t n) : v(n) {}
    T *GetDataPointer() { return v.data(); }
    size_t GetSize() { return v.size(); }
};
template <class T> struct Lines {
    Arr<T> x, y, z;
    explicit Lines(size_t n) : x(n), y(n), z(n) {}
    V3<T *> GetDataPointers() { return {x.GetDataPointer(), y.GetDataPointer(), z.GetDataPointer()}; }
    size_t GetSize() { return x.GetSize(); }
};
struct Perf {
    double performance, time;
    volatile double progress;
};

static int failures = 0;
static void expect(int got, int want, const char *what)
{
    if (got != want) {
        std::printf("FAIL %s: got %d want %d\n", what, got, want);
        ++failures;
    }
}

int main()
{
    Perf perf = {0, 0, 0};
    Arr<float> q(4 * 8);
    for (size_t i = 0; i < 8; ++i) {
        q.v[4 * i] = (float)i;
        q.v[4 * i + 1] = 1.5f * (float)i;
        q.v[4 * i + 2] = -0.5f * (float)i;
        q.v[4 * i + 3] = (i & 1) ? 2.f : -3.f;
    }
    // charges are passed as the record array: GetSize() must count records
    struct Q {
        Arr<float> *a;
        const float *GetDataPointer() { return a->GetDataPointer(); }
        size_t GetSize() { return a->GetSize() / 4; }
    } charges{&q};
    {
        Lines<float> l(64 * 4);
        expect(emgb300::calc_field<float>(l, charges, 0, 1.0f, perf, true), 1, "n == 0");
        expect(emgb300::calc_field<float>(l, charges, 64, 0.0f, perf, true), 2, "res == 0");
        expect(emgb300::calc_field<float>(l, charges, 32, 1.0f, perf, true), 5, "n % 64");
    }
    {
        Lines<float> l(64);
        expect(emgb300::calc_field<float>(l, charges, 64, 1.0f, perf, true), 3, "steps < 2");
    }
    {
        Lines<float> l(64 * 4);
        for (size_t i = 0; i < 64; ++i) {
            l.x.v[i] = 10.f + (float)i;
            l.y.v[i] = -3.f;
            l.z.v[i] = 0.25f * (float)i;
        }
        const int rc = emgb300::calc_field<float>(l, charges, 64, 1.0f, perf, true);
        if (em_device_count() > 0) {
            expect(rc, 0, "traced call");
            if (perf.progress != 1.0)
                expect(0, 1, "progress");
        } else {
            expect(rc, EM_ERR_NO_DEVICE, "traced call without a device");
        }
    }
    return failures ? 1 : 0;
}
