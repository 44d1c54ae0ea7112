/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * C entry points around the reference's own CalcField_CPU<float/double>
 * (declared in ElectroMag/src/"CPU Implement.h":25-30, defined in
 * ElectroMag/src/CPU_Implement.cpp:501-527).  oracle/build_ref.sh compiles
 * this file together with the unmodified reference source into
 * oracle/_ref/libemref_{strict,fast}.so; tests/golden/make_golden.py loads
 * those to produce the committed golden vectors.  The reference containers
 * own their storage, so the wrapper copies the caller's arrays in and out.
 */
#include "CPU Implement.h"

#include <cstring>

namespace {

template <class T>
int run_ref(T *x, T *y, T *z, size_t n, size_t total_steps, const T *charges,
            size_t p, T resolution, int use_curvature, double *time_s)
{
    Vector3<Array<T> > lines;
    if (n * total_steps && lines.AlignAlloc(n * total_steps))
        return -100;
    Array<electro::pointCharge<T> > q(p ? p : 1, 256);
    if (p)
        std::memcpy(q.GetDataPointer(), charges, p * 4 * sizeof(T));
    // GetSize() drives p in the reference; a zero-charge set is not
    // representable through Array(), so p == 0 is rejected here.
    if (!p)
        return -101;
    if (n * total_steps) {
        Vector3<T *> d = lines.GetDataPointers();
        std::memcpy(d.x, x, n * total_steps * sizeof(T));
        std::memcpy(d.y, y, n * total_steps * sizeof(T));
        std::memcpy(d.z, z, n * total_steps * sizeof(T));
    }
    perfPacket perf;
    perf.performance = perf.time = 0;
    const int rc = CalcField_CPU<T>(lines, q, n, resolution, perf,
                                    use_curvature != 0);
    if (n * total_steps) {
        Vector3<T *> d = lines.GetDataPointers();
        std::memcpy(x, d.x, n * total_steps * sizeof(T));
        std::memcpy(y, d.y, n * total_steps * sizeof(T));
        std::memcpy(z, d.z, n * total_steps * sizeof(T));
    }
    if (time_s)
        *time_s = perf.time;
    lines.Free();
    q.Free();
    return rc;
}

} // namespace

extern "C" int ref_calc_field_f32(float *x, float *y, float *z, size_t n,
                                  size_t total_steps, const float *charges,
                                  size_t p, float resolution,
                                  int use_curvature, double *time_s)
{
    return run_ref<float>(x, y, z, n, total_steps, charges, p, resolution,
                          use_curvature, time_s);
}

extern "C" int ref_calc_field_f64(double *x, double *y, double *z, size_t n,
                                  size_t total_steps, const double *charges,
                                  size_t p, double resolution,
                                  int use_curvature, double *time_s)
{
    return run_ref<double>(x, y, z, n, total_steps, charges, p, resolution,
                           use_curvature, time_s);
}
