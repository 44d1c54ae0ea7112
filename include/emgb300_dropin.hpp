// emgb300_dropin.hpp — C++ forwarding layer from ElectroMag's calc-field
// signatures to the C ABI in emgb300.h.
//
// The templates only use the member functions the reference's containers
// expose (include/SOA_utils.hpp:31-112, include/"Data Structures.h":42-236):
//   fieldLines.GetDataPointers() -> {T* x, T* y, T* z}, fieldLines.GetSize()
//   pointCharges.GetDataPointer(), pointCharges.GetSize()
//   perfData.time, perfData.performance, perfData.progress
// so this header includes none of the reference's code.  A maintainer
// replaces CPU_Implement.cpp's CalcField_CPU<float/double> specialisations
// (CPU_Implement.cpp:501-527) with one-line forwards to emgb300::calc_field
// and the GPGPU_Segment CalcField stubs (Electrostatics.cpp:28-42) with
// forwards to emgb300::calc_field_aos.
#ifndef EMGB300_DROPIN_HPP
#define EMGB300_DROPIN_HPP

#include <atomic>
#include <chrono>
#include <cstddef>
#include <thread>
#include <vector>

#include "emgb300.h"

namespace emgb300 {

inline int call(float *x, float *y, float *z, size_t n, size_t steps, const void *q,
                size_t p, float res, bool curv, em_perf *ep)
{
    return em_calc_field_f32(x, y, z, n, steps, static_cast<const float *>(q), p, res,
                             curv ? 1 : 0, ep);
}
inline int call(double *x, double *y, double *z, size_t n, size_t steps, const void *q,
                size_t p, double res, bool curv, em_perf *ep)
{
    return em_calc_field_f64(x, y, z, n, steps, static_cast<const double *>(q), p, res,
                             curv ? 1 : 0, ep);
}

// CalcField_CPU<T>(fieldLines, pointCharges, n, resolution, perfData,
// useCurvature) over the reference's SoA container (Vector3<Array<T>>).
// totalSteps = fieldLines.GetSize()/n as in CPU_Implement.cpp:219; the
// n == 0 check precedes the division like the reference's.
// perfData.progress follows the call's progress while it runs (a watcher
// thread copies em_perf.progress every millisecond), so a monitor thread
// polling it, as the reference's does ("Electromag utils.h":133-156), sees
// the rows traced so far.
template <class T, class Lines, class Charges, class Perf>
int calc_field(Lines &fieldLines, Charges &pointCharges, size_t n, T resolution,
               Perf &perfData, bool useCurvature)
{
    em_perf ep = em_perf();
    const size_t steps = n ? fieldLines.GetSize() / n : 0;
    auto d = fieldLines.GetDataPointers();
    std::atomic<bool> done(false);
    std::thread watcher([&] {
        while (!done.load(std::memory_order_acquire)) {
            const double v = ep.progress;
            if (v > 0 && v < 1)
                perfData.progress = v;
            std::this_thread::sleep_for(std::chrono::milliseconds(1));
        }
    });
    const int rc = call(d.x, d.y, d.z, n, steps,
                        static_cast<const void *>(pointCharges.GetDataPointer()),
                        pointCharges.GetSize(), resolution, useCurvature, &ep);
    done.store(true, std::memory_order_release);
    watcher.join();
    if (rc == EM_OK) {
        perfData.time = ep.time;
        perfData.performance = ep.performance;
        perfData.progress = ep.progress;
    }
    return rc;
}

// CalcField(Array<Vector3<T>>&, ...) of GPGPU_Segment/src/Electrostatics.cpp:
// 28-42: the same trace over an array-of-structures line container (element
// step*n + line is a {x, y, z} record).  Converted to SoA around the call.
template <class T, class LinesAoS, class Charges, class Perf>
int calc_field_aos(LinesAoS &fieldLines, Charges &pointCharges, size_t n, T resolution,
                   Perf &perfData, bool useCurvature)
{
    if (!n)
        return EM_ERR_N_ZERO;
    const size_t total = fieldLines.GetSize();
    std::vector<T> x(total), y(total), z(total);
    T *rec = reinterpret_cast<T *>(fieldLines.GetDataPointer());
    for (size_t i = 0; i < total; ++i) {
        x[i] = rec[3 * i];
        y[i] = rec[3 * i + 1];
        z[i] = rec[3 * i + 2];
    }
    em_perf ep = em_perf();
    const int rc = call(x.data(), y.data(), z.data(), n, total / n,
                        static_cast<const void *>(pointCharges.GetDataPointer()),
                        pointCharges.GetSize(), resolution, useCurvature, &ep);
    if (rc == EM_OK) {
        for (size_t i = n; i < total; ++i) {
            rec[3 * i] = x[i];
            rec[3 * i + 1] = y[i];
            rec[3 * i + 2] = z[i];
        }
        perfData.time = ep.time;
        perfData.performance = ep.performance;
        perfData.progress = ep.progress;
    }
    return rc;
}

} // namespace emgb300

#endif // EMGB300_DROPIN_HPP
