// The reference-side drop-in built against the reference's own headers:
// CalcField_CPU<float/double> (ElectroMag/src/"CPU Implement.h":25-30)
// specialised as one-line forwards to emgb300::calc_field, called on the
// reference's containers (Vector3<Array<T>>, Array<pointCharge<T>>,
// perfPacket).  Built by tests/test_capi.py where the reference tree exists.
#include <cstdio>

#include "CPU Implement.h"
#include "emgb300_dropin.hpp"

template <>
int CalcField_CPU<float>(Vector3<Array<float> > &lines,
                         Array<electro::pointCharge<float> > &charges, const size_t n,
                         float resolution, perfPacket &perf, bool useCurvature)
{
    return emgb300::calc_field<float>(lines, charges, n, resolution, perf, useCurvature);
}

template <>
int CalcField_CPU<double>(Vector3<Array<double> > &lines,
                          Array<electro::pointCharge<double> > &charges, const size_t n,
                          double resolution, perfPacket &perf, bool useCurvature)
{
    return emgb300::calc_field<double>(lines, charges, n, resolution, perf, useCurvature);
}

int main()
{
    const size_t n = 64, steps = 4;
    Vector3<Array<float> > lines;
    if (lines.AlignAlloc(n * steps))
        return 2;
    Array<electro::pointCharge<float> > charges(3, 256);
    perfPacket perf;
    perf.time = perf.performance = 0;
    // the reference's argument codes come back unchanged: resolution 0 -> 2
    const int rc_res = CalcField_CPU<float>(lines, charges, n, 0.0f, perf, true);
    // n == 0 -> 1
    const int rc_n = CalcField_CPU<float>(lines, charges, 0, 1.0f, perf, true);
    std::printf("rc_res=%d rc_n=%d\n", rc_res, rc_n);
    lines.Free();
    charges.Free();
    return (rc_res == 2 && rc_n == 1) ? 0 : 1;
}
