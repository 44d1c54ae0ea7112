// C ABI of the multi-device trace (em_calc_field_multi_*): the reference's
// functor lifecycle and remap policy (include/emgb300_functor.hpp) over the
// listed CUDA devices.
#include <vector>

#include "emgb300.h"
#include "emgb300_functor.hpp"

namespace {

template <class T>
int calc_field_multi(const int *devices, size_t ndev, T *x, T *y, T *z, size_t n,
                     size_t total_steps, const T *charges, size_t p, T resolution,
                     int use_curvature, const em_options *opt, em_perf *perf, size_t *nfailed,
                     int *ran_on)
{
    if (!devices || !ndev)
        return EM_ERR_ARG;
    if (!n)
        return EM_ERR_N_ZERO;
    if (resolution == 0)
        return EM_ERR_RESOLUTION;
    if (total_steps < 2)
        return EM_ERR_STEPS;
    if (!x || !y || !z || (p && !charges) || (opt && opt->device_ptrs))
        return EM_ERR_ARG;
    emgb300::CudaElectrostaticFunctor<T> f(std::vector<int>(devices, devices + ndev),
                                           opt ? *opt : em_options());
    typename emgb300::CudaElectrostaticFunctor<T>::BindDataParams b{};
    b.x = x;
    b.y = y;
    b.z = z;
    b.nLines = n;
    b.totalSteps = total_steps;
    b.charges = charges;
    b.nCharges = p;
    b.resolution = resolution;
    b.perfData = perf;
    b.useCurvature = use_curvature != 0;
    f.BindData(&b);
    const unsigned long failed = f.Run();
    if (failed >= (1ul << 16))
        return EM_ERR_ARG;
    if (nfailed)
        *nfailed = failed;
    int code = EM_OK;
    for (size_t i = 0; i < ndev; ++i) {
        if (ran_on)
            ran_on[i] = i < f.FunctorCount() ? f.FunctorDevice(i) : -1;
        if (i < f.FunctorCount() && f.FunctorDevice(i) < 0)
            code = f.FunctorCode(i);
    }
    return code;
}

} // namespace

extern "C" {

int em_calc_field_multi_f32(const int *devices, size_t ndevices, float *x, float *y, float *z,
                            size_t n, size_t total_steps, const float *charges, size_t p,
                            float resolution, int use_curvature, const em_options *opt,
                            em_perf *perf, size_t *nfailed, int *ran_on)
{
    return calc_field_multi<float>(devices, ndevices, x, y, z, n, total_steps, charges, p,
                                   resolution, use_curvature, opt, perf, nfailed, ran_on);
}

int em_calc_field_multi_f64(const int *devices, size_t ndevices, double *x, double *y,
                            double *z, size_t n, size_t total_steps, const double *charges,
                            size_t p, double resolution, int use_curvature,
                            const em_options *opt, em_perf *perf, size_t *nfailed, int *ran_on)
{
    return calc_field_multi<double>(devices, ndevices, x, y, z, n, total_steps, charges, p,
                                    resolution, use_curvature, opt, perf, nfailed, ran_on);
}

} // extern "C"
