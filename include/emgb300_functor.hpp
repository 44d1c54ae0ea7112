// emgb300_functor.hpp — the reference's multi-device functor interface over
// CUDA devices, on the C ABI of emgb300.h.
//
// AbstractFunctor keeps the reference's virtual interface and lifecycle
// (GPGPU_Segment/src/Abstract_Functor.hpp:52-146): BindData ->
// AllocateResources -> GenerateParameterList -> one host thread per functor
// running MainFunctor(functor, device) -> PostRun, with Fail() and
// FailOnFunctor(i) as the error checks and Run()'s return values (1 << 16
// when allocation fails, 2 << 16 when the parameter list fails, otherwise
// the number of functors that could not complete).  Its remap policy is the
// one of Abstract_Functor.cpp:29-90: functor i starts on device i; a functor
// that fails moves to a device that has gone idle after succeeding, or waits
// in the failed list, from which the next device that succeeds takes it.
//
// CudaElectrostaticFunctor<T> is the tracer's functor
// (ElectrostaticFunctor.hpp:28-70): BindData takes the reference-layout line
// arrays and the charges; GenerateParameterList splits the lines into one
// contiguous range per listed CUDA device; MainFunctor traces a range with
// em_calc_field_part_*.  Listing a device more than once runs several ranges
// on it (they serialise on that device).  C++17.
#ifndef EMGB300_FUNCTOR_HPP
#define EMGB300_FUNCTOR_HPP

#include <algorithm>
#include <cstddef>
#include <mutex>
#include <thread>
#include <type_traits>
#include <vector>

#include "emgb300.h"

namespace emgb300 {

class AbstractFunctor
{
  public:
    struct AbstractFunctorParams {
    };

    AbstractFunctor() = default;
    virtual ~AbstractFunctor() = default;

    virtual unsigned long Run();
    virtual void BindData(void *dataParameters) = 0;
    virtual void AllocateResources() = 0;
    virtual void ReleaseResources() = 0;
    virtual void GenerateParameterList(size_t *nDevices) = 0;
    virtual unsigned long MainFunctor(size_t functorIndex, size_t deviceIndex) = 0;
    virtual unsigned long AuxFunctor() = 0;
    virtual void PostRun() = 0;
    virtual bool Fail() = 0;
    virtual bool FailOnFunctor(size_t functorIndex) = 0;

  private:
    std::mutex remap_;
    std::vector<size_t> idle_;   // devices free after a success
    std::vector<size_t> failed_; // functors waiting for a device

    void Worker(size_t functorIndex);
};

inline void AbstractFunctor::Worker(size_t functor)
{
    size_t device = functor;
    for (;;) {
        MainFunctor(functor, device);
        const bool bad = FailOnFunctor(functor);
        std::lock_guard<std::mutex> hold(remap_);
        if (bad) {
            if (idle_.empty()) {
                failed_.push_back(functor);
                return;
            }
            device = idle_.back(); // retry this functor on an idle device
            idle_.pop_back();
        } else {
            if (failed_.empty()) {
                idle_.push_back(device);
                return;
            }
            functor = failed_.back(); // this device takes a failed functor
            failed_.pop_back();
        }
    }
}

inline unsigned long AbstractFunctor::Run()
{
    AllocateResources();
    if (Fail())
        return 1ul << 16;
    size_t n = 0;
    GenerateParameterList(&n);
    if (Fail())
        return 2ul << 16;
    idle_.clear();
    failed_.clear();
    idle_.reserve(n);
    failed_.reserve(n);
    std::vector<std::thread> workers;
    workers.reserve(n);
    for (size_t i = 0; i < n; ++i)
        workers.emplace_back(&AbstractFunctor::Worker, this, i);
    for (auto &w : workers)
        w.join();
    PostRun();
    return static_cast<unsigned long>(failed_.size());
}

template <class T> class CudaElectrostaticFunctor : public AbstractFunctor
{
  public:
    /// BindDataParams of ElectrostaticFunctor.hpp:35-50, on plain arrays:
    /// x/y/z hold nLines * totalSteps values (row 0 = seeds), charges hold
    /// nCharges {x, y, z, q} records.
    struct BindDataParams {
        T *x, *y, *z;
        size_t nLines, totalSteps;
        const T *charges;
        size_t nCharges;
        T resolution;
        em_perf *perfData; // optional: the run's aggregate
        bool useCurvature;
    };

    /// devices: CUDA ordinals, one functor each (empty: every visible device)
    explicit CudaElectrostaticFunctor(std::vector<int> devices = {},
                                      em_options options = em_options())
        : devices_(std::move(devices)), opt_(options)
    {
        opt_.device_ptrs = 0;
    }

    void BindData(void *dataParameters) override
    {
        d_ = *static_cast<const BindDataParams *>(dataParameters);
        bound_ = true;
    }

    void AllocateResources() override
    {
        fail_ = !bound_;
        if (devices_.empty())
            for (int i = 0; i < em_device_count(); ++i)
                devices_.push_back(i);
        if (devices_.empty())
            fail_ = true;
    }

    void ReleaseResources() override
    {
        std::vector<int> seen;
        for (int dev : devices_) {
            if (std::find(seen.begin(), seen.end(), dev) == seen.end()) {
                seen.push_back(dev);
                em_release_device(dev);
            }
        }
    }

    void GenerateParameterList(size_t *nDevices) override
    {
        const size_t nf = std::min(devices_.size(), d_.nLines);
        if (!nf || d_.totalSteps < 2) {
            fail_ = true;
            *nDevices = 0;
            return;
        }
        first_.assign(nf + 1, 0);
        for (size_t f = 0; f <= nf; ++f)
            first_[f] = d_.nLines * f / nf;
        codes_.assign(nf, -1);
        ranOn_.assign(nf, -1);
        perf_.assign(nf, em_perf());
        *nDevices = nf;
    }

    unsigned long MainFunctor(size_t functorIndex, size_t deviceIndex) override
    {
        const size_t f = functorIndex;
        const int dev = devices_[deviceIndex];
        const int rc = part(dev, first_[f], first_[f + 1] - first_[f], &perf_[f]);
        codes_[f] = rc;
        if (rc == EM_OK)
            ranOn_[f] = dev;
        return static_cast<unsigned long>(rc);
    }

    unsigned long AuxFunctor() override { return 0; }

    void PostRun() override
    {
        if (!d_.perfData)
            return;
        em_perf agg = em_perf();
        double flops = 0;
        for (size_t f = 0; f < perf_.size(); ++f) {
            if (codes_[f] != EM_OK)
                continue;
            agg.time = std::max(agg.time, perf_[f].time);
            agg.pairs += perf_[f].pairs;
            flops += perf_[f].performance * perf_[f].time;
        }
        agg.performance = agg.time > 0 ? flops / agg.time : 0;
        agg.progress = 1.0;
        *d_.perfData = agg;
    }

    bool Fail() override { return fail_; }
    bool FailOnFunctor(size_t functorIndex) override
    {
        return functorIndex >= codes_.size() || codes_[functorIndex] != EM_OK;
    }

    /// Return code of functor i's last attempt, and the device it completed
    /// on (-1: it did not).
    int FunctorCode(size_t i) const { return i < codes_.size() ? codes_[i] : EM_ERR_ARG; }
    int FunctorDevice(size_t i) const { return i < ranOn_.size() ? ranOn_[i] : -1; }
    size_t FunctorCount() const { return codes_.size(); }

  private:
    int part(int dev, size_t line0, size_t count, em_perf *perf);

    std::vector<int> devices_;
    em_options opt_;
    BindDataParams d_ = BindDataParams();
    bool bound_ = false, fail_ = false;
    std::vector<size_t> first_;
    std::vector<int> codes_, ranOn_;
    std::vector<em_perf> perf_;
};

template <class T>
int CudaElectrostaticFunctor<T>::part(int dev, size_t line0, size_t count, em_perf *perf)
{
    if constexpr (std::is_same<T, float>::value)
        return em_calc_field_part_f32(dev, d_.x, d_.y, d_.z, d_.nLines, d_.totalSteps, line0,
                                      count, d_.charges, d_.nCharges, d_.resolution,
                                      d_.useCurvature, &opt_, perf);
    else
        return em_calc_field_part_f64(dev, d_.x, d_.y, d_.z, d_.nLines, d_.totalSteps, line0,
                                      count, d_.charges, d_.nCharges, d_.resolution,
                                      d_.useCurvature, &opt_, perf);
}

} // namespace emgb300

#endif // EMGB300_FUNCTOR_HPP
