// The functor lifecycle and remap policy of include/emgb300_functor.hpp on
// fake devices (no GPU): devices listed as broken fail every functor they
// run.  Each scenario prints "ok <name>"; any mismatch exits non-zero.
#include <chrono>
#include <cstdio>
#include <mutex>
#include <set>
#include <thread>
#include <vector>

#include "emgb300_functor.hpp"

namespace {

struct Fake : emgb300::AbstractFunctor {
    size_t ndev = 4;
    std::set<size_t> broken;
    int slow_dev = -1, slow_ms = 0;
    bool fail_alloc = false, fail_params = false, fail = false;
    std::mutex m;
    std::vector<int> done_on, attempts, last_ok;
    std::vector<std::pair<size_t, size_t>> runs; // (functor, device)

    void BindData(void *) override {}
    void AllocateResources() override { fail = fail_alloc; }
    void ReleaseResources() override {}
    void GenerateParameterList(size_t *n) override
    {
        if (fail_params) {
            fail = true;
            *n = 0;
            return;
        }
        *n = ndev;
        done_on.assign(ndev, -1);
        attempts.assign(ndev, 0);
        last_ok.assign(ndev, 0);
    }
    unsigned long MainFunctor(size_t f, size_t d) override
    {
        if ((int)d == slow_dev)
            std::this_thread::sleep_for(std::chrono::milliseconds(slow_ms));
        std::lock_guard<std::mutex> g(m);
        ++attempts[f];
        runs.emplace_back(f, d);
        const bool ok = !broken.count(d);
        last_ok[f] = ok;
        if (ok)
            done_on[f] = (int)d;
        return ok ? 0 : 1;
    }
    unsigned long AuxFunctor() override { return 0; }
    void PostRun() override {}
    bool Fail() override { return fail; }
    bool FailOnFunctor(size_t f) override { return !last_ok[f]; }
};

int bad = 0;
void check(bool c, const char *name)
{
    std::printf("%s %s\n", c ? "ok" : "FAIL", name);
    if (!c)
        ++bad;
}

} // namespace

int main()
{
    {
        Fake f;
        const unsigned long r = f.Run();
        bool same = true;
        for (size_t i = 0; i < f.ndev; ++i)
            same &= f.done_on[i] == (int)i && f.attempts[i] == 1;
        check(r == 0 && same, "no_failures_each_functor_on_its_device");
    }
    {
        Fake f;
        f.broken = {2};
        f.slow_dev = 2; // the others finish and go idle first
        f.slow_ms = 50;
        const unsigned long r = f.Run();
        bool none_on_2 = true, all_done = true;
        for (size_t i = 0; i < f.ndev; ++i) {
            none_on_2 &= f.done_on[i] != 2;
            all_done &= f.done_on[i] >= 0;
        }
        check(r == 0 && all_done && none_on_2 && f.attempts[2] == 2,
              "failed_functor_moves_to_idle_device");
    }
    {
        Fake f;
        f.broken = {1, 2, 3};
        f.slow_dev = 0; // the failures queue up before device 0 is free
        f.slow_ms = 50;
        const unsigned long r = f.Run();
        bool on0 = true;
        for (size_t i = 0; i < f.ndev; ++i)
            on0 &= f.done_on[i] == 0;
        check(r == 0 && on0, "queued_failures_drain_on_the_working_device");
    }
    {
        Fake f;
        f.broken = {1, 2, 3};
        const unsigned long r = f.Run();
        bool on0 = true;
        for (size_t i = 0; i < f.ndev; ++i)
            on0 &= f.done_on[i] == 0;
        check(r == 0 && on0, "one_working_device_completes_everything");
    }
    {
        Fake f;
        f.ndev = 8;
        f.broken = {0, 1, 2, 3, 4, 5, 6};
        const unsigned long r = f.Run();
        bool on7 = true;
        for (size_t i = 0; i < f.ndev; ++i)
            on7 &= f.done_on[i] == 7;
        check(r == 0 && on7, "eight_functors_one_working_device");
    }
    {
        Fake f;
        f.broken = {0, 1, 2, 3};
        const unsigned long r = f.Run();
        bool none = true;
        for (size_t i = 0; i < f.ndev; ++i)
            none &= f.done_on[i] == -1 && f.attempts[i] == 1;
        check(r == 4 && none, "all_devices_broken_reports_every_functor");
    }
    {
        Fake f;
        f.fail_alloc = true;
        check(f.Run() == (1ul << 16) && f.runs.empty(), "allocation_failure_code");
    }
    {
        Fake f;
        f.fail_params = true;
        check(f.Run() == (2ul << 16) && f.runs.empty(), "parameter_list_failure_code");
    }
    return bad ? 1 : 0;
}
