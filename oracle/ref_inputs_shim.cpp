/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * C entry points around the reference's own input generators,
 * InitializePointChargeArray and InitializeFieldLineArray (grid mode)
 * (ElectroMag/src/"Electromag utils.h":29-111), and around the C library's
 * srand()/rand() that the former draws from.  oracle/build_ref.sh compiles
 * this file against the unmodified reference headers into
 * oracle/_ref/libemref_inputs.so; tests/golden/make_inputs_golden.py loads
 * it to produce the committed input fixtures.
 */
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <thread>

#include "X-Compat/HPC Timing.h"
#include "CPU Implement.h"
#include "Electromag utils.h"

namespace {

template <class T> void charges(T *out, size_t p)
{
    Array<electro::pointCharge<T> > q(p, 256);
    InitializePointChargeArray(q, p, false); // srand(1), as without --randseed
    std::memcpy(out, q.GetDataPointer(), p * 4 * sizeof(T));
    q.Free();
}

template <class T> void grid(T *x, T *y, T *z, size_t w, size_t h, size_t d)
{
    const size_t n = w * h * d;
    Vector3<Array<T> > a;
    a.AlignAlloc(n);
    InitializeFieldLineArray(a, n, w, h, d, false);
    Vector3<T *> p = a.GetDataPointers();
    std::memcpy(x, p.x, n * sizeof(T));
    std::memcpy(y, p.y, n * sizeof(T));
    std::memcpy(z, p.z, n * sizeof(T));
    a.Free();
}

} // namespace

extern "C" void ref_init_charges_f32(float *out, size_t p) { charges<float>(out, p); }
extern "C" void ref_init_charges_f64(double *out, size_t p) { charges<double>(out, p); }
extern "C" void ref_init_grid_f32(float *x, float *y, float *z, size_t w, size_t h, size_t d)
{
    grid<float>(x, y, z, w, h, d);
}
extern "C" void ref_init_grid_f64(double *x, double *y, double *z, size_t w, size_t h,
                                  size_t d)
{
    grid<double>(x, y, z, w, h, d);
}
extern "C" void ref_libc_rand(unsigned seed, int *out, size_t count)
{
    srand(seed);
    for (size_t i = 0; i < count; ++i)
        out[i] = rand();
}
