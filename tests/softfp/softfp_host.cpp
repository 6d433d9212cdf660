// Host build of bgk_softfp64.h for tests/test_softfp64.py: the integer add and multiply over
// arrays of bit patterns, with a flag per element telling whether the integer path applied.
#include <stdint.h>

#include "../../bgk2d_gpu_gb300/csrc/bgk_softfp64.h"

extern "C" void soft_add_n(const uint64_t *a, const uint64_t *b, uint64_t *r, uint8_t *ok, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) ok[i] = bgk::sfp::add(a[i], b[i], &r[i]) ? 1 : 0;
}

extern "C" void soft_mul_n(const uint64_t *a, const uint64_t *b, uint64_t *r, uint8_t *ok, int64_t n)
{
    for (int64_t i = 0; i < n; ++i) ok[i] = bgk::sfp::mul(a[i], b[i], &r[i]) ? 1 : 0;
}
