// Device build of bgk_softfp64.h for tests/test_softfp64.py: each thread computes the integer sum
// and product of its pair and the hardware DADD and DMUL of the same pair (__dadd_rn, __dmul_rn).
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../bgk2d_gpu_gb300/csrc/bgk_softfp64.h"

__global__ void softfp_kernel(const uint64_t *a, const uint64_t *b, uint64_t *out, uint8_t *ok, int64_t n)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t s = 0, p = 0;
    const bool oks = bgk::sfp::add(a[i], b[i], &s), okp = bgk::sfp::mul(a[i], b[i], &p);
    const double x = __longlong_as_double((long long)a[i]), y = __longlong_as_double((long long)b[i]);
    out[4 * i + 0] = s;
    out[4 * i + 1] = (uint64_t)__double_as_longlong(__dadd_rn(x, y));
    out[4 * i + 2] = p;
    out[4 * i + 3] = (uint64_t)__double_as_longlong(__dmul_rn(x, y));
    ok[2 * i] = oks;
    ok[2 * i + 1] = okp;
}

// host arrays in, host arrays out (out: 4 words per pair, ok: 2 flags per pair); 0 on success
extern "C" int softfp_device_run(const uint64_t *a, const uint64_t *b, uint64_t *out, uint8_t *ok, int64_t n)
{
    uint64_t *da = nullptr, *db = nullptr, *dout = nullptr;
    uint8_t *dok = nullptr;
    int rc = 0;
    if (cudaMalloc(&da, n * 8) || cudaMalloc(&db, n * 8) || cudaMalloc(&dout, n * 32) || cudaMalloc(&dok, n * 2)) rc = 1;
    if (!rc && (cudaMemcpy(da, a, n * 8, cudaMemcpyHostToDevice) || cudaMemcpy(db, b, n * 8, cudaMemcpyHostToDevice))) rc = 2;
    if (!rc) {
        softfp_kernel<<<(unsigned)((n + 255) / 256), 256>>>(da, db, dout, dok, n);
        if (cudaGetLastError() || cudaDeviceSynchronize()) rc = 3;
    }
    if (!rc && (cudaMemcpy(out, dout, n * 32, cudaMemcpyDeviceToHost) || cudaMemcpy(ok, dok, n * 2, cudaMemcpyDeviceToHost))) rc = 4;
    cudaFree(da);
    cudaFree(db);
    cudaFree(dout);
    cudaFree(dok);
    return rc;
}
