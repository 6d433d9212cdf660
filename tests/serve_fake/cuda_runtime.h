/* Host-only stand-in for the few CUDA runtime calls of bgk_serve.cpp, so that the serving
 * scheduler can be compiled and exercised on a machine without a GPU (tests/test_serve_host.py).
 * It reports one device with 80 GiB, of which g_fake_free_bytes (64 GiB unless a test sets it
 * through fake_set_free_bytes) are free. */
#pragma once
#include <stddef.h>

typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount = 16 };

static inline cudaError_t cudaSetDevice(int device) { return device == 0 ? cudaSuccess : 101; }
static inline cudaError_t cudaGetLastError(void) { return cudaSuccess; }
extern size_t g_fake_free_bytes;
static inline cudaError_t cudaMemGetInfo(size_t *free_b, size_t *total_b)
{
    *free_b = g_fake_free_bytes;
    *total_b = (size_t)80 << 30;
    return cudaSuccess;
}
static inline cudaError_t cudaDeviceGetAttribute(int *value, enum cudaDeviceAttr, int)
{
    *value = 152;
    return cudaSuccess;
}
