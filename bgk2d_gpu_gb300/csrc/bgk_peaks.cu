// bgk_peaks.cu -- measured FP64 instruction rates of the GPU (the roofline of the FP64 kernels).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the DOUBLE and MIXED2 steps are
// bound by the FP64 pipe, not by HBM.  Their roofline is the rate at which the pipe retires
// DFMA, DADD and DMUL instructions, measured here: every thread runs eight independent chains
// of one operation (enough to hide the pipe's latency), on 8 blocks of 256 threads per SM, timed
// with CUDA events around the launch, best of five after one warm-up launch.
#include <cuda_runtime.h>

#include "../../include/bgk2d_gb300.h"

namespace {

constexpr int PK_THREADS = 256, PK_BLOCKS_PER_SM = 8, PK_ITERS = 2048, PK_CHAINS = 8;

template <int OP>
__global__ void __launch_bounds__(PK_THREADS) fp64_chain_kernel(double *out, double b, double c)
{
    double x[PK_CHAINS];
#pragma unroll
    for (int k = 0; k < PK_CHAINS; ++k) x[k] = threadIdx.x * 1e-9 + k;
    for (int i = 0; i < PK_ITERS; ++i) {
#pragma unroll
        for (int k = 0; k < PK_CHAINS; ++k) {
            if (OP == 0) x[k] = fma(x[k], b, c);
            else if (OP == 1) x[k] = __dadd_rn(x[k], c);
            else x[k] = __dmul_rn(x[k], b);
        }
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < PK_CHAINS; ++k) s += x[k];
    out[blockIdx.x * PK_THREADS + threadIdx.x] = s;  // keeps the chains live; one slot per thread
}

template <int OP>
int time_op(int blocks, double *buf, cudaEvent_t e0, cudaEvent_t e1, double *rate)
{
    float best = 1e30f;
    for (int r = 0; r < 6; ++r) {
        if (cudaEventRecord(e0) != cudaSuccess) return BGK_E_CUDA;
        fp64_chain_kernel<OP><<<blocks, PK_THREADS>>>(buf, 0.9999999, 1e-7);
        if (cudaGetLastError() != cudaSuccess || cudaEventRecord(e1) != cudaSuccess ||
            cudaEventSynchronize(e1) != cudaSuccess)
            return BGK_E_CUDA;
        float ms = 0;
        if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return BGK_E_CUDA;
        if (r > 0 && ms < best) best = ms;
    }
    const double ops = (double)blocks * PK_THREADS * PK_ITERS * PK_CHAINS;
    *rate = ops / (best * 1e-3);
    return BGK_OK;
}

}  // namespace

extern "C" int bgk_peak_fp64(int32_t device, double out[3])
{
    if (!out) return BGK_E_INVALID;
    (void)cudaGetLastError();
    int nsm = 0;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        (void)cudaGetLastError();
        return BGK_E_CUDA;
    }
    const int blocks = nsm * PK_BLOCKS_PER_SM;
    double *buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = BGK_OK;
    if (cudaMalloc(&buf, sizeof(double) * blocks * PK_THREADS) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        rc = BGK_E_CUDA;
    if (rc == BGK_OK) rc = time_op<0>(blocks, buf, e0, e1, &out[0]);
    if (rc == BGK_OK) rc = time_op<1>(blocks, buf, e0, e1, &out[1]);
    if (rc == BGK_OK) rc = time_op<2>(blocks, buf, e0, e1, &out[2]);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (buf) cudaFree(buf);
    if (rc != BGK_OK) (void)cudaGetLastError();
    return rc;
}
