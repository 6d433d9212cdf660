// bgk_noalloc.cu -- diagno sums on caller-owned device arrays, without any allocation.
//
// For callers that cannot let this library allocate device memory: for example a Fortran
// OpenACC or OpenMP-offload build whose populations live in data regions owned by the
// compiler's runtime, or a program running under a fixed device-memory budget.  Such a caller
// passes device pointers to its own nine population arrays (reference layout: column-major
// (0:lx+1, 0:ly+1) planes with leading dimension ld, direction order 01,03,05,08,10,12,14,17,19,
// deviations f - w) and a host array for the four means.
//
// The FP64 partial sums go to a fixed static device array instead of allocated scratch.  Every
// GPU that loads the library holds that array until the process exits.  Each call overwrites
// the partials it reads, so nothing has to be cleared between calls.  Calls from different host
// threads share the array: one process-wide mutex covers each call from its launches to the
// synchronous read of the totals, so calls never overlap on the GPU.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/bgk2d_gb300.h"

// fixed device scratch of every call: 4 partial sums per chunk, then the four totals (128 KiB)
static __device__ __align__(256) double g_diag_scratch[4 * 4096 + 4];

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CHUNK = 4096;                      // cells reduced by one block
constexpr int NA_MAX_CHUNKS = 4096;                 // at most 4096 * 4096 = 16,777,216 cells

struct Planes {
    const void *p[9];
};

// per-cell moments as SRC/diagno.F90:82-93, in the storage kind T
template <typename T>
__global__ void __launch_bounds__(NA_THREADS) noalloc_diagno_kernel(Planes P, long long ld, int lx, int ly,
                                                                    double *scratch)
{
    double acc[4] = {0, 0, 0, 0};
    const long long n = (long long)lx * ly;
    const long long c0 = (long long)blockIdx.x * NA_CHUNK;
    for (int k = threadIdx.x; k < NA_CHUNK; k += NA_THREADS) {
        const long long c = c0 + k;
        if (c >= n) break;
        const int i = (int)(c % lx) + 1, j = (int)(c / lx) + 1;
        const long long e = (long long)i + (long long)j * ld;
        T a[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) a[q] = reinterpret_cast<const T *>(P.p[q])[e];
        const T rho = ((((a[0] + a[1]) + a[4]) + a[5]) + (((a[2] + a[3]) + a[6]) + a[7]) + a[8]) + (T)1;
        const T rinv = (T)1 / rho;
        const T xj = (((a[1] - a[5]) + (a[0] - a[4])) + (a[2] - a[6])) * rinv;
        const T yj = (((a[1] - a[0]) + (a[5] - a[4])) + (a[3] - a[7])) * rinv;
        acc[0] += (double)xj;
        acc[1] += (double)yj;
        acc[2] += (double)rho;
        acc[3] += (double)(xj * xj + yj * yj);
    }
    __shared__ double sh[NA_THREADS / 32][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[q] += __shfl_down_sync(0xffffffffu, acc[q], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) sh[threadIdx.x >> 5][q] = acc[q];
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0;
        for (int w = 0; w < NA_THREADS / 32; ++w) s += sh[w][threadIdx.x];
        scratch[4 * blockIdx.x + threadIdx.x] = s;  // every slot this call reads is written here
    }
}

// fixed-order sum of the partials of nb chunks into the four total slots
__global__ void noalloc_total_kernel(double *scratch, int nb)
{
    if (threadIdx.x < 4) {
        double s = 0;
        for (int b = 0; b < nb; ++b) s += scratch[4 * b + threadIdx.x];
        scratch[4 * NA_MAX_CHUNKS + threadIdx.x] = s;
    }
}

std::mutex g_mu;

// with g_mu held and the caller's device current: the device address of the static array in
// the current context.  Looked up on every call (a cheap runtime query next to the synchronous
// copy of the totals), so a context created after a cudaDeviceReset, or another context made
// current by the caller's runtime, gets its own module's address rather than a stale one.
int scratch_for_current_device(double **out)
{
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_diag_scratch) != cudaSuccess) return BGK_E_CUDA;
    *out = static_cast<double *>(p);
    return BGK_OK;
}

}  // namespace

extern "C" int bgk_diagno_noalloc(const void *const pops[9], int64_t ld, int32_t lx, int32_t ly, int32_t storage,
                                  double out[4])
{
    if (!pops || !out || lx < 1 || ly < 1 || ld < (int64_t)lx + 2) return BGK_E_INVALID;
    if (storage != BGK_STORE_F32 && storage != BGK_STORE_F64) return BGK_E_INVALID;
    const long long cells = (long long)lx * ly;
    const long long chunks = (cells + NA_CHUNK - 1) / NA_CHUNK;
    if (chunks > NA_MAX_CHUNKS) return BGK_E_TOOLARGE;
    for (int q = 0; q < 9; ++q)
        if (!pops[q]) return BGK_E_INVALID;
    std::lock_guard<std::mutex> g(g_mu);  // held until the totals are back on the host
    (void)cudaGetLastError();  // an error left pending by an earlier failed call is not ours
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != BGK_OK) return rc;
    Planes P;
    for (int q = 0; q < 9; ++q) P.p[q] = pops[q];
    if (storage == BGK_STORE_F32)
        noalloc_diagno_kernel<float><<<(unsigned)chunks, NA_THREADS>>>(P, (long long)ld, lx, ly, scratch);
    else
        noalloc_diagno_kernel<double><<<(unsigned)chunks, NA_THREADS>>>(P, (long long)ld, lx, ly, scratch);
    noalloc_total_kernel<<<1, 32>>>(scratch, (int)chunks);
    if (cudaGetLastError() != cudaSuccess) return BGK_E_CUDA;
    double s[4];
    if (cudaMemcpy(s, scratch + 4 * NA_MAX_CHUNKS, sizeof(s), cudaMemcpyDeviceToHost) != cudaSuccess) return BGK_E_CUDA;
    for (int q = 0; q < 4; ++q) out[q] = (s[q] / (double)lx) / (double)ly;  // SRC/diagno.F90:98-101
    for (int q = 0; q < 4; ++q)
        if (!(s[q] == s[q]) || s[q] - s[q] != 0.0) return BGK_E_NUMERIC;
    return BGK_OK;
}
