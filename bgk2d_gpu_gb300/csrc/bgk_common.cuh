// bgk_common.cuh -- shared device definitions for the GB300 D2Q9 BGK step.
//
// Direction order and vectors follow the reference (SRC/bgk2d.F90:29-39):
//   q : 01      03     05     08     10       12      14      17      19
//   c : (1,-1) (1,1)  (1,0)  (0,1)  (-1,-1)  (-1,1)  (-1,0)  (0,-1)  (0,0)
// Populations are stored as deviations f_q - w_q (the reference's "shifted" form,
// SRC/col_MC.F90:70-75).
//
// HBM layout of one domain ("lattice"): SoA planes.  Plane p holds rows y = 0..ly+1 (ghost
// rows included), each row `pitch` elements long; cell (x, y), x = 0..lx+1, sits at element
//   p * plane_elems + y * pitch + xoff + x,   xoff = VEC - 1,
// so that interior cell x = 1 starts a 16-byte vector (VEC = 16 / sizeof(storage)).
// Ping-pong keeps buffer A in planes 0..8 and buffer B in planes 9..17 (the rest population is
// double-buffered too, so a step never writes its source); AA keeps planes 0..8 only.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace bgk {

constexpr int Q = 9;
constexpr int D01 = 0, D03 = 1, D05 = 2, D08 = 3, D10 = 4, D12 = 5, D14 = 6, D17 = 7, D19 = 8;

__host__ __device__ constexpr int cx_of(int q) {
    return q == D01 ? 1 : q == D03 ? 1 : q == D05 ? 1 : q == D08 ? 0 : q == D10 ? -1 : q == D12 ? -1 : q == D14 ? -1 : 0;
}
__host__ __device__ constexpr int cy_of(int q) {
    return q == D01 ? -1 : q == D03 ? 1 : q == D05 ? 0 : q == D08 ? 1 : q == D10 ? -1 : q == D12 ? 1 : q == D14 ? 0 : q == D17 ? -1 : 0;
}
// opposite direction: 01<->12, 03<->10, 05<->14, 08<->17, 19<->19
__host__ __device__ constexpr int opp_of(int q) {
    return q == D01 ? D12 : q == D03 ? D10 : q == D05 ? D14 : q == D08 ? D17 : q == D10 ? D03 : q == D12 ? D01 : q == D14 ? D05 : q == D17 ? D08 : D19;
}

enum Face { XLO = 0, XHI = 1, YLO = 2, YHI = 3 };
enum FaceKind { FK_WALL = 0, FK_PERIODIC = 1, FK_INFLOW = 2, FK_OUTFLOW_EQ = 3, FK_OUTFLOW_ZG = 4 };

// 16-bit storage keeps (f_q - w_q) * s_q with a power-of-two s_q close to 1/w_q, so the
// scaling is exact and only the 16-bit rounding loses information.
__host__ __device__ constexpr float scale_of(int q) {
    return q == D19 ? 2.0f : ((q == D05 || q == D08 || q == D14 || q == D17) ? 8.0f : 32.0f);
}

// Storage traits: conversion between the stored element and the compute kind K.
template <typename S> struct Store;
template <typename S> struct Is16 { static constexpr bool value = false; };
template <> struct Is16<__half> { static constexpr bool value = true; };
template <> struct Is16<__nv_bfloat16> { static constexpr bool value = true; };

// float -> double without the FP64 pipe (GB300 has little FP64 throughput, and the conversion
// instruction competes with the arithmetic for it).  Exact for every float: zeros and normal
// numbers by moving the fields (exponent rebiased by 1023 - 127 = 896, mantissa into the top
// of the 52-bit field); subnormals, infinities and NaN, which do not occur in a running
// simulation, by the hardware conversion.
__device__ __forceinline__ double widen(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t mag = b & 0x7fffffffu, e = mag >> 23;
    uint64_t d = (uint64_t)(b & 0x80000000u) << 32;
    if (mag != 0u) {
        if (e == 0u || e == 0xffu) return (double)f;
        d |= ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7fffffu) << 29);
    }
    return __longlong_as_double((long long)d);
}
template <typename K> __device__ __forceinline__ K widen_to(float v)
{
    if constexpr (sizeof(K) == 8) return widen(v);
    else return (K)v;
}

// double -> float, rounded to nearest with ties to even, without the FP64 pipe.  Results in the
// normal float range and zeros by integer operations on the fields; a result that would be
// subnormal or overflow, and infinities and NaN, by the hardware conversion.
__device__ __forceinline__ float narrow(double d)
{
    const uint64_t b = (uint64_t)__double_as_longlong(d);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int ed = (int)((b >> 52) & 0x7ffu);
    const uint64_t m = b & 0xfffffffffffffull;
    if (ed == 0 && m == 0) return __uint_as_float(sign);
    const int ef = ed - 896;
    if (ef <= 0 || ef >= 255) return (float)d;
    uint32_t w = ((uint32_t)ef << 23) | (uint32_t)(m >> 29);
    const uint32_t r = (uint32_t)m & 0x1fffffffu;  // the 29 bits dropped
    w += (r > 0x10000000u || (r == 0x10000000u && (w & 1u))) ? 1u : 0u;  // a carry into the exponent is right
    return __uint_as_float(sign | w);
}
template <typename K> __device__ __forceinline__ float narrow_from(K v)
{
    if constexpr (sizeof(K) == 8) return narrow(v);
    else return (float)v;
}

template <> struct Store<float> {
    static constexpr int VEC = 4;
    __device__ __forceinline__ static float raw_get(float v) { return v; }
    __device__ __forceinline__ static float raw_put(float v) { return v; }
    template <typename K, int q> __device__ __forceinline__ static K get(float v) { return widen_to<K>(v); }
    template <typename K, int q> __device__ __forceinline__ static float put(K v) { return narrow_from<K>(v); }
    template <typename K> __device__ __forceinline__ static K getq(float v, int) { return widen_to<K>(v); }
    template <typename K> __device__ __forceinline__ static float putq(K v, int) { return narrow_from<K>(v); }
};
template <> struct Store<double> {
    static constexpr int VEC = 2;
    __device__ __forceinline__ static double raw_get(double v) { return v; }
    __device__ __forceinline__ static double raw_put(double v) { return v; }
    template <typename K, int q> __device__ __forceinline__ static K get(double v) { return (K)v; }
    template <typename K, int q> __device__ __forceinline__ static double put(K v) { return (double)v; }
    template <typename K> __device__ __forceinline__ static K getq(double v, int) { return (K)v; }
    template <typename K> __device__ __forceinline__ static double putq(K v, int) { return (double)v; }
};
// Stochastic rounding FP32 -> 16 bits with the conversion instruction's own random-bits operand
// (`cvt.rs`, Blackwell): each value goes to one of its two neighbouring representable values,
// with the probabilities that make the expected result equal to the input, so updates smaller
// than half an ulp are not lost on average (round-to-nearest would drop them).  Zero stays zero.
// The random bits come from a hash per pair of cells (vector stores) or a hash of the value's own
// bit pattern (lone values).

// per-cell random word: multiplicative hash of the cell index and a value that changes every step
__device__ __forceinline__ uint32_t cell_hash(uint32_t idx, float v)
{
    uint32_t h = idx * 0x9e3779b1u ^ __float_as_uint(v);
    h ^= h >> 15;
    return h * 0x85ebca77u;
}

// random word for a lone value: the well-mixed upper half of a multiplicative hash of its bit
// pattern, in both halves of the word
__device__ __forceinline__ uint32_t lone_bits(float x) { return __byte_perm(__float_as_uint(x) * 0x9e3779b1u, 0u, 0x3232); }

// hash words held by a thread of N cells: one per pair (at least one)
template <int N> __host__ __device__ constexpr int npair() { return N > 1 ? N / 2 : 1; }

// direction q's random word for a pair of cells with hash word h: h rotated by a
// direction-dependent amount
template <int q>
__device__ __forceinline__ uint32_t pair_bits(uint32_t h) { return __funnelshift_l(h, h, 3 * q + 2); }

template <> struct Store<__half> {
    static constexpr int VEC = 8;
    __device__ __forceinline__ static float raw_get(__half v) { return __half2float(v); }
    // lo in the low half, hi in the high half of the result
    __device__ __forceinline__ static uint32_t pack2_rs(float lo, float hi, uint32_t rbits) {
        uint32_t r;
        asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(r) : "f"(hi), "f"(lo), "r"(rbits));
        return r;
    }
    __device__ __forceinline__ static __half raw_put(float v) {
        return __ushort_as_half((unsigned short)(pack2_rs(v, 0.0f, lone_bits(v)) & 0xffffu));
    }
    template <typename K, int q> __device__ __forceinline__ static K get(__half v) {
        return (K)(__half2float(v) * (1.0f / scale_of(q)));
    }
    template <typename K> __device__ __forceinline__ static K getq(__half v, int q) {
        return (K)(__half2float(v) * (1.0f / scale_of(q)));
    }
    template <typename K> __device__ __forceinline__ static __half putq(K v, int q) {
        return raw_put((float)v * scale_of(q));
    }
    template <typename K, int q> __device__ __forceinline__ static __half put(K v) { return putq<K>(v, q); }
};
template <> struct Store<__nv_bfloat16> {
    static constexpr int VEC = 8;
    __device__ __forceinline__ static float raw_get(__nv_bfloat16 v) { return __bfloat162float(v); }
    __device__ __forceinline__ static uint32_t pack2_rs(float lo, float hi, uint32_t rbits) {
        uint32_t r;
        asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(r) : "f"(hi), "f"(lo), "r"(rbits));
        return r;
    }
    __device__ __forceinline__ static __nv_bfloat16 raw_put(float v) {
        return __ushort_as_bfloat16((unsigned short)(pack2_rs(v, 0.0f, lone_bits(v)) & 0xffffu));
    }
    template <typename K, int q> __device__ __forceinline__ static K get(__nv_bfloat16 v) {
        return (K)(__bfloat162float(v) * (1.0f / scale_of(q)));
    }
    template <typename K> __device__ __forceinline__ static K getq(__nv_bfloat16 v, int q) {
        return (K)(__bfloat162float(v) * (1.0f / scale_of(q)));
    }
    template <typename K> __device__ __forceinline__ static __nv_bfloat16 putq(K v, int q) {
        return raw_put((float)v * scale_of(q));
    }
    template <typename K, int q> __device__ __forceinline__ static __nv_bfloat16 put(K v) { return putq<K>(v, q); }
};

// One domain as the kernels see it.  Scalars of the compute kind are kept in double and
// cast in the kernel (exact for both kinds, since they were computed in that kind).
struct Lattice {
    void *planes;            // base of all planes (storage elements)
    int64_t plane_elems;     // elements per plane (rows * pitch, padded)
    int32_t pitch;           // elements per row
    int32_t lx, ly;          // interior size
    int32_t nvec;            // ceil(lx / VEC)
    int32_t scheme;          // 0 ping-pong, 1 AA
    int32_t faces[4];        // FaceKind per face
    int32_t corner_x;        // 1: at a corner the x-face rule wins over the y-face rule (-DTRICK1)
    int32_t noshift;         // 1: planes hold the populations f, not the deviations f - w (-DNOSHIFT)
    int32_t inflow_y0;       // an x_lo inflow face supplies rows >= inflow_y0; below it bounces back
    int32_t step_x, step_y;  // backward-facing step corner (stepx, stepy), 0 without a step
    void *step_aux;          // AA with a step: 10 storage elements, the five bounced-back inputs of
                             // step_bounce (0-4) and the five pushes their neighbours hold back (5-9)
    double wt[4][9];         // wall term added to the bounced population, per face and direction
    double omega, fgrad;     // relaxation rate and body-force gradient (compute kind)
    int32_t forced;          // 1 when the x body force fgrad*rho is applied (CHANNEL)
    int32_t les;             // 1: Smagorinsky eddy viscosity in the collision (-DLES)
    double cte_s;            // Smagorinsky constant cteS (compute kind)
    float omega_f, fgrad_f, cte_s_f;  // the same three in single precision (exact for FP32 compute),
                                      // so that FP32 kernels convert nothing on the FP64 pipe
    const double *inflow;    // [3][ly+2] equilibrium deviations of 01,03,05 at the x_lo inflow
    const uint32_t *mask;    // obstacle bits, row y (0..ly+1) at mask + y*mask_pitch, bit x
    int32_t mask_pitch;      // 32-bit words per mask row
    int32_t ob_x0, ob_x1, ob_y0, ob_y1;  // cells whose pull may touch an obstacle
    uint32_t *status;        // device word set by a kernel whose bounded wait ran out (0: fine)
    int32_t inject_stall;    // test hook (BGK_FAULT_INJECT_STALL=1): staged copies never complete
    int32_t pf_ahead;        // ping-pong kernels: L2 prefetch of the block this many places ahead (0: off)
};

template <typename S> __host__ __device__ constexpr int vec_of() { return 16 / (int)sizeof(S); }

// Row of tiles processed by grid row b of gy: the last row of the domain (whose cells take the
// slow boundary-rule path) runs second instead of last, so its blocks overlap with the bulk of
// the launch instead of forming its tail.  A bijection of 0..gy-1.
__device__ __forceinline__ int tile_row(int b, int gy)
{
    return (gy < 2 || b == 0) ? b : (b == 1 ? gy - 1 : b - 1);
}

// relaxation scalars of a lattice in the compute kind K
template <typename K> __device__ __forceinline__ K lat_omega(const Lattice &L);
template <> __device__ __forceinline__ float lat_omega<float>(const Lattice &L) { return L.omega_f; }
template <> __device__ __forceinline__ double lat_omega<double>(const Lattice &L) { return L.omega; }
template <typename K> __device__ __forceinline__ K lat_fgrad(const Lattice &L);
template <> __device__ __forceinline__ float lat_fgrad<float>(const Lattice &L) { return L.fgrad_f; }
template <> __device__ __forceinline__ double lat_fgrad<double>(const Lattice &L) { return L.fgrad; }
template <typename K> __device__ __forceinline__ K lat_cte_s(const Lattice &L);
template <> __device__ __forceinline__ float lat_cte_s<float>(const Lattice &L) { return L.cte_s_f; }
template <> __device__ __forceinline__ double lat_cte_s<double>(const Lattice &L) { return L.cte_s; }

template <typename S>
__device__ __forceinline__ int64_t cell_index(const Lattice &L, int x, int y) {
    return (int64_t)y * L.pitch + (vec_of<S>() - 1) + x;
}

__device__ __forceinline__ bool obs_bit(const Lattice &L, int x, int y) {
    uint32_t w = __ldg(L.mask + (int64_t)y * L.mask_pitch + (x >> 5));
    return (w >> (x & 31)) & 1u;
}

// Backward-facing step (SRC/bcond.step.F90:207-255).  Its two face loops run one cell past the
// solid block (i = 1..stepx at row stepy-1, j = 1..stepy at column stepx-1, the block being
// x < stepx, y < stepy), so they also overwrite populations at fluid positions; after both loops,
// in their order, four inputs of the corner cell (stepx, stepy) and one of (stepx-1, stepy) are
// bounce-backs of the cell's own opposite population: 01, 05, 08 and 12 of the corner, 12 of its
// left neighbour.  (The D01 input of (stepx, stepy-1) is overwritten twice and ends with its
// normal value.)  Returns whether input q of cell (x, y) is such a bounce-back.
__device__ __forceinline__ bool step_bounce(const Lattice &L, int x, int y, int q)
{
    if (L.step_x <= 0 || y != L.step_y) return false;
    if (x == L.step_x) return q == D01 || q == D05 || q == D08 || q == D12;
    return x == L.step_x - 1 && q == D12;
}

// index 0..4 of a step_bounce input (x, y, q) among the five (L.step_aux)
__device__ __forceinline__ int step_slot(const Lattice &L, int x, int q)
{
    if (x != L.step_x) return 4;
    return q == D01 ? 0 : q == D05 ? 1 : q == D08 ? 2 : 3;
}

}  // namespace bgk
