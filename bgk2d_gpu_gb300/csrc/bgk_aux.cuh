// bgk_aux.cuh -- state access, host-layout conversion and FP64 reductions (templated bodies).
#pragma once

#include <type_traits>

#include "bgk_kernels.cuh"
#include "bgk_table.h"

namespace bgk {

// Post-collision value of direction q at interior cell (x, y), i.e. the reference's a_q(x, y)
// after `collision` (SRC/col_MC.F90:311-341 swap included), for every scheme and phase.
template <typename S, typename K, bool HAS_OBS>
__device__ __forceinline__ K post_value(const Lattice &L, int cur, int phase, int q, int x, int y)
{
    const S *base = reinterpret_cast<const S *>(L.planes);
    const int64_t pe = L.plane_elems;
    if (L.scheme == 0) return ldq<S, K>(base + ((cur ? 9 : 0) + q) * pe, cell_index<S>(L, x, y), q);
    if (phase == 0 || q == D19) return ldq<S, K>(base + opp_of(q) * pe, cell_index<S>(L, x, y), q);
    // phase 1: the value was pushed to x + c_q (or kept where the push rule put it)
    int tx = x + cx_of(q), ty = y + cy_of(q);
    if (ty < 1 || ty > L.ly) {
        if (L.faces[ty < 1 ? YLO : YHI] != FK_PERIODIC) return ldq<S, K>(base + q * pe, cell_index<S>(L, tx, ty), q);
        ty = ty < 1 ? L.ly : 1;
    }
    if (tx < 1 || tx > L.lx) {
        if (L.faces[tx < 1 ? XLO : XHI] != FK_PERIODIC) return ldq<S, K>(base + q * pe, cell_index<S>(L, tx, ty), q);
        tx = tx < 1 ? L.lx : 1;
    }
    if (HAS_OBS) {
        // a push a backward-facing step's corner holds back (aa_push_rule)
        if (L.step_aux && step_bounce(L, tx, ty, q))
            return Store<S>::template getq<K>(reinterpret_cast<const S *>(L.step_aux)[5 + step_slot(L, tx, q)], q);
        if (obs_bit(L, tx, ty)) return ldq<S, K>(base + opp_of(q) * pe, cell_index<S>(L, x, y), q);
    }
    return ldq<S, K>(base + q * pe, cell_index<S>(L, tx, ty), q);
}

// host-kind staging plane (lx+2) x (ly+2), i fastest, -> device storage
template <typename S, typename H>
__global__ void scatter_plane_kernel(Lattice L, int cur, int q, const H *__restrict__ stage, int64_t ld)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x > L.lx + 1) return;
    S *base = reinterpret_cast<S *>(L.planes);
    const int64_t pe = L.plane_elems;
    int p;
    if (L.scheme == 0) p = (cur ? 9 : 0) + q;
    else p = opp_of(q);
    const H v = stage[(int64_t)y * ld + x];
    base[p * pe + cell_index<S>(L, x, y)] = Store<S>::template putq<double>((double)v, q);
}

// Pressure-corrected Taylor-Green start (BGK_INIT_TGV), computed on the device in FP64:
// u = U0 sin(kx x) cos(ky y), v = -U0 cos(kx x) sin(ky y),
// rho = 1 - 3 U0^2/4 (cos 2kx x + cos 2ky y), x = i - 1/2, y = j - 1/2, f - w = feq - w
// (f = feq when the populations are stored whole, L.noshift).
template <typename S>
__global__ void init_tgv_kernel(Lattice L, double u0)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x > L.lx + 1) return;
    S *base = reinterpret_cast<S *>(L.planes);
    const int64_t pe = L.plane_elems;
    const double kx = 2.0 * 3.14159265358979323846 / L.lx, ky = 2.0 * 3.14159265358979323846 / L.ly;
    const double xx = x - 0.5, yy = y - 0.5;
    double sx, cx, sy, cy;
    sincos(kx * xx, &sx, &cx);
    sincos(ky * yy, &sy, &cy);
    const double u = u0 * sx * cy, v = -u0 * cx * sy;
    const double rho = 1.0 - 0.75 * u0 * u0 * ((2.0 * cx * cx - 1.0) + (2.0 * cy * cy - 1.0));
    const double usq = u * u + v * v;
    const double w[9] = {1. / 36, 1. / 36, 1. / 9, 1. / 9, 1. / 36, 1. / 36, 1. / 9, 1. / 9, 4. / 9};
    const int64_t i = cell_index<S>(L, x, y);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const double cu = cx_of(q) * u + cy_of(q) * v;
        const double f = w[q] * rho * (1.0 + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq) - (L.noshift ? 0.0 : w[q]);
        const int p = L.scheme == 0 ? q : opp_of(q);
        base[p * pe + i] = Store<S>::template putq<double>(f, q);
    }
}

// device storage -> host-kind staging plane; ghost entries are written as zero
template <typename S, typename K, typename H, bool HAS_OBS>
__global__ void gather_plane_kernel(Lattice L, int cur, int phase, int q, H *__restrict__ stage, int64_t ld)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x > L.lx + 1) return;
    H v = (H)0;
    if (x >= 1 && x <= L.lx && y >= 1 && y <= L.ly) v = (H)post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
    stage[(int64_t)y * ld + x] = v;
}

// Rows ya..yb of the nine mapped host planes <-> state buffer cur, moved by warp wid of nw.
// Work unit: 32 consecutive host elements of one plane, the first of them on a 128-byte boundary
// of the host address space (units run across row ends when ld = lx + 2), so that each warp
// access covers whole lines of the host link.  A warp keeps XFER_UNROLL units in flight.
// Callers keep (yb - ya + 1) * ld below 2^26, so the unit arithmetic fits 32 bits.
// UP: host -> device, the conversion of scatter_plane_kernel; !UP: device -> host, the values of
// gather_plane_kernel (ghost entries written as zero).
constexpr int XFER_UNROLL = 4;

template <typename S, typename K, typename H, bool HAS_OBS, bool UP>
__device__ __forceinline__ void xfer_rows(const Lattice &L, const int cur, const int phase, const HostPlanes &hp,
                                          const int ya, const int yb, const int wid, const int nw)
{
    const int64_t ld = hp.ld;
    const uint32_t n = (uint32_t)((int64_t)(yb - ya + 1) * ld);
    const uint32_t ld32 = (uint32_t)ld;
    const uint32_t umax = (n + 63u) / 32u;  // units of any plane: its first unit starts < 32 elements early
    const uint32_t total = 9u * umax;
    const int lane = threadIdx.x & 31;
    S *base = reinterpret_cast<S *>(L.planes);
    const int64_t pe = L.plane_elems;
    for (uint32_t u0 = (uint32_t)wid; u0 < total; u0 += (uint32_t)nw * XFER_UNROLL) {
        H v[XFER_UNROLL];
        H *hptr[XFER_UNROLL];
        int qs[XFER_UNROLL], xs[XFER_UNROLL], ys[XFER_UNROLL];
        bool ok[XFER_UNROLL];
#pragma unroll
        for (int i = 0; i < XFER_UNROLL; ++i) {
            const uint32_t uu = u0 + (uint32_t)i * (uint32_t)nw;
            ok[i] = false;
            qs[i] = 0; xs[i] = 0; ys[i] = 0;
            hptr[i] = nullptr;
            if (uu < total) {
                const int q = (int)(uu / umax);
                const uint32_t u = uu - (uint32_t)q * umax;
                H *row = reinterpret_cast<H *>(hp.p[q]) + (int64_t)ya * ld;
                const uint32_t sh = (uint32_t)(((uintptr_t)row & 127u) / sizeof(H));
                const int64_t e = (int64_t)u * 32 + lane - (int64_t)sh;
                if (e >= 0 && e < (int64_t)n) {
                    const uint32_t r = (uint32_t)e / ld32;
                    const int x = (int)((uint32_t)e - r * ld32);
                    if (x <= L.lx + 1) {
                        ok[i] = true;
                        qs[i] = q; xs[i] = x; ys[i] = ya + (int)r;
                        hptr[i] = row + e;
                    }
                }
            }
        }
        if constexpr (UP) {
#pragma unroll
            for (int i = 0; i < XFER_UNROLL; ++i)
                if (ok[i]) v[i] = *hptr[i];
#pragma unroll
            for (int i = 0; i < XFER_UNROLL; ++i)
                if (ok[i]) {
                    const int p = L.scheme == 0 ? (cur ? 9 : 0) + qs[i] : opp_of(qs[i]);
                    base[p * pe + cell_index<S>(L, xs[i], ys[i])] = Store<S>::template putq<double>((double)v[i], qs[i]);
                }
        } else {
#pragma unroll
            for (int i = 0; i < XFER_UNROLL; ++i) {
                v[i] = (H)0;
                if (ok[i] && xs[i] >= 1 && xs[i] <= L.lx && ys[i] >= 1 && ys[i] <= L.ly)
                    v[i] = (H)post_value<S, K, HAS_OBS>(L, cur, phase, qs[i], xs[i], ys[i]);
            }
#pragma unroll
            for (int i = 0; i < XFER_UNROLL; ++i)
                if (ok[i]) *hptr[i] = v[i];
        }
    }
}

// whole-lattice transfer of rows ya..yb (one launch per chunk of rows), 8 warps per block
template <typename S, typename K, typename H, bool HAS_OBS, bool UP>
__global__ void __launch_bounds__(256) xfer_kernel(const Lattice L, const int cur, const int phase, const HostPlanes hp,
                                                   const int ya, const int yb)
{
    xfer_rows<S, K, H, HAS_OBS, UP>(L, cur, phase, hp, ya, yb, (int)(blockIdx.x * 8 + (threadIdx.x >> 5)),
                                    (int)(gridDim.x * 8));
}

// host rows of band b (interior rows b*R+1 .. (b+1)*R, and the ghost row beside the first and
// the last band)
__device__ __forceinline__ void band_rows(const Lattice &L, const WaveArgs &a, int b, int &ya, int &yb)
{
    ya = b == 0 ? 0 : 1 + b * a.band_rows;
    yb = b == a.nbands - 1 ? L.ly + 1 : (b + 1) * a.band_rows;
}

// One wave of bgk_advance_host (WaveArgs): grid rows 0.. carry the upload of band up_band, then
// the download of band down_band (xfer_rows grid rows each, scheduled first so that the host
// link is busy from the start of the wave), then band_rows grid rows per step item.  The step
// items are pp_kernel's tiles (128 x 1 threads, N cells per thread) of one row each, with the
// handle's collision variant CV.
template <typename S, typename K, typename H, bool HAS_OBS, int N, int CV = 0>
__global__ void __launch_bounds__(128, (N * sizeof(S) <= 8 || (sizeof(S) == 4 && N == 4)) ? 8 : (sizeof(S) == 2 ? 4 : 1))
    wave_kernel(const Lattice L, const WaveArgs a)
{
    int by = blockIdx.y;
    const int nw = a.xfer_rows * (int)gridDim.x * 4;
    if (a.up_band >= 0) {
        if (by < a.xfer_rows) {
            int ya, yb;
            band_rows(L, a, a.up_band, ya, yb);
            xfer_rows<S, K, H, HAS_OBS, true>(L, a.cur0, 0, a.in, ya, yb,
                                              (by * (int)gridDim.x + (int)blockIdx.x) * 4 + (int)(threadIdx.x >> 5), nw);
            return;
        }
        by -= a.xfer_rows;
    }
    if (a.down_band >= 0) {
        if (by < a.xfer_rows) {
            int ya, yb;
            band_rows(L, a, a.down_band, ya, yb);
            xfer_rows<S, K, H, HAS_OBS, false>(L, (a.cur0 + a.nsteps) & 1, 0, a.out, ya, yb,
                                               (by * (int)gridDim.x + (int)blockIdx.x) * 4 + (int)(threadIdx.x >> 5), nw);
            return;
        }
        by -= a.xfer_rows;
    }
    const int k = a.k_lo + by / a.band_rows;
    const int y = (a.wave - 2 * k) * a.band_rows + by % a.band_rows + 1;
    if (y > L.ly) return;
    pp_tile<S, K, 128, 1, HAS_OBS, N, CV>(L, (int)blockIdx.x, y - 1, (a.cur0 + k - 1) & 1);
}

// AA phase-0 outflow ghosts at x = lx+1, from cell (lx, y)'s stored post-collision values
template <typename S, typename K>
__global__ void aa_fill_outflow_kernel(Lattice L)
{
    const int y = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (y > L.ly) return;
    S *base = reinterpret_cast<S *>(L.planes);
    const int64_t pe = L.plane_elems;
    const int64_t i = cell_index<S>(L, L.lx, y);
    K g[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) g[q] = ldq<S, K>(base + opp_of(q) * pe, i, q);
    aa_outflow_ghost<S, K>(L, base, y, g);
}

// moments with the reference's per-cell arithmetic (SRC/diagno.F90:82-93); cte1 = 1, or 0 for
// populations stored whole (SRC/diagno.F90:42-46)
template <typename K>
__device__ __forceinline__ void moments(const K (&a)[9], K &rho, K &xj, K &yj, bool noshift)
{
    const K cte1 = noshift ? (K)0 : (K)1, uno = (K)1;
    rho = ((((a[0] + a[1]) + a[4]) + a[5]) + (((a[2] + a[3]) + a[6]) + a[7]) + a[8]) + cte1;
    K rhoinv = uno / rho;
    xj = (((a[1] - a[5]) + (a[0] - a[4])) + (a[2] - a[6])) * rhoinv;
    yj = (((a[1] - a[0]) + (a[5] - a[4])) + (a[3] - a[7])) * rhoinv;
}

template <int NT>
__device__ __forceinline__ void block_sum4(double (&v)[4], double *out)
{
    __shared__ double sh[NT / 32][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], o);
    }
    const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
    if (ln == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) sh[w][i] = v[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[4] = {0, 0, 0, 0};
        for (int k = 0; k < NT / 32; ++k)
#pragma unroll
            for (int i = 0; i < 4; ++i) s[i] += sh[k][i];
#pragma unroll
        for (int i = 0; i < 4; ++i) out[i] = s[i];
    }
}

constexpr int RED_NT = 256;

// diagno: partial sums of rho, u, v, |u|^2 (FP64) per block
// exact widening to FP64 for the FP64 sums; from FP32 by integer operations (widen), since the
// FP64 pipe bounds these reductions on GB300
__device__ __forceinline__ double to_f64(float v) { return widen(v); }
__device__ __forceinline__ double to_f64(double v) { return v; }

template <typename S, typename K, bool HAS_OBS>
__global__ void __launch_bounds__(RED_NT) diagno_kernel(Lattice L, int cur, int phase, int fluid_only, double *partial)
{
    double acc[4] = {0, 0, 0, 0};
    const int64_t n = (int64_t)L.lx * L.ly;
    for (int64_t c = (int64_t)blockIdx.x * RED_NT + threadIdx.x; c < n; c += (int64_t)gridDim.x * RED_NT) {
        const int x = (int)(c % L.lx) + 1, y = (int)(c / L.lx) + 1;
        if (HAS_OBS && fluid_only) {
            if (obs_bit(L, x, y)) continue;
        }
        K a[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) a[q] = post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
        K rho, xj, yj;
        moments<K>(a, rho, xj, yj, L.noshift != 0);
        acc[0] += to_f64(xj);
        acc[1] += to_f64(yj);
        acc[2] += to_f64(rho);
        acc[3] += to_f64(xj * xj + yj * yj);
    }
    block_sum4<RED_NT>(acc, partial + 4 * blockIdx.x);
}

// diagno in the reference's own arithmetic (SRC/diagno.F90:63-101): sums in the compute kind K,
// in the serial j-outer / i-inner order, then (sum / l) / m.  The per-cell moments of a chunk of
// 1024 cells are computed in parallel; one thread adds them in order.  One block.
template <typename S, typename K, bool HAS_OBS>
__global__ void __launch_bounds__(1024) diagno_seq_kernel(Lattice L, int cur, int phase, double *out)
{
    __shared__ K sh[4][1024];
    const int64_t n = (int64_t)L.lx * L.ly;
    K rtot = (K)0, xtot = (K)0, ytot = (K)0, stot = (K)0;
    for (int64_t c0 = 0; c0 < n; c0 += 1024) {
        const int64_t c = c0 + threadIdx.x;
        if (c < n) {
            const int x = (int)(c % L.lx) + 1, y = (int)(c / L.lx) + 1;
            K a[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) a[q] = post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
            K rho, xj, yj;
            moments<K>(a, rho, xj, yj, L.noshift != 0);
            sh[0][threadIdx.x] = rho;
            sh[1][threadIdx.x] = xj;
            sh[2][threadIdx.x] = yj;
            sh[3][threadIdx.x] = xj * xj + yj * yj;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const int cnt = (int)min((int64_t)1024, n - c0);
            for (int k = 0; k < cnt; ++k) {
                rtot = rtot + sh[0][k];
                xtot = xtot + sh[1][k];
                ytot = ytot + sh[2][k];
                stot = stot + sh[3][k];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const K fl = (K)(float)L.lx, fm = (K)(float)L.ly;  // float(l), float(m)
        out[0] = (double)((xtot / fl) / fm);
        out[1] = (double)((ytot / fl) / fm);
        out[2] = (double)((rtot / fl) / fm);
        out[3] = (double)((stot / fl) / fm);
    }
}

// residual: sum |u - u_prev|^2 and |u|^2 (FP64); the snapshot is refreshed
template <typename S, typename K, bool HAS_OBS>
__global__ void __launch_bounds__(RED_NT) residual_kernel(Lattice L, int cur, int phase, double *uprev, double *vprev,
                                                          double *partial)
{
    double acc[4] = {0, 0, 0, 0};
    const int64_t n = (int64_t)L.lx * L.ly;
    for (int64_t c = (int64_t)blockIdx.x * RED_NT + threadIdx.x; c < n; c += (int64_t)gridDim.x * RED_NT) {
        const int x = (int)(c % L.lx) + 1, y = (int)(c / L.lx) + 1;
        if (HAS_OBS) {
            if (obs_bit(L, x, y)) continue;
        }
        K a[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) a[q] = post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
        K rho, xj, yj;
        moments<K>(a, rho, xj, yj, L.noshift != 0);
        const double u = (double)xj, v = (double)yj;
        const double du = u - uprev[c], dv = v - vprev[c];
        acc[0] += du * du + dv * dv;
        acc[1] += u * u + v * v;
        acc[2] += (isfinite(u) && isfinite(v)) ? 0.0 : 1.0;
        uprev[c] = u;
        vprev[c] = v;
    }
    block_sum4<RED_NT>(acc, partial + 4 * blockIdx.x);
}

// momentum-exchange force on the obstacle (SRC/draglift.F90:62-100) over a box of cells
template <typename S, typename K, bool HAS_OBS>
__global__ void __launch_bounds__(RED_NT) draglift_kernel(Lattice L, int cur, int phase, int i0, int i1, int j0, int j1,
                                                          double *partial)
{
    double acc[4] = {0, 0, 0, 0};
    const int nx = i1 - i0 + 1, ny = j1 - j0 + 1;
    const int64_t n = (int64_t)nx * ny;
    for (int64_t c = (int64_t)blockIdx.x * RED_NT + threadIdx.x; c < n; c += (int64_t)gridDim.x * RED_NT) {
        const int x = i0 + (int)(c % nx), y = j0 + (int)(c / nx);
        if (!HAS_OBS) continue;
        if (obs_bit(L, x, y)) continue;
        K fx[8], fy[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int ox = x + cx_of(q), oy = y + cy_of(q);
            const bool ob = ox >= 1 && ox <= L.lx && oy >= 1 && oy <= L.ly && obs_bit(L, ox, oy);
            const K a = post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
            const K o = ob ? (K)1 : (K)0;
            fx[q] = (((K)2 * (K)cx_of(q)) * a) * o;
            fy[q] = (((K)2 * (K)cy_of(q)) * a) * o;
        }
        K sx = ((((((fx[0] + fx[1]) + fx[2]) + fx[3]) + fx[4]) + fx[5]) + fx[6]) + fx[7];
        K sy = ((((((fy[0] + fy[1]) + fy[2]) + fy[3]) + fy[4]) + fy[5]) + fy[6]) + fy[7];
        acc[0] += (double)sx;
        acc[1] += (double)sy;
    }
    block_sum4<RED_NT>(acc, partial + 4 * blockIdx.x);
}

// drag/lift in the reference's own arithmetic (SRC/draglift.F90:41-100): the x then the y sum in
// the compute kind, in the serial j/i order over the box, then times norm = 1/(u_in^2 R).  One
// thread (the box is (2R+7)^2 cells); cells of the box outside the interior are skipped.
template <typename S, typename K, bool HAS_OBS>
__global__ void draglift_seq_kernel(Lattice L, int cur, int phase, int i0, int i1, int j0, int j1, K norm, double *out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    K f[2] = {(K)0, (K)0};
    for (int comp = 0; comp < 2; ++comp) {
        for (int y = j0; y <= j1; ++y) {
            for (int x = i0; x <= i1; ++x) {
                if (obs_bit(L, x, y)) continue;
                K t[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int ox = x + cx_of(q), oy = y + cy_of(q);
                    const bool ob = ox >= 1 && ox <= L.lx && oy >= 1 && oy <= L.ly && obs_bit(L, ox, oy);
                    const K c = (K)(comp == 0 ? cx_of(q) : cy_of(q));
                    t[q] = (((K)2 * c) * post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y)) * (ob ? (K)1 : (K)0);
                }
                f[comp] = f[comp] + (((((((t[0] + t[1]) + t[2]) + t[3]) + t[4]) + t[5]) + t[6]) + t[7]);
            }
        }
    }
    out[0] = (double)(f[0] * norm);
    out[1] = (double)(f[1] * norm);
}

// rho, u, v fields of the interior (double), i fastest
template <typename S, typename K, bool HAS_OBS>
__global__ void fields_kernel(Lattice L, int cur, int phase, double *rho, double *u, double *v)
{
    const int64_t n = (int64_t)L.lx * L.ly;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % L.lx) + 1, y = (int)(c / L.lx) + 1;
        K a[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) a[q] = post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
        K r, xj, yj;
        moments<K>(a, r, xj, yj, L.noshift != 0);
        rho[c] = (double)r;
        u[c] = (double)xj;
        v[c] = (double)yj;
    }
}

// ---------------------------------------------------------------------------------------------
// The reference's profile readers on the device (SRC/prof_i.F90:47-62, SRC/prof_j.F90:47-67,
// SRC/varm.F90:49-88, SRC/probe.F90:46-62), so that a diagnostic stop downloads profiles instead
// of the nine planes.  Their arithmetic is that of the host readers on downloaded arrays: the
// values as they download (H: FP64 for FP64 storage, FP32 otherwise) summed in H as they lie in
// the arrays, cte1 (1, or 0 for populations stored whole) added and the quotients taken in the
// compute kind K; probe copies the values into K temporaries first.  Results are K values held
// exactly in doubles.
template <typename S> using ReaderKind = typename std::conditional<std::is_same<S, double>::value, double, float>::type;

template <typename S, typename K, bool HAS_OBS>
__device__ __forceinline__ void reader_cell(const Lattice &L, int cur, int phase, int x, int y,
                                            ReaderKind<S> (&c)[9])
{
#pragma unroll
    for (int q = 0; q < 9; ++q) c[q] = (ReaderKind<S>)post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
}

// kind 0: prof_i along row a (lx values), kind 1: prof_j along column a (ly values);
// out = u[n], v[n], den[n]
template <typename S, typename K, bool HAS_OBS>
__global__ void prof_kernel(Lattice L, int cur, int phase, int kind, int a, double *out)
{
    using H = ReaderKind<S>;
    const int n = kind == 0 ? L.lx : L.ly;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int x = kind == 0 ? t + 1 : a, y = kind == 0 ? a : t + 1;
    H c[9];
    reader_cell<S, K, HAS_OBS>(L, cur, phase, x, y, c);
    const K cte1 = L.noshift ? (K)0 : (K)1;
    const H s = ((((((((c[0] + c[1]) + c[2]) + c[3]) + c[4]) + c[5]) + c[6]) + c[7]) + c[8]);
    const K den = (K)s + cte1;
    H nu, nv;
    if (kind == 0) {  // prof_i.F90:55-62
        nu = ((((c[0] + c[1]) + c[2]) - c[4]) - c[5]) - c[6];
        nv = ((((c[1] + c[3]) + c[5]) - c[0]) - c[4]) - c[7];
    } else {          // prof_j.F90:56-67
        nu = ((c[0] - c[4]) + (c[1] - c[5])) + (c[2] - c[6]);
        nv = ((c[1] - c[0]) + (c[3] - c[7])) + (c[5] - c[4]);
    }
    out[t] = (double)((K)nu / den);
    out[n + t] = (double)((K)nv / den);
    out[2 * n + t] = (double)den;
}

// varm: one block per row j; the per-cell terms in parallel, their sums over i = 1..lx in order
// by one thread (varm.F90:53-69); out = u[ly], w[ly], den[ly], each times rvol = 1.0/float(lx)
constexpr int VARM_NT = 256;
template <typename S, typename K, bool HAS_OBS>
__global__ void __launch_bounds__(VARM_NT) varm_kernel(Lattice L, int cur, int phase, double *out)
{
    using H = ReaderKind<S>;
    __shared__ K sh[3][VARM_NT];
    const int j = blockIdx.x + 1, t = threadIdx.x;
    const K cte1 = L.noshift ? (K)0 : (K)1;
    K su = (K)0, sw = (K)0, sd = (K)0;
    for (int i0 = 1; i0 <= L.lx; i0 += VARM_NT) {
        const int i = i0 + t;
        if (i <= L.lx) {
            H c[9];
            reader_cell<S, K, HAS_OBS>(L, cur, phase, i, j, c);
            const K rho = (K)((((((((c[0] + c[1]) + c[2]) + c[3]) + c[4]) + c[5]) + c[6]) + c[7]) + c[8]) + cte1;
            const K rhoinv = (K)1 / rho;
            sh[0][t] = rho;
            sh[1][t] = (K)(((((c[0] + c[1]) + c[2]) - c[4]) - c[5]) - c[6]) * rhoinv;
            sh[2][t] = (K)(((((c[1] + c[3]) + c[5]) - c[0]) - c[4]) - c[7]) * rhoinv;
        }
        __syncthreads();
        if (t == 0) {
            const int cnt = min(VARM_NT, L.lx - i0 + 1);
            for (int k = 0; k < cnt; ++k) {
                sd = sd + sh[0][k];
                su = su + sh[1][k];
                sw = sw + sh[2][k];
            }
        }
        __syncthreads();
    }
    if (t == 0) {
        const K rvol = (K)(1.0f / (float)L.lx);  // a default-real quotient (varm.F90:71)
        out[j - 1] = (double)(su * rvol);
        out[L.ly + j - 1] = (double)(sw * rvol);
        out[2 * L.ly + j - 1] = (double)(sd * rvol);
    }
}

// probe at (i0, j0): u, v, rho (probe.F90:46-62), in K temporaries
template <typename S, typename K, bool HAS_OBS>
__global__ void probe_kernel(Lattice L, int cur, int phase, int i0, int j0, double *out)
{
    using H = ReaderKind<S>;
    H c[9];
    reader_cell<S, K, HAS_OBS>(L, cur, phase, i0, j0, c);
    K x[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) x[q] = (K)c[q];
    const K cte1 = L.noshift ? (K)0 : (K)1;
    const K rho = ((((((((x[0] + x[1]) + x[2]) + x[3]) + x[4]) + x[5]) + x[6]) + x[7]) + x[8]) + cte1;
    const K xj = ((((x[0] + x[1]) + x[2]) - x[4]) - x[5]) - x[6];
    const K yj = ((((x[1] + x[3]) + x[5]) - x[0]) - x[4]) - x[7];
    out[0] = (double)(xj / rho);
    out[1] = (double)(yj / rho);
    out[2] = (double)rho;
}

// ---------------------------------------------------------------------------------------------
// Fields of the reference's VTK writers (SRC/vtk_xy.binary.F90:75-140, SRC/vtk_om.binary.F90:61-155),
// in their real(sp) arithmetic: sums of stored values in the storage kind (FP32 for the 16-bit
// kinds), rounded to single precision; the vorticity's quotients divide a storage-kind numerator by
// a single-precision density in the wider kind.
template <typename S> struct VtkSum { using T = S; };
template <> struct VtkSum<__half> { using T = float; };
template <> struct VtkSum<__nv_bfloat16> { using T = float; };

template <typename S, typename K, bool HAS_OBS>
__device__ __forceinline__ void vtk_sums(const Lattice &L, int cur, int phase, int x, int y, float &den,
                                         typename VtkSum<S>::T &u, typename VtkSum<S>::T &v)
{
    using T = typename VtkSum<S>::T;
    T a[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) a[q] = (T)post_value<S, K, HAS_OBS>(L, cur, phase, q, x, y);
    const T t = ((((((((a[0] + a[1]) + a[2]) + a[3]) + a[4]) + a[5]) + a[6]) + a[7]) + a[8]);
    den = (float)(t + (T)(L.noshift ? 0.0f : 1.0f));  // + cte1 (SRC/vtk_xy.binary.F90:46-50)
    u = ((((a[D01] + a[D03]) + a[D05]) - a[D10]) - a[D12]) - a[D14];
    v = ((((a[D03] + a[D08]) + a[D12]) - a[D01]) - a[D10]) - a[D17];
}

// u/rho, w/rho, rho over the interior and the vorticity over 2..lx-1 x 2..ly-1, one cell per thread
template <typename S, typename K, bool HAS_OBS>
__global__ void vtk_cells_kernel(Lattice L, int cur, int phase, float *u, float *w, float *rho, float *vort)
{
    using T = typename VtkSum<S>::T;
    const int l = L.lx, m = L.ly;
    const int64_t n = (int64_t)l * m;
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % l) + 1, y = (int)(c / l) + 1;
        float den;
        T su, sv;
        vtk_sums<S, K, HAS_OBS>(L, cur, phase, x, y, den, su, sv);
        u[c] = (float)su / den;
        w[c] = (float)sv / den;
        rho[c] = den;
        if (x >= 2 && x <= l - 1 && y >= 2 && y <= m - 1) {
            float d_up, d_down, d_left, d_right;
            T u_up, u_down, v_left, v_right, unused;
            vtk_sums<S, K, HAS_OBS>(L, cur, phase, x, y + 1, d_up, u_up, unused);
            vtk_sums<S, K, HAS_OBS>(L, cur, phase, x, y - 1, d_down, u_down, unused);
            vtk_sums<S, K, HAS_OBS>(L, cur, phase, x - 1, y, d_left, unused, v_left);
            vtk_sums<S, K, HAS_OBS>(L, cur, phase, x + 1, y, d_right, unused, v_right);
            const float up1 = (float)(u_up / (T)d_up), down1 = (float)(u_down / (T)d_down);
            const float left1 = (float)(v_left / (T)d_left), right1 = (float)(v_right / (T)d_right);
            vort[(int64_t)(y - 2) * (l - 2) + (x - 2)] = 0.5f * (up1 - down1) - 0.5f * (right1 - left1);
        }
    }
}

// stream function: the column integral of u at x = 1 from row 1 up (one thread, in row order),
// then each row's running sum of -v/rho along x (one thread per row, in column order)
template <typename S, typename K, bool HAS_OBS>
__global__ void vtk_stream_kernel(Lattice L, int cur, int phase, float *phi)
{
    using T = typename VtkSum<S>::T;
    const int m = L.ly;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        float prev = 0.0f;
        for (int y = 1; y <= m; ++y) {
            float den;
            T su, sv;
            vtk_sums<S, K, HAS_OBS>(L, cur, phase, 1, y, den, su, sv);
            prev = prev + (float)su / den;
            phi[y] = prev;
        }
    }
}

template <typename S, typename K, bool HAS_OBS>
__global__ void vtk_stream_rows_kernel(Lattice L, int cur, int phase, const float *phi, float *stream)
{
    using T = typename VtkSum<S>::T;
    const int l = L.lx, m = L.ly;
    const int y = 2 + blockIdx.x * blockDim.x + threadIdx.x;
    if (y > m - 1) return;
    float p = phi[y];
    for (int x = 2; x <= l - 1; ++x) {
        float den;
        T su, sv;
        vtk_sums<S, K, HAS_OBS>(L, cur, phase, x, y, den, su, sv);
        p = p - (float)sv / den;
        stream[(int64_t)(y - 2) * (l - 2) + (x - 2)] = p;
    }
}

// fixed-order sum of nb partial 4-vectors (deterministic)
__global__ void finalize4_kernel(const double *partial, int nb, double *out);

}  // namespace bgk
