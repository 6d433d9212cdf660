// bgk_instantiate.cuh -- builds the KernelTable of one (storage S, compute K) pair.
// Each bgk_inst_*.cu translation unit includes this once, so the pairs compile in parallel.
#pragma once

#include <algorithm>

#include "bgk_aux.cuh"
#include "bgk_staged.cuh"
#include "bgk_table.h"

namespace bgk {
namespace inst {

template <typename S> using Host = typename std::conditional<std::is_same<S, double>::value, double, float>::type;

template <typename S, typename K, int TXV, int TY, bool OBS, int CDIV>
cudaError_t step_cfg(int kind, const Lattice &L, int parity, cudaStream_t st)
{
    const dim3 block(TXV, TY);
    if (kind == STEP_PP || kind == STEP_STREAM || kind == STEP_COLLIDE) {
        constexpr int N = vec_of<S>() / CDIV;
        const int nv = (L.lx + N - 1) / N;
        const dim3 grid((unsigned)((nv + TXV - 1) / TXV), (unsigned)((L.ly + TY - 1) / TY));
        if (kind == STEP_PP) pp_kernel<S, K, TXV, TY, OBS, N><<<grid, block, 0, st>>>(L, parity);
        else if (kind == STEP_STREAM) pp_kernel<S, K, TXV, TY, OBS, N, false, false><<<grid, block, 0, st>>>(L, parity);
        else col_kernel<S, K, TXV, TY, N><<<grid, block, 0, st>>>(L, parity);
    } else {
        constexpr int N = vec_of<S>() / CDIV;
        const int nv = (L.lx + N - 1) / N;
        const dim3 grid((unsigned)((nv + TXV - 1) / TXV), (unsigned)((L.ly + TY - 1) / TY));
        if (kind == STEP_AA_P) aa_p_kernel<S, K, TXV, TY, OBS, false, N><<<grid, block, 0, st>>>(L);
        else aa_l_kernel<S, K, TXV, TY, OBS, false, N><<<grid, block, 0, st>>>(L);
    }
    return cudaGetLastError();
}

// ping-pong step through shared-memory staging: one wave of blocks, each a band of T*N columns
// and a stripe of rows
template <typename S, typename K, int T, int STAGES, bool OBS, int CV = 0, int MINB = 0>
cudaError_t step_staged(const Lattice &L, int parity, cudaStream_t st)
{
    constexpr int N = vec_of<S>() / 2;
    constexpr size_t smem = staged_smem_bytes<S, T, N, STAGES>();
    auto kern = pp_staged_kernel<S, K, T, N, STAGES, OBS, CV, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    // A stripe of STAGES rows per block: every copy of the block is issued at once, and the
    // hardware scheduler balances the many short blocks over the SMs.  One wave of long stripes
    // (27 rows per block at 4096^2) left the SMs 27% idle on average, waiting for the slowest
    // block: 116-128 GLUPS in FP16 against 168-172 with stripes of 3 or 4 rows.
    const int bands = (L.lx + T * N - 1) / (T * N);
    const int rows = std::min(STAGES, L.ly);
    const int stripes = (L.ly + rows - 1) / rows;
    kern<<<dim3((unsigned)bands, (unsigned)stripes), T, smem, st>>>(L, parity, rows);
    return cudaGetLastError();
}

// steps with a collision variant (CV_LES, CV_NOSHIFT or both): their own instantiation (128 x 1
// threads, a whole vector per thread), so that the variant's code takes no registers from the
// plain kernels
template <typename S, typename K, bool OBS, int N, int MINB>
cudaError_t les16_launch(const Lattice &L, int parity, cudaStream_t st)
{
    const int nv = (L.lx + N - 1) / N;
    pp_les_kernel<S, K, OBS, N, MINB><<<dim3((unsigned)((nv + 127) / 128), (unsigned)L.ly), 128, 0, st>>>(L, parity);
    return cudaGetLastError();
}

template <typename S, typename K, bool OBS, int CV>
cudaError_t step_cv(int kind, const Lattice &L, int parity, int cfg, cudaStream_t st)
{
    const dim3 block(128, 1);
    // 16-bit ping-pong: register budgets tried by the autotuner (tile configuration 0-3): 4 cells
    // per thread at 8 blocks per SM (64 registers) or 6 (80); 8 cells at 4 (128) or 3 (168).
    // Configurations 4 and 5: the source rows staged in shared memory by bulk async copies (4 cells
    // per thread, stripes of 4 rows at 5 blocks per SM or of 3 rows at 6), so that no register
    // holds a load in flight.
    if constexpr (Is16<S>::value) {
        if (kind == STEP_PP && cfg >= 1 && cfg <= 5) {
            if (cfg == 1) return les16_launch<S, K, OBS, vec_of<S>() / 2, 6>(L, parity, st);
            if (cfg == 2) return les16_launch<S, K, OBS, vec_of<S>(), 4>(L, parity, st);
            if (cfg == 3) return les16_launch<S, K, OBS, vec_of<S>(), 3>(L, parity, st);
            if (cfg == 4) return step_staged<S, K, 128, 4, OBS, CV_LES, 5>(L, parity, st);
            return step_staged<S, K, 128, 3, OBS, CV_LES, 6>(L, parity, st);
        }
    }
    // staged configurations of a single-domain ping-pong step (6-8): one staged LES shape
    if constexpr (CV == CV_LES)
        if (kind == STEP_PP && cfg >= NUM_CFG) return step_staged<S, K, 128, 4, OBS, CV_LES>(L, parity, st);
    // 16-bit kinds: 8 bytes per thread and plane (64 registers, 8 blocks per SM), the fastest shape
    // of their non-LES step; the 32/64-bit kinds: 16 bytes
    constexpr int N = Is16<S>::value ? vec_of<S>() / 2 : vec_of<S>();
    const int nv = (L.lx + N - 1) / N;
    const dim3 grid((unsigned)((nv + 127) / 128), (unsigned)L.ly);
    if (kind == STEP_PP) pp_kernel<S, K, 128, 1, OBS, N, CV><<<grid, block, 0, st>>>(L, parity);
    else if (kind == STEP_STREAM) pp_kernel<S, K, 128, 1, OBS, N, 0, false><<<grid, block, 0, st>>>(L, parity);
    else if (kind == STEP_COLLIDE) col_kernel<S, K, 128, 1, N, CV><<<grid, block, 0, st>>>(L, parity);
    else if (kind == STEP_AA_P) aa_p_kernel<S, K, 128, 1, OBS, CV, N><<<grid, block, 0, st>>>(L);
    else aa_l_kernel<S, K, 128, 1, OBS, CV, N><<<grid, block, 0, st>>>(L);
    return cudaGetLastError();
}

template <typename S, typename K, bool OBS>
cudaError_t step_obs(int kind, const Lattice &L, int parity, int cfg, cudaStream_t st)
{
    if (L.les || L.noshift) {
        // whole-population storage exists for the exact kinds only (bgk_create refuses the rest)
        if constexpr (!Is16<S>::value) {
            if (L.noshift)
                return L.les ? step_cv<S, K, OBS, CV_LES | CV_NOSHIFT>(kind, L, parity, cfg, st)
                             : step_cv<S, K, OBS, CV_NOSHIFT>(kind, L, parity, cfg, st);
        }
        return step_cv<S, K, OBS, CV_LES>(kind, L, parity, cfg, st);
    }
    if (kind == STEP_PP && cfg >= NUM_CFG) {
        if (cfg == 6) return step_staged<S, K, 128, 3, OBS>(L, parity, st);
        if (cfg == 7) return step_staged<S, K, 128, 4, OBS>(L, parity, st);
        return step_staged<S, K, 256, 3, OBS>(L, parity, st);
    }
    switch (cfg) {
    case 0: return step_cfg<S, K, 32, 4, OBS, 1>(kind, L, parity, st);
    case 1: return step_cfg<S, K, 64, 2, OBS, 1>(kind, L, parity, st);
    case 3: return step_cfg<S, K, 128, 2, OBS, 1>(kind, L, parity, st);
    case 4: return step_cfg<S, K, 32, 4, OBS, 2>(kind, L, parity, st);
    case 5: return step_cfg<S, K, 128, 1, OBS, 2>(kind, L, parity, st);
    default: return step_cfg<S, K, 128, 1, OBS, 1>(kind, L, parity, st);
    }
}

template <typename S, typename K>
cudaError_t step(int kind, const Lattice &L, int parity, bool obs, int cfg, cudaStream_t st)
{
    return obs ? step_obs<S, K, true>(kind, L, parity, cfg, st) : step_obs<S, K, false>(kind, L, parity, cfg, st);
}

template <typename S>
cudaError_t scatter(const Lattice &L, int cur, int q, const void *stage, int64_t ld, cudaStream_t st)
{
    const dim3 block(256), grid((unsigned)((L.lx + 2 + 255) / 256), (unsigned)(L.ly + 2));
    scatter_plane_kernel<S, Host<S>><<<grid, block, 0, st>>>(L, cur, q, reinterpret_cast<const Host<S> *>(stage), ld);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t gather(const Lattice &L, int cur, int phase, int q, void *stage, int64_t ld, bool obs, cudaStream_t st)
{
    const dim3 block(256), grid((unsigned)((L.lx + 2 + 255) / 256), (unsigned)(L.ly + 2));
    if (obs) gather_plane_kernel<S, K, Host<S>, true><<<grid, block, 0, st>>>(L, cur, phase, q, reinterpret_cast<Host<S> *>(stage), ld);
    else gather_plane_kernel<S, K, Host<S>, false><<<grid, block, 0, st>>>(L, cur, phase, q, reinterpret_cast<Host<S> *>(stage), ld);
    return cudaGetLastError();
}

// All nine mapped host planes <-> buffer cur in chunks of rows of fewer than 2^26 host elements
// (the 32-bit unit arithmetic of xfer_rows), 4 blocks of 256 threads per SM at most.
template <typename S, typename K, bool OBS, bool UP>
cudaError_t xfer_launch(const Lattice &L, int cur, int phase, const HostPlanes &hp, cudaStream_t st)
{
    const int64_t rows_per_chunk = std::max<int64_t>(1, ((int64_t)1 << 26) / hp.ld - 1);
    for (int64_t ya = 0; ya <= L.ly + 1; ya += rows_per_chunk) {
        const int64_t yb = std::min<int64_t>(ya + rows_per_chunk - 1, L.ly + 1);
        const int64_t units = 9 * (((yb - ya + 1) * hp.ld + 63) / 32);
        const int64_t warps = (units + XFER_UNROLL - 1) / XFER_UNROLL;
        const unsigned grid = (unsigned)std::min<int64_t>(4 * 152, (warps + 7) / 8);
        xfer_kernel<S, K, Host<S>, OBS, UP><<<grid, 256, 0, st>>>(L, cur, phase, hp, (int)ya, (int)yb);
    }
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t xfer(const Lattice &L, int cur, int phase, bool up, const HostPlanes &hp, bool obs, cudaStream_t st)
{
    if (up) return obs ? xfer_launch<S, K, true, true>(L, cur, phase, hp, st) : xfer_launch<S, K, false, true>(L, cur, phase, hp, st);
    return obs ? xfer_launch<S, K, true, false>(L, cur, phase, hp, st) : xfer_launch<S, K, false, false>(L, cur, phase, hp, st);
}

template <typename S, typename K, bool OBS, int N>
cudaError_t wave_launch(const Lattice &L, const WaveArgs &a, int grid_y, cudaStream_t st)
{
    const int nv = (L.lx + N - 1) / N;
    const dim3 grid((unsigned)((nv + 127) / 128), (unsigned)grid_y);
    // a collision variant steps with its own kernel shape: 16 bytes per thread for the exact
    // kinds, 8 for the 16-bit ones (step_cv); the caller passes that N
    if (L.les || L.noshift) {
        if constexpr (Is16<S>::value) {
            if constexpr (N == vec_of<S>() / 2) {
                wave_kernel<S, K, Host<S>, OBS, N, CV_LES><<<grid, 128, 0, st>>>(L, a);
                return cudaGetLastError();
            }
        } else if constexpr (N == vec_of<S>()) {
            const int cv = (L.les ? CV_LES : 0) | (L.noshift ? CV_NOSHIFT : 0);
            if (cv == CV_LES) wave_kernel<S, K, Host<S>, OBS, N, CV_LES><<<grid, 128, 0, st>>>(L, a);
            else if (cv == CV_NOSHIFT) wave_kernel<S, K, Host<S>, OBS, N, CV_NOSHIFT><<<grid, 128, 0, st>>>(L, a);
            else wave_kernel<S, K, Host<S>, OBS, N, CV_LES | CV_NOSHIFT><<<grid, 128, 0, st>>>(L, a);
            return cudaGetLastError();
        }
        return cudaErrorInvalidValue;
    }
    wave_kernel<S, K, Host<S>, OBS, N><<<grid, 128, 0, st>>>(L, a);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t wave(const Lattice &L, const WaveArgs &a, bool obs, int cdiv, int grid_y, cudaStream_t st)
{
    constexpr int V = vec_of<S>();
    if (cdiv == 2) return obs ? wave_launch<S, K, true, V / 2>(L, a, grid_y, st) : wave_launch<S, K, false, V / 2>(L, a, grid_y, st);
    return obs ? wave_launch<S, K, true, V>(L, a, grid_y, st) : wave_launch<S, K, false, V>(L, a, grid_y, st);
}

template <typename S, typename K>
cudaError_t fill_outflow(const Lattice &L, cudaStream_t st)
{
    aa_fill_outflow_kernel<S, K><<<(L.ly + 127) / 128, 128, 0, st>>>(L);
    return cudaGetLastError();
}


template <typename S, typename K>
cudaError_t batch_les(const Lattice *lats, const int *cur, const int4 *tiles, int n, int parity, cudaStream_t st)
{
    constexpr int N = Is16<S>::value ? vec_of<S>() / 2 : vec_of<S>();
    batch_les_kernel<S, K, N><<<n, 128, 0, st>>>(lats, cur, tiles, parity);
    return cudaGetLastError();
}


template <typename S>
cudaError_t init_tgv(const Lattice &L, double u0, cudaStream_t st)
{
    const dim3 block(256), grid((unsigned)((L.lx + 2 + 255) / 256), (unsigned)(L.ly + 2));
    init_tgv_kernel<S><<<grid, block, 0, st>>>(L, u0);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t diagno(const Lattice &L, int cur, int phase, int fluid_only, bool obs, double *partial, int nb, cudaStream_t st)
{
    if (obs) diagno_kernel<S, K, true><<<nb, RED_NT, 0, st>>>(L, cur, phase, fluid_only, partial);
    else diagno_kernel<S, K, false><<<nb, RED_NT, 0, st>>>(L, cur, phase, fluid_only, partial);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t diagno_seq(const Lattice &L, int cur, int phase, bool obs, double *out, cudaStream_t st)
{
    if (obs) diagno_seq_kernel<S, K, true><<<1, 1024, 0, st>>>(L, cur, phase, out);
    else diagno_seq_kernel<S, K, false><<<1, 1024, 0, st>>>(L, cur, phase, out);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t residual(const Lattice &L, int cur, int phase, bool obs, double *uprev, double *vprev, double *partial, int nb,
                     cudaStream_t st)
{
    if (obs) residual_kernel<S, K, true><<<nb, RED_NT, 0, st>>>(L, cur, phase, uprev, vprev, partial);
    else residual_kernel<S, K, false><<<nb, RED_NT, 0, st>>>(L, cur, phase, uprev, vprev, partial);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t draglift(const Lattice &L, int cur, int phase, int i0, int i1, int j0, int j1, double *partial, int nb,
                     cudaStream_t st)
{
    draglift_kernel<S, K, true><<<nb, RED_NT, 0, st>>>(L, cur, phase, i0, i1, j0, j1, partial);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t draglift_seq(const Lattice &L, int cur, int phase, int i0, int i1, int j0, int j1, double norm, double *out,
                         cudaStream_t st)
{
    draglift_seq_kernel<S, K, true><<<1, 32, 0, st>>>(L, cur, phase, i0, i1, j0, j1, (K)norm, out);
    return cudaGetLastError();
}

template <typename S, typename K>
cudaError_t fields(const Lattice &L, int cur, int phase, bool obs, double *rho, double *u, double *v, cudaStream_t st)
{
    const int nb = 4 * 152;
    if (obs) fields_kernel<S, K, true><<<nb, 256, 0, st>>>(L, cur, phase, rho, u, v);
    else fields_kernel<S, K, false><<<nb, 256, 0, st>>>(L, cur, phase, rho, u, v);
    return cudaGetLastError();
}

// the reference's profile readers: kind 0 prof_i (row a), 1 prof_j (column a), 2 varm, 3 probe
// at (a, b); out holds 3 x (lx, ly, ly, 1) doubles
template <typename S, typename K, bool OBS>
void readers_launch(const Lattice &L, int cur, int phase, int kind, int a, int b, double *out, cudaStream_t st)
{
    if (kind <= 1) {
        const int n = kind == 0 ? L.lx : L.ly;
        prof_kernel<S, K, OBS><<<(n + 255) / 256, 256, 0, st>>>(L, cur, phase, kind, a, out);
    } else if (kind == 2) {
        varm_kernel<S, K, OBS><<<L.ly, VARM_NT, 0, st>>>(L, cur, phase, out);
    } else {
        probe_kernel<S, K, OBS><<<1, 1, 0, st>>>(L, cur, phase, a, b, out);
    }
}

template <typename S, typename K>
cudaError_t readers(const Lattice &L, int cur, int phase, bool obs, int kind, int a, int b, double *out, cudaStream_t st)
{
    if (obs) readers_launch<S, K, true>(L, cur, phase, kind, a, b, out, st);
    else readers_launch<S, K, false>(L, cur, phase, kind, a, b, out, st);
    return cudaGetLastError();
}

template <typename S, typename K, bool OBS>
void vtk_launch(const Lattice &L, int cur, int phase, float *u, float *w, float *rho, float *vort, float *stream,
                float *phi, cudaStream_t st)
{
    vtk_cells_kernel<S, K, OBS><<<4 * 152, 256, 0, st>>>(L, cur, phase, u, w, rho, vort);
    vtk_stream_kernel<S, K, OBS><<<1, 32, 0, st>>>(L, cur, phase, phi);
    if (L.ly > 2) vtk_stream_rows_kernel<S, K, OBS><<<(L.ly - 2 + 127) / 128, 128, 0, st>>>(L, cur, phase, phi, stream);
}

template <typename S, typename K>
cudaError_t vtk(const Lattice &L, int cur, int phase, bool obs, float *u, float *w, float *rho, float *vort,
                float *stream, float *phi, cudaStream_t st)
{
    if (obs) vtk_launch<S, K, true>(L, cur, phase, u, w, rho, vort, stream, phi, st);
    else vtk_launch<S, K, false>(L, cur, phase, u, w, rho, vort, stream, phi, st);
    return cudaGetLastError();
}

template <typename S, typename K, int TXV, int TY, int N>
void batch_launch(const Lattice *lats, const int *cur, const int4 *tiles, int ntiles, int parity, int grid, int pf,
                  cudaStream_t st)
{
    if (grid <= 0)
        batch_pp_flat_kernel<S, K, TXV, TY, N><<<ntiles, dim3(TXV, TY), 0, st>>>(lats, cur, tiles, ntiles, parity, pf);
    else batch_pp_kernel<S, K, TXV, TY, N><<<grid, dim3(TXV, TY), 0, st>>>(lats, cur, tiles, ntiles, parity);
}

// grid <= 0: one block per tile; otherwise a persistent grid walking contiguous chunks
template <typename S, typename K>
cudaError_t batch_step(const Lattice *lats, const int *cur, const int4 *tiles, int ntiles, int parity, int cfg, int grid,
                       int pf, cudaStream_t st)
{
    constexpr int V = vec_of<S>();
    switch (cfg) {
    case 0: batch_launch<S, K, 32, 4, V>(lats, cur, tiles, ntiles, parity, grid, pf, st); break;
    case 1: batch_launch<S, K, 64, 2, V>(lats, cur, tiles, ntiles, parity, grid, pf, st); break;
    case 3: batch_launch<S, K, 128, 2, V>(lats, cur, tiles, ntiles, parity, grid, pf, st); break;
    case 4: batch_launch<S, K, 32, 4, V / 2>(lats, cur, tiles, ntiles, parity, grid, pf, st); break;
    case 5: batch_launch<S, K, 128, 1, V / 2>(lats, cur, tiles, ntiles, parity, grid, pf, st); break;
    default: batch_launch<S, K, 128, 1, V>(lats, cur, tiles, ntiles, parity, grid, pf, st); break;
    }
    return cudaGetLastError();
}

template <typename S, typename K>
KernelTable make_table()
{
    KernelTable t;
    t.vec = vec_of<S>();
    t.elem_bytes = (int)sizeof(S);
    t.step = &step<S, K>;
    t.scatter = &scatter<S>;
    t.gather = &gather<S, K>;
    t.fill_outflow = &fill_outflow<S, K>;
    t.batch_les = &batch_les<S, K>;
    t.init_tgv = &init_tgv<S>;
    t.diagno = &diagno<S, K>;
    t.diagno_seq = &diagno_seq<S, K>;
    t.residual = &residual<S, K>;
    t.draglift = &draglift<S, K>;
    t.draglift_seq = &draglift_seq<S, K>;
    t.fields = &fields<S, K>;
    t.readers = &readers<S, K>;
    t.vtk = &vtk<S, K>;
    t.batch_step = &batch_step<S, K>;
    t.xfer = &xfer<S, K>;
    t.wave = &wave<S, K>;
    return t;
}

}  // namespace inst
}  // namespace bgk
