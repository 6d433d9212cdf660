// bgk_table.h -- host-side table of the kernels instantiated for one (storage, compute) pair.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace bgk {

struct Lattice;

// step kinds
enum StepKind { STEP_PP = 0, STEP_AA_P = 1, STEP_AA_L = 2, STEP_STREAM = 3, STEP_COLLIDE = 4 };
// STEP_STREAM and STEP_COLLIDE are the two halves of the two-pass form (SRC/movef.F90 then
// SRC/col.F90): parity = the source buffer for STREAM, the buffer collided in place for COLLIDE.

// thread-block shapes: threads along a row segment x rows, and cells per thread as a divisor of
// the 16-byte vector (1: a thread updates 16 bytes of each plane, 2: 8 bytes).
struct TileCfg { int txv, ty, cdiv; };
constexpr int NUM_CFG = 6;
constexpr TileCfg TILE_CFGS[NUM_CFG] = {{32, 4, 1}, {64, 2, 1}, {128, 1, 1}, {128, 2, 1}, {32, 4, 2}, {128, 1, 2}};
// Single-domain ping-pong only: configurations NUM_CFG .. NUM_STEP_CFG-1 select the kernel whose
// source rows are staged in shared memory by bulk async copies (8 bytes of each plane per thread):
// 6 = 128 threads, 3 rows in flight; 7 = 128 threads, 4 rows; 8 = 256 threads, 3 rows.
constexpr int NUM_STEP_CFG = 9;

// Nine host planes in the reference layout: element (x, y) of direction q at p[q] + y * ld + x.
// Page-locked and mapped into the device address space: the transfer code reads and writes them
// in place over the host link.
struct HostPlanes {
    void *p[9];
    int64_t ld;
};

// One launch (a "wave") of the pipelined upload -> steps -> download of bgk_advance_host.  The
// interior rows are cut into bands of band_rows rows.  Wave w uploads band w, runs local step k
// (1..nsteps) on band w - 2k for k in [k_lo, k_hi], and downloads band w - 2 nsteps - 1.  Step k
// reads buffer (cur0 + k - 1) & 1.  Band b's step k thus runs after step k-1 on bands b-1, b and
// b+1 (the rows it pulls from, and the rows whose pulls read the rows it overwrites), and the
// bands of one wave are two apart, so no two items of a wave touch the same rows of a buffer.
struct WaveArgs {
    HostPlanes in, out;
    int32_t band_rows, nbands, nsteps, cur0;
    int32_t wave, k_lo, k_hi;
    int32_t up_band, down_band;  // -1: none in this wave
    int32_t xfer_rows;           // grid rows (blockIdx.y) given to each transfer of the wave
};

struct KernelTable {
    int vec;  // cells per 16-byte vector
    int elem_bytes;
    cudaError_t (*step)(int kind, const Lattice &L, int parity, bool obs, int cfg, cudaStream_t st);
    cudaError_t (*scatter)(const Lattice &L, int cur, int q, const void *src, int64_t ld, cudaStream_t st);
    cudaError_t (*gather)(const Lattice &L, int cur, int phase, int q, void *dst, int64_t ld, bool obs, cudaStream_t st);
    cudaError_t (*fill_outflow)(const Lattice &L, cudaStream_t st);
    // the Smagorinsky step of a batch's LES members over their n work-list entries
    cudaError_t (*batch_les)(const Lattice *lats, const int *cur, const int4 *tiles, int n, int parity, cudaStream_t st);
    cudaError_t (*init_tgv)(const Lattice &L, double u0, cudaStream_t st);
    cudaError_t (*diagno)(const Lattice &L, int cur, int phase, int fluid_only, bool obs, double *partial, int nb,
                          cudaStream_t st);
    cudaError_t (*diagno_seq)(const Lattice &L, int cur, int phase, bool obs, double *out, cudaStream_t st);
    cudaError_t (*residual)(const Lattice &L, int cur, int phase, bool obs, double *uprev, double *vprev,
                            double *partial, int nb, cudaStream_t st);
    cudaError_t (*draglift)(const Lattice &L, int cur, int phase, int i0, int i1, int j0, int j1, double *partial,
                            int nb, cudaStream_t st);
    cudaError_t (*draglift_seq)(const Lattice &L, int cur, int phase, int i0, int i1, int j0, int j1, double norm,
                                double *out, cudaStream_t st);
    cudaError_t (*batch_step)(const Lattice *lats, const int *cur, const int4 *tiles, int ntiles, int parity, int cfg,
                              int grid, int pf, cudaStream_t st);
    cudaError_t (*fields)(const Lattice &L, int cur, int phase, bool obs, double *rho, double *u, double *v,
                          cudaStream_t st);
    // the reference's profile readers (0 prof_i row a, 1 prof_j column a, 2 varm, 3 probe at (a, b))
    cudaError_t (*readers)(const Lattice &L, int cur, int phase, bool obs, int kind, int a, int b, double *out,
                           cudaStream_t st);
    cudaError_t (*vtk)(const Lattice &L, int cur, int phase, bool obs, float *u, float *w, float *rho, float *vort,
                       float *stream, float *phi, cudaStream_t st);
    // all nine mapped host planes <-> state buffer cur, one launch per chunk of rows
    cudaError_t (*xfer)(const Lattice &L, int cur, int phase, bool up, const HostPlanes &hp, bool obs, cudaStream_t st);
    // one wave of bgk_advance_host: cdiv as in TileCfg (128 x 1 threads), grid_y grid rows
    cudaError_t (*wave)(const Lattice &L, const WaveArgs &a, bool obs, int cdiv, int grid_y, cudaStream_t st);
};

KernelTable table_f32_f32();
KernelTable table_f32_f64();
KernelTable table_f64_f64();
KernelTable table_f16_f32();
KernelTable table_bf16_f32();

cudaError_t launch_finalize4(const double *partial, int nb, double *out, cudaStream_t st);

}  // namespace bgk
