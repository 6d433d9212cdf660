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

struct KernelTable {
    int vec;  // cells per 16-byte vector
    int elem_bytes;
    cudaError_t (*step)(int kind, const Lattice &L, int parity, bool obs, int cfg, cudaStream_t st);
    cudaError_t (*scatter)(const Lattice &L, int cur, int q, const void *src, int64_t ld, cudaStream_t st);
    cudaError_t (*gather)(const Lattice &L, int cur, int phase, int q, void *dst, int64_t ld, bool obs, cudaStream_t st);
    cudaError_t (*fill_outflow)(const Lattice &L, cudaStream_t st);
    cudaError_t (*bcond_step)(const Lattice &L, int cur, int stepx, int stepy, cudaStream_t st);
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
    cudaError_t (*vtk)(const Lattice &L, int cur, int phase, bool obs, float *u, float *w, float *rho, float *vort,
                       float *stream, float *phi, cudaStream_t st);
};

KernelTable table_f32_f32();
KernelTable table_f32_f64();
KernelTable table_f64_f64();
KernelTable table_f16_f32();
KernelTable table_bf16_f32();

cudaError_t launch_finalize4(const double *partial, int nb, double *out, cudaStream_t st);

}  // namespace bgk
