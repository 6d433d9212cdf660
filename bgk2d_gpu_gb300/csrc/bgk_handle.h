// bgk_handle.h -- internal definition of the opaque handle (shared by bgk_api.cu and bgk_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/bgk2d_gb300.h"
#include "bgk_common.cuh"
#include "bgk_setup.h"
#include "bgk_table.h"

using bgk::CaseSetup;
using bgk::KernelTable;
using bgk::Lattice;

// Entry of every call that works on a device: select it and drop a runtime error that an
// earlier failed call left pending (that call already reported it), so that the launch checks of
// this call see only their own errors.  A sticky error still fails the next call.
inline cudaError_t enter_device(int dev)
{
    const cudaError_t e = cudaSetDevice(dev);
    (void)cudaGetLastError();
    return e;
}

struct bgk_handle {
    bgk_case_desc desc;
    int dev = 0;
    KernelTable T{};

    Lattice L{};
    CaseSetup cs;
    void *d_planes = nullptr;
    size_t planes_bytes = 0;
    uint32_t *d_mask = nullptr;
    void *d_step_aux = nullptr;    // Lattice::step_aux (AA with a backward-facing step)
    double *d_inflow = nullptr;
    double *d_partial = nullptr;
    double *d_out = nullptr;
    uint32_t *d_status = nullptr;  // kernel-side failure word (Lattice::status)
    int nb_red = 0;
    double *d_uprev = nullptr, *d_vprev = nullptr;
    int64_t res_itime = -1;
    void *d_stage = nullptr;
    size_t stage_bytes = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_steps = 32;
    int cur = 0;     // ping-pong: buffer holding the current state
    int phase = 0;   // AA: 0 = post-collision (swapped slots), 1 = streamed
    int64_t itime = 0;
    int64_t launches = 0;
    int cfg = 2;
    bool two_pass = false;  // BGK_SCHEME_ORIGINAL: ping-pong layout, streaming then collision
    bool streamed = false;  // two-pass: bgk_propagation has run, bgk_collision completes the step
    int host_bytes = 4;
    int sticky = BGK_OK;
    void *batch = nullptr;   // owning batch while attached (steps go through the batch)
    cudaEvent_t wait_ev = nullptr;  // batch event the handle's stream waits on before touching the state
    std::string err;
};
