// bgk_api.cu -- C ABI of libbgk2d_gb300.so: handle lifecycle, transfers, stepping, reductions.
//
// The reference keeps its populations in `module storage` and runs boundaries, propagation
// and collision as separate directive loops (SRC/bgk2d.F90:100-102).  Here a handle owns the
// populations in HBM.  One fused kernel per time step applies the boundary rules, streams and
// collides (ping-pong or AA); the two-pass scheme streams and collides in two kernels as the
// ORIGINAL build does; the backward-facing step adds its boundary kernel in front.  Steps are
// replayed from CUDA graphs, the tile shape and L2 prefetch distance come from the autotuner,
// and reductions run on the device (FP64, or the reference's own order for diagno).
#include <cuda_runtime.h>

#include <utility>

#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bgk2d_gb300.h"
#include "bgk_common.cuh"
#include "bgk_setup.h"
#include "bgk_table.h"

using namespace bgk;

namespace bgk {

__global__ void finalize4_kernel(const double *partial, int nb, double *out)
{
    __shared__ double sh[256][4];
    double s[4] = {0, 0, 0, 0};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int i = 0; i < 4; ++i) s[i] += partial[4 * b + i];
    for (int i = 0; i < 4; ++i) sh[threadIdx.x][i] = s[i];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int i = 0; i < 4; ++i) sh[threadIdx.x][i] += sh[threadIdx.x + w][i];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int i = 0; i < 4; ++i) out[i] = sh[0][i];
}

cudaError_t launch_finalize4(const double *partial, int nb, double *out, cudaStream_t st)
{
    finalize4_kernel<<<1, 256, 0, st>>>(partial, nb, out);
    return cudaGetLastError();
}

}  // namespace bgk

#include "bgk_handle.h"

namespace {

int fail(bgk_handle *h, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) {
        h->err = buf;  // the most recent failure (bgk_last_error)
        if (code == BGK_E_CUDA) h->sticky = code;
    }
    if (code == BGK_E_CUDA || code == BGK_E_NOMEM) (void)cudaGetLastError();  // reported here
    return code;
}

#define CK(h, call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return fail(h, BGK_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CHECK_HANDLE(h)                                     \
    do {                                                    \
        if (!(h)) return BGK_E_INVALID;                     \
        if ((h)->sticky != BGK_OK) return (h)->sticky;      \
        if (enter_device((h)->dev) != cudaSuccess) return fail(h, BGK_E_CUDA, "cudaSetDevice"); \
        if ((h)->wait_ev) CK(h, cudaStreamWaitEvent((h)->st, (h)->wait_ev, 0)); \
    } while (0)

#define NOT_IN_BATCH(h) \
    do { if ((h)->batch) return fail(h, BGK_E_INVALID, "handle is attached to a batch; step the batch"); } while (0)

// Stream-ordered allocations: creating or destroying a case does not synchronise the device,
// so a serving loop can admit and retire cases while other work runs.
template <typename T>
cudaError_t dalloc(bgk_handle *h, T **p, size_t bytes)
{
    const cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(p), bytes, h->st);
    if (e != cudaSuccess) *p = nullptr;  // release() frees only what was allocated
    return e;
}

void dfree(bgk_handle *h, void *p)
{
    if (p) cudaFreeAsync(p, h->st);
}

bool get_table(int storage, int compute, KernelTable &t)
{
    if (storage == BGK_STORE_F32 && compute == BGK_COMPUTE_F32) t = table_f32_f32();
    else if (storage == BGK_STORE_F32 && compute == BGK_COMPUTE_F64) t = table_f32_f64();
    else if (storage == BGK_STORE_F64 && compute == BGK_COMPUTE_F64) t = table_f64_f64();
    else if (storage == BGK_STORE_F16 && compute == BGK_COMPUTE_F32) t = table_f16_f32();
    else if (storage == BGK_STORE_BF16 && compute == BGK_COMPUTE_F32) t = table_bf16_f32();
    else return false;
    return true;
}

int default_cfg(int nvec)
{
    if (nvec >= 128) return 2;  // 128 x 1
    if (nvec >= 64) return 1;   // 64 x 2
    return 0;                   // 32 x 4
}

int ensure_stage(bgk_handle *h)
{
    const size_t need = (size_t)(h->desc.lx + 2) * (size_t)(h->desc.ly + 2) * (size_t)h->host_bytes;
    if (h->stage_bytes >= need) return BGK_OK;
    dfree(h, h->d_stage);
    h->d_stage = nullptr;
    h->stage_bytes = 0;
    if (dalloc(h, &h->d_stage, need) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, BGK_E_NOMEM, "staging buffer of %zu bytes", need);
    }
    h->stage_bytes = need;
    return BGK_OK;
}

// Device address of a page-locked host array (cudaHostAlloc, cudaHostRegister, torch pinned
// memory), or null for pageable memory.  The transfer kernels read and write such an array in
// place over the host link.  Measured on GB300 after a long run of steps, this path moved 604 MB
// in 3.2 ms up and 3.8 ms down every time, while copies by the copy engines through a staging
// buffer took 3.7 ms or about 30 ms, unpredictably.  Pageable arrays take the staging path.
const void *mapped_host(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Mapped device addresses of nine page-locked host planes, or false when one of them is
// pageable (or not aligned to its element size).
bool all_mapped(const bgk_handle *h, void *const pops[9], int64_t ld, HostPlanes &hp)
{
    hp.ld = ld;
    for (int q = 0; q < 9; ++q) {
        const void *dp = mapped_host(pops[q]);
        if (!dp || ((uintptr_t)dp % (uintptr_t)h->host_bytes) != 0) return false;
        hp.p[q] = const_cast<void *>(dp);
    }
    return true;
}

// host population arrays (reference layout) -> device state.  Page-locked arrays are read in
// place by one transfer launch for all nine planes; pageable ones go through the staging plane.
int upload_impl(bgk_handle *h, const void *const pops[9], int64_t ld, bool sync = true)
{
    const int l = h->desc.lx, m = h->desc.ly;
    if (ld < l + 2) return fail(h, BGK_E_INVALID, "leading dimension %lld < lx+2", (long long)ld);
    const size_t hb = (size_t)h->host_bytes;
    for (int q = 0; q < 9; ++q)
        if (!pops[q]) return fail(h, BGK_E_INVALID, "population %d is NULL", q);
    HostPlanes hp;
    if (all_mapped(h, const_cast<void *const *>(pops), ld, hp)) {
        CK(h, h->T.xfer(h->L, h->cur, h->phase, true, hp, h->cs.has_obs, h->st));
        h->launches++;
    } else {
        for (int q = 0; q < 9; ++q) {
            int rc = ensure_stage(h);
            if (rc) return rc;
            if (ld == l + 2)  // contiguous host plane: one linear copy (3x faster than the 2D form)
                CK(h, cudaMemcpyAsync(h->d_stage, pops[q], (size_t)(l + 2) * (m + 2) * hb, cudaMemcpyHostToDevice, h->st));
            else
                CK(h, cudaMemcpy2DAsync(h->d_stage, (l + 2) * hb, pops[q], (size_t)ld * hb, (l + 2) * hb, m + 2,
                                        cudaMemcpyHostToDevice, h->st));
            CK(h, h->T.scatter(h->L, h->cur, q, h->d_stage, l + 2, h->st));
            h->launches++;
        }
    }
    if (h->L.scheme == BGK_SCHEME_AA) {
        h->phase = 0;
        if (h->cs.faces[XHI] == FK_OUTFLOW_EQ || h->cs.faces[XHI] == FK_OUTFLOW_ZG) {
            CK(h, h->T.fill_outflow(h->L, h->st));
            h->launches++;
        }
    }
    if (sync) CK(h, cudaStreamSynchronize(h->st));
    return BGK_OK;
}

// device state -> host population arrays (synchronises)
int download_impl(bgk_handle *h, void *const pops[9], int64_t ld)
{
    const int l = h->desc.lx, m = h->desc.ly;
    if (!pops || ld < l + 2) return fail(h, BGK_E_INVALID, "bad download arguments");
    const size_t hb = (size_t)h->host_bytes;
    for (int q = 0; q < 9; ++q)
        if (!pops[q]) return fail(h, BGK_E_INVALID, "population %d is NULL", q);
    HostPlanes hp;
    if (all_mapped(h, pops, ld, hp)) {
        CK(h, h->T.xfer(h->L, h->cur, h->phase, false, hp, h->cs.has_obs, h->st));
        h->launches++;
    } else {
        for (int q = 0; q < 9; ++q) {
            h->launches++;
            int rc = ensure_stage(h);
            if (rc) return rc;
            CK(h, h->T.gather(h->L, h->cur, h->phase, q, h->d_stage, l + 2, h->cs.has_obs, h->st));
            if (ld == l + 2)
                CK(h, cudaMemcpyAsync(pops[q], h->d_stage, (size_t)(l + 2) * (m + 2) * hb, cudaMemcpyDeviceToHost, h->st));
            else
                CK(h, cudaMemcpy2DAsync(pops[q], (size_t)ld * hb, h->d_stage, (l + 2) * hb, (l + 2) * hb, m + 2,
                                        cudaMemcpyDeviceToHost, h->st));
        }
    }
    CK(h, cudaStreamSynchronize(h->st));
    return BGK_OK;
}

int launch_step(bgk_handle *h)
{
    if (h->L.scheme == BGK_SCHEME_PINGPONG) {
        if (h->two_pass) {
            CK(h, h->T.step(STEP_STREAM, h->L, h->cur, h->cs.has_obs, h->cfg, h->st));
            CK(h, h->T.step(STEP_COLLIDE, h->L, h->cur ^ 1, h->cs.has_obs, h->cfg, h->st));
            h->launches++;
        } else {
            CK(h, h->T.step(STEP_PP, h->L, h->cur, h->cs.has_obs, h->cfg, h->st));
        }
        h->cur ^= 1;
    } else {
        CK(h, h->T.step(h->phase == 0 ? STEP_AA_P : STEP_AA_L, h->L, 0, h->cs.has_obs, h->cfg, h->st));
        h->phase ^= 1;
    }
    h->launches++;
    h->itime++;
    return BGK_OK;
}

// graph of graph_steps steps starting from the state slot `start` (PP buffer / AA phase 0)
int build_graph(bgk_handle *h, int start)
{
    cudaGraph_t g = nullptr;
    const int cur0 = h->cur, ph0 = h->phase;
    const int64_t it0 = h->itime, ln0 = h->launches;
    if (h->L.scheme == BGK_SCHEME_PINGPONG) h->cur = start;
    else h->phase = 0;
    CK(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    int rc = BGK_OK;
    for (int s = 0; s < h->graph_steps && rc == BGK_OK; ++s) rc = launch_step(h);
    cudaError_t e = cudaStreamEndCapture(h->st, &g);
    h->cur = cur0;
    h->phase = ph0;
    h->itime = it0;
    h->launches = ln0;
    if (rc != BGK_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return fail(h, BGK_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&h->graph[start], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(h, BGK_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    return BGK_OK;
}

int steps_impl(bgk_handle *h, int32_t n)
{
    if (n < 0) return fail(h, BGK_E_INVALID, "negative step count");
    if (h->streamed) return fail(h, BGK_E_INVALID, "two-pass step half done: call bgk_collision first");
    int rc;
    // AA graphs start at phase 0; the odd step that brings phase 1 back to 0 runs directly
    if (h->L.scheme == BGK_SCHEME_AA && h->phase == 1 && n > 0) {
        if ((rc = launch_step(h))) return rc;
        --n;
    }
    while (n >= h->graph_steps) {
        const int slot = h->L.scheme == BGK_SCHEME_PINGPONG ? h->cur : 0;
        if (!h->graph[slot] && (rc = build_graph(h, slot))) return rc;
        CK(h, cudaGraphLaunch(h->graph[slot], h->st));
        h->launches += (int64_t)h->graph_steps * (1 + (h->two_pass ? 1 : 0));
        h->itime += h->graph_steps;
        n -= h->graph_steps;
    }
    while (n-- > 0)
        if ((rc = launch_step(h))) return rc;
    return BGK_OK;
}

// Status word of the step kernels, read once the stream is idle: non-zero when a bounded wait
// inside a kernel ran out, which leaves the state undefined (the handle stays failed).
int check_status(bgk_handle *h)
{
    uint32_t s = 0;
    CK(h, cudaMemcpyAsync(&s, h->d_status, sizeof(s), cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    if (s != 0) {
        h->sticky = BGK_E_TIMEOUT;
        return fail(h, BGK_E_TIMEOUT, "step kernel: a wait for staged rows ran out (status 0x%x)", s);
    }
    return BGK_OK;
}

int reduce4(bgk_handle *h, double out[4])
{
    CK(h, launch_finalize4(h->d_partial, h->nb_red, h->d_out, h->st));
    h->launches++;
    CK(h, cudaMemcpyAsync(out, h->d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return check_status(h);
}

// ---- pipelined host -> steps -> host (bgk_advance_host) ----------------------------------
// The state moves over the host link while the steps run: the rows are cut into bands, and
// wave w uploads band w, applies step k to band w - 2k and downloads band w - 2K - 1 in one
// launch (WaveArgs).  Up and down traffic share the link and the steps hide under both, so a
// short run costs about one transfer time instead of upload + steps + download.

// Steps pipelined with each transfer when a run is long: the rest run from the step graphs.
constexpr int PIPE_STEPS = 16;

bool pipeline_ok(const bgk_handle *h)
{
    // pulls reach one row up and one row down, nothing else: no periodic y faces (row 1 pulls
    // from row ly), no two-pass form
    return h->L.scheme == BGK_SCHEME_PINGPONG && !h->two_pass &&
           h->cs.faces[YLO] != FK_PERIODIC && h->cs.faces[YHI] != FK_PERIODIC && h->desc.ly >= 8;
}

int env_int(const char *name, int dflt)
{
    const char *v = std::getenv(name);
    return (v && *v) ? std::atoi(v) : dflt;
}

// One pipelined run of K steps: with the upload of `in` (or from the state in buffer h->cur)
// and with the download into `out` (or leaving the state on the device).  The waves' own blocks
// move each band between the mapped host planes and the state.  (Copy-engine forms, 3D copies per
// band or per-plane copies of chunks of bands through a device staging copy, measured slower:
// 6.98-7.27 ms against 6.6 ms for 20 steps of the 4096^2 cavity.  So did either direction by the
// copy engines through a device copy of the host planes and the other by the waves, in chunks of
// 128 to 2048 rows: 6.6-7.8 ms, although one 604 MB transfer each way, one by the SMs and one by
// the copy engines, took 4.15-4.35 ms together against 6.1 ms one after the other.)
int run_waves(bgk_handle *h, const HostPlanes *in, const HostPlanes *out, int K)
{
    const int lx = h->desc.lx, ly = h->desc.ly;
    // bands of about ly/128 rows (32 at 4096^2); BGK_PIPE_ROWS / BGK_PIPE_XFER override the band
    // height and the blocks of each transfer
    const int R = std::max(1, std::min(ly, env_int("BGK_PIPE_ROWS", std::max(4, (ly + 127) / 128))));
    // the shape of the handle's step: a collision variant (LES, NOSHIFT) has one, 16 bytes per
    // thread for the exact kinds and 8 for the 16-bit ones
    const bool cv = h->L.les || h->L.noshift;
    const int cdiv = h->T.elem_bytes == 2 ? 2 : cv ? 1 : (h->cfg < NUM_CFG && TILE_CFGS[h->cfg].cdiv == 2) ? 2 : 1;
    const int nvec = (lx + h->T.vec / cdiv - 1) / (h->T.vec / cdiv);
    const int gx = (nvec + 127) / 128;
    // 256 blocks of 128 threads each way keep the host link busy
    const int xrows = std::max(1, (env_int("BGK_PIPE_XFER", 256) + gx - 1) / gx);
    WaveArgs a{};
    if (in) a.in = *in;
    if (out) a.out = *out;
    a.band_rows = R;
    a.nbands = (ly + R - 1) / R;
    a.nsteps = K;
    a.cur0 = h->cur;
    a.xfer_rows = xrows;
    const int nb = a.nbands;
    const int last = (nb - 1) + 2 * K + (out ? 1 : 0);
    for (int w = 0; w <= last; ++w) {
        a.wave = w;
        a.up_band = (in && w < nb) ? w : -1;
        const int d = w - 2 * K - 1;
        a.down_band = (out && d >= 0 && d < nb) ? d : -1;
        a.k_lo = std::max(1, w - nb + 1 > 0 ? (w - nb + 2) / 2 : 1);
        a.k_hi = std::min(K, w / 2);
        const int nk = std::max(0, a.k_hi - a.k_lo + 1);
        const int gy = (a.up_band >= 0 ? xrows : 0) + (a.down_band >= 0 ? xrows : 0) + nk * R;
        if (gy > 0) {
            CK(h, h->T.wave(h->L, a, h->cs.has_obs, cdiv, gy, h->st));
            h->launches++;
        }
    }
    h->cur = (h->cur + K) & 1;
    h->itime += K;
    return BGK_OK;
}

int advance_impl(bgk_handle *h, void *const in[9], void *const out[9], int64_t ld, int32_t nsteps)
{
    const int l = h->desc.lx;
    if (!in || !out || ld < l + 2 || nsteps < 0) return fail(h, BGK_E_INVALID, "bad advance arguments");
    for (int q = 0; q < 9; ++q)
        if (!in[q] || !out[q]) return fail(h, BGK_E_INVALID, "population %d is NULL", q);
    if (h->streamed) return fail(h, BGK_E_INVALID, "two-pass step half done: call bgk_collision first");
    HostPlanes hin, hout;
    int rc;
    if (nsteps == 0 || !pipeline_ok(h) || !all_mapped(h, in, ld, hin) || !all_mapped(h, out, ld, hout)) {
        // the same three calls in sequence
        if ((rc = upload_impl(h, in, ld, false))) return rc;
        if ((rc = steps_impl(h, nsteps))) return rc;
        if ((rc = download_impl(h, out, ld))) return rc;
        return check_status(h);
    }
    if (nsteps <= 2 * PIPE_STEPS) {
        if ((rc = run_waves(h, &hin, &hout, nsteps))) return rc;
    } else {
        if ((rc = run_waves(h, &hin, nullptr, PIPE_STEPS))) return rc;
        if ((rc = steps_impl(h, nsteps - 2 * PIPE_STEPS))) return rc;
        if ((rc = run_waves(h, nullptr, &hout, PIPE_STEPS))) return rc;
    }
    CK(h, cudaStreamSynchronize(h->st));
    return check_status(h);
}

void release(bgk_handle *h)
{
    for (int i = 0; i < 2; ++i)
        if (h->graph[i]) cudaGraphExecDestroy(h->graph[i]);
    if (h->st) {
        for (void *p : {(void *)h->d_planes, (void *)h->d_mask, h->d_step_aux, (void *)h->d_inflow, (void *)h->d_partial,
                        (void *)h->d_out, (void *)h->d_status, (void *)h->d_uprev, (void *)h->d_vprev, h->d_stage})
            dfree(h, p);
        cudaStreamSynchronize(h->st);
    }
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->st) cudaStreamDestroy(h->st);
}

template <typename K>
std::string setup_for(const bgk_case_desc &d, CaseSetup &cs) { return setup_case<K>(d, cs); }

// one of the reference's profile readers on the device (kind as KernelTable::readers); n values
// per output array
int readers_impl(bgk_handle *h, int kind, int a, int b, double *o0, double *o1, double *o2, size_t n)
{
    double *d = nullptr;
    if (dalloc(h, &d, 3 * n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, BGK_E_NOMEM, "readers buffer");
    }
    cudaError_t e = h->T.readers(h->L, h->cur, h->phase, h->cs.has_obs, kind, a, b, d, h->st);
    h->launches++;
    double *outs[3] = {o0, o1, o2};
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaMemcpyAsync(outs[k], d + k * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    dfree(h, d);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) return fail(h, BGK_E_CUDA, "readers: %s", cudaGetErrorString(e));
    return BGK_OK;
}

}  // namespace

extern "C" {

const char *bgk_version(void) { return "bgk2d_gb300 1.0 (sm_103a)"; }

int bgk_default_desc(bgk_case_desc *d)
{
    if (!d) return BGK_E_INVALID;
    std::memset(d, 0, sizeof(*d));
    d->lx = 256; d->ly = 256;
    d->storage = BGK_STORE_F32;
    d->compute = BGK_COMPUTE_F32;
    d->scheme = BGK_SCHEME_PINGPONG;
    d->tcase = BGK_CASE_LDC;
    d->svisc = 0.1;
    d->u0 = 0.1;
    d->radius = 16;
    d->obs_icoord = -1;
    d->obs_jcoord = -1;
    d->tgv_u0 = 0.02;
    d->cte_s = 0.1;
    return BGK_OK;
}

int bgk_create(const bgk_case_desc *desc, bgk_handle **out)
{
    if (!desc || !out) return BGK_E_INVALID;
    *out = nullptr;
    const bgk_case_desc &d = *desc;
    if (d.lx < 2 || d.ly < 2 || d.ipad < 0 || d.jpad < 0) return BGK_E_INVALID;
    if (d.ly > BGK_MAX_LY) return BGK_E_TOOLARGE;  // ly + 2 grid rows must fit gridDim.y (65535)
    if (d.scheme != BGK_SCHEME_PINGPONG && d.scheme != BGK_SCHEME_AA && d.scheme != BGK_SCHEME_ORIGINAL)
        return BGK_E_INVALID;
    KernelTable T;
    if (!get_table(d.storage, d.compute, T)) return BGK_E_INVALID;

    bgk_handle *h = new bgk_handle();
    h->desc = d;
    h->desc.obs_mask = nullptr;
    h->dev = d.device;
    h->T = T;
    h->host_bytes = d.storage == BGK_STORE_F64 ? 8 : 4;
    std::string msg = d.compute == BGK_COMPUTE_F64 ? setup_for<double>(d, h->cs) : setup_for<float>(d, h->cs);
    if (!msg.empty()) {
        delete h;
        return BGK_E_INVALID;
    }
    if (enter_device(h->dev) != cudaSuccess) {
        delete h;
        return BGK_E_CUDA;
    }

    // geometry: interior cell x=1 starts a 16-byte vector; rows padded to 128 bytes
    const int l = d.lx, m = d.ly, vec = T.vec, eb = T.elem_bytes;
    const int nvec = (l + vec - 1) / vec;
    const int row_align = 128 / eb;
    int64_t pitch = (vec - 1) + 2 + (int64_t)(nvec + 1) * vec;
    pitch = (pitch + row_align - 1) / row_align * row_align;
    // an even number of rows per plane: every plane starts on a 256-byte boundary, and a plane is
    // a whole number of rows (the copy engines move the nine planes as one 3D copy)
    const int64_t plane = pitch * ((m + 2 + 1) / 2 * 2);
    const int nplanes = d.scheme == BGK_SCHEME_AA ? 9 : 18;
    h->planes_bytes = (size_t)plane * nplanes * eb;

    // admission against free HBM (populations + staging plane + mask + reduction scratch)
    const size_t stage = (size_t)(l + 2) * (m + 2) * h->host_bytes;
    const size_t mask_words = (size_t)((l + 2 + 31) / 32) * (m + 2);
    const size_t need = h->planes_bytes + stage + mask_words * 4 + (64u << 20);
    size_t free_b = 0, total_b = 0;
    const char *inj = std::getenv("BGK_FAULT_INJECT_NOMEM");
    if (inj && inj[0] == '1') { delete h; return BGK_E_NOMEM; }
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { delete h; return BGK_E_CUDA; }
    if (need > free_b) { delete h; return BGK_E_NOMEM; }

    if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess) {
        release(h); delete h; return BGK_E_CUDA;
    }
    if (dalloc(h, &h->d_planes, h->planes_bytes) != cudaSuccess) {
        cudaGetLastError(); release(h); delete h; return BGK_E_NOMEM;
    }
    cudaMemsetAsync(h->d_planes, 0, h->planes_bytes, h->st);

    Lattice &L = h->L;
    L.planes = h->d_planes;
    L.plane_elems = plane;
    L.pitch = (int32_t)pitch;
    L.lx = l; L.ly = m;
    L.nvec = nvec;
    L.scheme = d.scheme == BGK_SCHEME_AA ? BGK_SCHEME_AA : BGK_SCHEME_PINGPONG;  // layout
    h->two_pass = d.scheme == BGK_SCHEME_ORIGINAL;
    for (int f = 0; f < 4; ++f) {
        L.faces[f] = h->cs.faces[f];
        for (int q = 0; q < 9; ++q) L.wt[f][q] = h->cs.wt[f][q];
    }
    L.corner_x = h->cs.corner_x;
    L.noshift = h->cs.noshift;
    L.inflow_y0 = h->cs.inflow_y0;
    L.step_x = h->cs.bfs ? h->cs.stepx : 0;
    L.step_y = h->cs.bfs ? h->cs.stepy : 0;
    L.omega = h->cs.omega;
    L.fgrad = h->cs.fgrad;
    L.forced = h->cs.forced;
    L.les = h->cs.les;
    L.cte_s = h->cs.cte_s;
    L.omega_f = (float)L.omega;  // exact when the compute kind is FP32 (the values were computed in it)
    L.fgrad_f = (float)L.fgrad;
    L.cte_s_f = (float)L.cte_s;

    // inflow table
    if (dalloc(h, &h->d_inflow, h->cs.inflow.size() * sizeof(double)) != cudaSuccess) {
        cudaGetLastError(); release(h); delete h; return BGK_E_NOMEM;
    }
    cudaMemcpyAsync(h->d_inflow, h->cs.inflow.data(), h->cs.inflow.size() * sizeof(double), cudaMemcpyHostToDevice,
                    h->st);
    L.inflow = h->d_inflow;

    // obstacle bits, rows 0..m+1, bit x for x = 0..l+1
    L.mask_pitch = (l + 2 + 31) / 32;
    std::vector<uint32_t> bits((size_t)L.mask_pitch * (m + 2), 0u);
    for (int j = 1; j <= m; ++j)
        for (int i = 1; i <= l; ++i)
            if (h->cs.obs[(size_t)(i - 1) + (size_t)(j - 1) * l] == 1)
                bits[(size_t)j * L.mask_pitch + (i >> 5)] |= 1u << (i & 31);
    if (dalloc(h, &h->d_mask, bits.size() * 4) != cudaSuccess) {
        cudaGetLastError(); release(h); delete h; return BGK_E_NOMEM;
    }
    cudaMemcpyAsync(h->d_mask, bits.data(), bits.size() * 4, cudaMemcpyHostToDevice, h->st);
    cudaStreamSynchronize(h->st);  // `bits` and the inflow table are host temporaries
    L.mask = h->d_mask;
    L.step_aux = nullptr;
    if (h->cs.bfs && L.scheme == BGK_SCHEME_AA) {
        if (dalloc(h, &h->d_step_aux, 128) != cudaSuccess) {  // 10 storage elements
            cudaGetLastError(); release(h); delete h; return BGK_E_NOMEM;
        }
        cudaMemsetAsync(h->d_step_aux, 0, 128, h->st);
        L.step_aux = h->d_step_aux;
    }
    if (h->cs.has_obs) {
        L.ob_x0 = h->cs.bbox[0] - 1; L.ob_x1 = h->cs.bbox[1] + 1;
        L.ob_y0 = h->cs.bbox[2] - 1; L.ob_y1 = h->cs.bbox[3] + 1;
        if (h->cs.bfs) {  // and the step corner's neighbours (step_bounce)
            L.ob_x1 = std::max(L.ob_x1, h->cs.stepx + 1);
            L.ob_y1 = std::max(L.ob_y1, h->cs.stepy + 1);
        }
    } else {
        L.ob_x0 = L.ob_y0 = 1 << 30; L.ob_x1 = L.ob_y1 = -1;
    }

    // reduction scratch
    h->nb_red = 4 * 152;
    if (dalloc(h, &h->d_partial, (size_t)h->nb_red * 4 * sizeof(double)) != cudaSuccess ||
        dalloc(h, &h->d_out, 4 * sizeof(double)) != cudaSuccess ||
        dalloc(h, &h->d_status, sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError(); release(h); delete h; return BGK_E_NOMEM;
    }
    cudaMemsetAsync(h->d_status, 0, sizeof(uint32_t), h->st);
    L.status = h->d_status;
    const char *stall = std::getenv("BGK_FAULT_INJECT_STALL");
    L.inject_stall = (stall && stall[0] == '1') ? 1 : 0;
    L.pf_ahead = 0;
    h->cfg = default_cfg(nvec);

    // initial state (SRC/initialize.F90:85-125: init(init_v))
    int rc = BGK_OK;
    if (d.init_v == BGK_INIT_TGV) {
        // computed on the device: no host loop over the lattice at admission time
        if (h->T.init_tgv(h->L, d.tgv_u0, h->st) != cudaSuccess) rc = BGK_E_CUDA;
        h->launches++;
        if (rc == BGK_OK && d.scheme == BGK_SCHEME_AA &&
            (h->cs.faces[XHI] == FK_OUTFLOW_EQ || h->cs.faces[XHI] == FK_OUTFLOW_ZG)) {
            if (h->T.fill_outflow(h->L, h->st) != cudaSuccess) rc = BGK_E_CUDA;
        }
    } else if (d.init_v == BGK_INIT_TGV_REF || (d.init_v == BGK_INIT_REST && h->cs.noshift)) {
        // the reference's init (SRC/init.F90:83-137) on the host; the rest state of whole
        // populations is f = w, which the zeroed planes do not hold
        const bool vortex = d.init_v == BGK_INIT_TGV_REF, ns = h->cs.noshift != 0;
        const size_t n = (size_t)(l + 2) * (m + 2);
        void *ptrs[9];
        if (h->host_bytes == 8) {
            std::vector<double> a;
            init_reference<double, double>(l, m, vortex, a, ns);
            for (int q = 0; q < 9; ++q) ptrs[q] = a.data() + q * n;
            rc = upload_impl(h, ptrs, l + 2);
        } else {
            std::vector<float> a;
            if (d.compute == BGK_COMPUTE_F64) init_reference<double, float>(l, m, vortex, a, ns);
            else init_reference<float, float>(l, m, vortex, a, ns);
            for (int q = 0; q < 9; ++q) ptrs[q] = a.data() + q * n;
            rc = upload_impl(h, ptrs, l + 2);
        }
    } else if (d.init_v != BGK_INIT_REST) {
        rc = BGK_E_INVALID;
    }
    if (rc == BGK_OK && cudaStreamSynchronize(h->st) != cudaSuccess) rc = BGK_E_CUDA;
    if (rc != BGK_OK) { release(h); delete h; return rc; }
    *out = h;
    return BGK_OK;
}

int bgk_destroy(bgk_handle *h)
{
    if (!h) return BGK_E_INVALID;
    if (h->batch) bgk_batch_remove((bgk_batch *)h->batch, h);
    enter_device(h->dev);
    if (h->st) cudaStreamSynchronize(h->st);
    release(h);
    delete h;
    return BGK_OK;
}

int bgk_upload(bgk_handle *h, void *const pops[9], int64_t ld)
{
    CHECK_HANDLE(h);
    if (!pops) return BGK_E_INVALID;
    return upload_impl(h, pops, ld);
}

int bgk_download(bgk_handle *h, void *const pops[9], int64_t ld)
{
    CHECK_HANDLE(h);
    return download_impl(h, pops, ld);
}

int bgk_boundaries(bgk_handle *h)
{
    CHECK_HANDLE(h);
    return BGK_OK;  // folded into the step launched by bgk_propagation / bgk_collision
}

int bgk_propagation(bgk_handle *h)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    if (!h->two_pass || h->streamed) return BGK_OK;  // fused: the pull streaming is part of the step
    // two-pass: the streaming pass (with the boundary rules) now, the collision in
    // bgk_collision, as SRC/propagation.F90 and SRC/collision.F90 split them
    CK(h, h->T.step(STEP_STREAM, h->L, h->cur, h->cs.has_obs, h->cfg, h->st));
    h->launches++;
    h->streamed = true;
    return BGK_OK;
}

int bgk_collision(bgk_handle *h, int32_t itime)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    (void)itime;
    if (h->two_pass && h->streamed) {
        CK(h, h->T.step(STEP_COLLIDE, h->L, h->cur ^ 1, h->cs.has_obs, h->cfg, h->st));
        h->launches++;
        h->streamed = false;
        h->cur ^= 1;
        h->itime++;
        return BGK_OK;
    }
    return launch_step(h);
}

int bgk_step(bgk_handle *h, int32_t nsteps)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    return steps_impl(h, nsteps);
}

int bgk_step_timed(bgk_handle *h, int32_t nsteps, float *ms)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    if (!ms) return BGK_E_INVALID;
    CK(h, cudaEventRecord(h->ev0, h->st));
    int rc = steps_impl(h, nsteps);
    if (rc) return rc;
    CK(h, cudaEventRecord(h->ev1, h->st));
    CK(h, cudaEventSynchronize(h->ev1));
    CK(h, cudaEventElapsedTime(ms, h->ev0, h->ev1));
    return check_status(h);
}

int bgk_advance_host(bgk_handle *h, void *const in[9], void *const out[9], int64_t ld, int32_t nsteps)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    return advance_impl(h, in, out, ld, nsteps);
}

int bgk_sync(bgk_handle *h)
{
    CHECK_HANDLE(h);
    CK(h, cudaStreamSynchronize(h->st));
    return check_status(h);
}

int bgk_diagno(bgk_handle *h, int32_t fluid_only, double out[4])
{
    CHECK_HANDLE(h);
    if (!out || fluid_only < BGK_DIAGNO_ALL || fluid_only > BGK_DIAGNO_REFERENCE) return BGK_E_INVALID;
    if (fluid_only == BGK_DIAGNO_REFERENCE) {
        CK(h, h->T.diagno_seq(h->L, h->cur, h->phase, h->cs.has_obs, h->d_out, h->st));
        h->launches++;
        CK(h, cudaMemcpyAsync(out, h->d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
        CK(h, cudaStreamSynchronize(h->st));
        if (int rc = check_status(h)) return rc;
        for (int i = 0; i < 4; ++i)
            if (!std::isfinite(out[i])) return fail(h, BGK_E_NUMERIC, "diagno: non-finite mean");
        return BGK_OK;
    }
    CK(h, h->T.diagno(h->L, h->cur, h->phase, fluid_only, h->cs.has_obs, h->d_partial, h->nb_red, h->st));
    h->launches++;
    double s[4];
    int rc = reduce4(h, s);
    if (rc) return rc;
    const double l = h->desc.lx, m = h->desc.ly;
    for (int i = 0; i < 4; ++i) out[i] = (s[i] / l) / m;  // SRC/diagno.F90:98-101
    for (int i = 0; i < 4; ++i)
        if (!std::isfinite(s[i])) return fail(h, BGK_E_NUMERIC, "diagno: non-finite sum");
    return BGK_OK;
}

int bgk_residual(bgk_handle *h, double *out)
{
    CHECK_HANDLE(h);
    if (!out) return BGK_E_INVALID;
    const size_t n = (size_t)h->desc.lx * h->desc.ly;
    bool first = false;
    if (!h->d_uprev) {
        if (dalloc(h, &h->d_uprev, n * sizeof(double)) != cudaSuccess ||
            dalloc(h, &h->d_vprev, n * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, BGK_E_NOMEM, "residual snapshot");
        }
        CK(h, cudaMemsetAsync(h->d_uprev, 0, n * sizeof(double), h->st));
        CK(h, cudaMemsetAsync(h->d_vprev, 0, n * sizeof(double), h->st));
        first = true;
    }
    CK(h, h->T.residual(h->L, h->cur, h->phase, h->cs.has_obs, h->d_uprev, h->d_vprev, h->d_partial, h->nb_red, h->st));
    h->launches++;
    double s[4];
    int rc = reduce4(h, s);
    if (rc) return rc;
    const int64_t dt = h->itime - h->res_itime;
    h->res_itime = h->itime;
    if (s[2] != 0.0 || !std::isfinite(s[0]) || !std::isfinite(s[1])) {
        *out = NAN;
        return fail(h, BGK_E_NUMERIC, "residual: non-finite velocity");
    }
    if (first || dt <= 0) *out = 1.0;
    else *out = (s[1] > 0 ? std::sqrt(s[0] / s[1]) : (s[0] > 0 ? 1.0 : 0.0)) / (double)dt;
    return BGK_OK;
}

int bgk_draglift_reference(bgk_handle *h, double out[2])
{
    CHECK_HANDLE(h);
    if (!out) return BGK_E_INVALID;
    if (!h->cs.has_obs) return fail(h, BGK_E_UNSUPPORTED, "draglift needs an obstacle");
    const int l = h->desc.lx, m = h->desc.ly, r = h->cs.radius, delta = 3;
    int i0 = h->cs.icoord - r - delta, i1 = h->cs.icoord + r + delta;
    int j0 = h->cs.jcoord - r - delta, j1 = h->cs.jcoord + r + delta;
    i0 = std::max(i0, 1); j0 = std::max(j0, 1); i1 = std::min(i1, l); j1 = std::min(j1, m);
    double norm;  // uno / (u_inflow * u_inflow * radius) in the compute kind
    if (h->desc.compute == BGK_COMPUTE_F64) {
        const double u = h->cs.u_inflow;
        norm = 1.0 / ((u * u) * (double)r);
    } else {
        const float u = (float)h->cs.u_inflow;
        norm = (double)(1.0f / ((u * u) * (float)r));
    }
    CK(h, h->T.draglift_seq(h->L, h->cur, h->phase, i0, i1, j0, j1, norm, h->d_out, h->st));
    h->launches++;
    CK(h, cudaMemcpyAsync(out, h->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(h, cudaStreamSynchronize(h->st));
    return check_status(h);
}

int bgk_draglift(bgk_handle *h, double out[2])
{
    CHECK_HANDLE(h);
    if (!out) return BGK_E_INVALID;
    if (!h->cs.has_obs) return fail(h, BGK_E_UNSUPPORTED, "draglift needs an obstacle");
    const int l = h->desc.lx, m = h->desc.ly, r = h->cs.radius, delta = 3;
    int i0 = h->cs.icoord - r - delta, i1 = h->cs.icoord + r + delta;
    int j0 = h->cs.jcoord - r - delta, j1 = h->cs.jcoord + r + delta;
    i0 = std::max(i0, 1); j0 = std::max(j0, 1); i1 = std::min(i1, l); j1 = std::min(j1, m);
    CK(h, h->T.draglift(h->L, h->cur, h->phase, i0, i1, j0, j1, h->d_partial, h->nb_red, h->st));
    h->launches++;
    double s[4];
    int rc = reduce4(h, s);
    if (rc) return rc;
    double norm;
    if (h->desc.compute == BGK_COMPUTE_F64) {
        const double u = h->cs.u_inflow;
        norm = 1.0 / ((u * u) * (double)r);
    } else {
        const float u = (float)h->cs.u_inflow;
        norm = (double)(1.0f / ((u * u) * (float)r));
    }
    out[0] = s[0] * norm;
    out[1] = s[1] * norm;
    return BGK_OK;
}

int bgk_fields(bgk_handle *h, double *rho, double *u, double *v)
{
    CHECK_HANDLE(h);
    if (!rho || !u || !v) return BGK_E_INVALID;
    const size_t n = (size_t)h->desc.lx * h->desc.ly;
    double *d = nullptr;
    if (dalloc(h, &d, 3 * n * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, BGK_E_NOMEM, "fields buffer");
    }
    cudaError_t e = h->T.fields(h->L, h->cur, h->phase, h->cs.has_obs, d, d + n, d + 2 * n, h->st);
    h->launches++;
    if (e == cudaSuccess) e = cudaMemcpyAsync(rho, d, n * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(u, d + n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v, d + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, h->st);
    dfree(h, d);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) return fail(h, BGK_E_CUDA, "fields: %s", cudaGetErrorString(e));
    return BGK_OK;
}

int bgk_prof_i(bgk_handle *h, int32_t jcoord, double *u, double *v, double *den)
{
    CHECK_HANDLE(h);
    if (!u || !v || !den || jcoord < 1 || jcoord > h->desc.ly) return fail(h, BGK_E_INVALID, "prof_i arguments");
    return readers_impl(h, 0, jcoord, 0, u, v, den, (size_t)h->desc.lx);
}

int bgk_prof_j(bgk_handle *h, int32_t icoord, double *u, double *v, double *den)
{
    CHECK_HANDLE(h);
    if (!u || !v || !den || icoord < 1 || icoord > h->desc.lx) return fail(h, BGK_E_INVALID, "prof_j arguments");
    return readers_impl(h, 1, icoord, 0, u, v, den, (size_t)h->desc.ly);
}

int bgk_varm(bgk_handle *h, double *u, double *w, double *den)
{
    CHECK_HANDLE(h);
    if (!u || !w || !den) return fail(h, BGK_E_INVALID, "varm arguments");
    return readers_impl(h, 2, 0, 0, u, w, den, (size_t)h->desc.ly);
}

int bgk_probe(bgk_handle *h, int32_t i0, int32_t j0, double out[3])
{
    CHECK_HANDLE(h);
    if (!out || i0 < 1 || i0 > h->desc.lx || j0 < 1 || j0 > h->desc.ly) return fail(h, BGK_E_INVALID, "probe arguments");
    return readers_impl(h, 3, i0, j0, out, out + 1, out + 2, 1);
}

int bgk_vtk_fields(bgk_handle *h, float *u, float *w, float *rho, float *vort, float *stream)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    const int l = h->desc.lx, m = h->desc.ly;
    if (l < 3 || m < 3) return fail(h, BGK_E_INVALID, "vtk fields need lx, ly >= 3");
    const size_t n = (size_t)l * m, n2 = (size_t)(l - 2) * (m - 2);
    float *d = nullptr;
    if (dalloc(h, &d, (3 * n + 2 * n2 + (size_t)m + 2) * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, BGK_E_NOMEM, "vtk fields buffer");
    }
    float *du = d, *dw = d + n, *dr = d + 2 * n, *dv = d + 3 * n, *ds = dv + n2, *dphi = ds + n2;
    cudaError_t e = h->T.vtk(h->L, h->cur, h->phase, h->cs.has_obs, du, dw, dr, dv, ds, dphi, h->st);
    h->launches += 3;
    const std::pair<float *, const float *> out[5] = {{u, du}, {w, dw}, {rho, dr}, {vort, dv}, {stream, ds}};
    for (int k = 0; k < 5 && e == cudaSuccess; ++k)
        if (out[k].first)
            e = cudaMemcpyAsync(out[k].first, out[k].second, (k < 3 ? n : n2) * sizeof(float), cudaMemcpyDeviceToHost,
                                h->st);
    dfree(h, d);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    if (e != cudaSuccess) return fail(h, BGK_E_CUDA, "vtk fields: %s", cudaGetErrorString(e));
    return BGK_OK;
}

int bgk_get_obs(bgk_handle *h, int32_t *mask, int32_t bbox[5])
{
    if (!h || !bbox) return BGK_E_INVALID;
    if (mask) std::memcpy(mask, h->cs.obs.data(), h->cs.obs.size() * sizeof(int32_t));
    for (int i = 0; i < 5; ++i) bbox[i] = h->cs.bbox[i];
    return BGK_OK;
}

int bgk_get_scalars(bgk_handle *h, double out[4], int64_t *itime)
{
    if (!h || !out) return BGK_E_INVALID;
    out[0] = h->cs.omega; out[1] = h->cs.fgrad; out[2] = h->cs.u00; out[3] = h->cs.u0;
    if (itime) *itime = h->itime;
    return BGK_OK;
}

int bgk_footprint(bgk_handle *h, int64_t *device_bytes, int32_t *bytes_per_cell)
{
    if (!h) return BGK_E_INVALID;
    if (device_bytes) *device_bytes = (int64_t)(h->planes_bytes + h->stage_bytes);
    if (bytes_per_cell) *bytes_per_cell = 18 * h->T.elem_bytes;
    return BGK_OK;
}

int bgk_set_tile(bgk_handle *h, int32_t tile_cfg)
{
    CHECK_HANDLE(h);
    const int ncfg = (h->L.scheme == BGK_SCHEME_PINGPONG && !h->two_pass) ? NUM_STEP_CFG : NUM_CFG;
    if (tile_cfg < 0 || tile_cfg >= ncfg) return fail(h, BGK_E_INVALID, "tile configuration %d", tile_cfg);
    if (tile_cfg != h->cfg) {
        for (int i = 0; i < 2; ++i)
            if (h->graph[i]) { cudaGraphExecDestroy(h->graph[i]); h->graph[i] = nullptr; }
        h->cfg = tile_cfg;
    }
    return BGK_OK;
}

int bgk_set_prefetch(bgk_handle *h, int32_t blocks_ahead)
{
    CHECK_HANDLE(h);
    if (blocks_ahead < 0) return fail(h, BGK_E_INVALID, "negative prefetch distance");
    if (blocks_ahead != h->L.pf_ahead) {
        for (int i = 0; i < 2; ++i)
            if (h->graph[i]) { cudaGraphExecDestroy(h->graph[i]); h->graph[i] = nullptr; }
        h->L.pf_ahead = blocks_ahead;
    }
    return BGK_OK;
}

int bgk_get_prefetch(bgk_handle *h, int32_t *blocks_ahead)
{
    if (!h || !blocks_ahead) return BGK_E_INVALID;
    *blocks_ahead = h->L.pf_ahead;
    return BGK_OK;
}

int bgk_tune(bgk_handle *h, int32_t trial_steps, int32_t *tile_cfg, int32_t *steps_run)
{
    CHECK_HANDLE(h);
    NOT_IN_BATCH(h);
    if (trial_steps < 2) return fail(h, BGK_E_INVALID, "trial_steps < 2");
    const int n = trial_steps & ~1;
    float best = 1e30f;
    int best_cfg = h->cfg, best_pf = h->L.pf_ahead, rc;
    int64_t run = 0;
    int sms = 0;
    CK(h, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->dev));
    // L2 prefetch distances for the register-vector ping-pong and AA kernels: off, half a wave
    // and one wave of 8 resident blocks per SM ahead
    const int pfs[3] = {0, 4 * sms, 8 * sms};
    const int ncfg = (h->L.scheme == BGK_SCHEME_PINGPONG && !h->two_pass) ? NUM_STEP_CFG : NUM_CFG;
    // AA with 16-bit storage rounds each value that crosses a warp edge on its own, and where
    // the warp edges fall depends on the bytes per thread.  Only the 8-byte shapes (4, 5) are
    // tried, so the populations of a tuned run do not depend on which of them wins.
    const bool aa16 = h->L.scheme == BGK_SCHEME_AA && h->T.elem_bytes == 2;
    // A handle with the Smagorinsky collision runs one kernel shape whatever the tile
    // configuration, except 16-bit ping-pong, whose configurations 0-3 are register budgets of
    // its LES kernel and 4-5 its staged forms; otherwise only the prefetch distance is tried.
    const bool les16 = h->L.les && h->T.elem_bytes == 2 && h->L.scheme == BGK_SCHEME_PINGPONG && !h->two_pass;
    const int c0 = les16 ? 0 : h->L.les ? h->cfg : aa16 ? 4 : 0;
    const int c1 = les16 ? 6 : h->L.les ? h->cfg + 1 : ncfg;
    for (int c = c0; c < c1; ++c) {
        const bool staged = c >= NUM_CFG || (les16 && c >= 4);
        const int npf = staged ? 1 : 3;
        for (int p = 0; p < npf; ++p) {
            if ((rc = bgk_set_tile(h, c)) || (rc = bgk_set_prefetch(h, pfs[p]))) return rc;
            for (int s = 0; s < 2; ++s)
                if ((rc = launch_step(h))) return rc;
            float ms = 0;
            CK(h, cudaEventRecord(h->ev0, h->st));
            for (int s = 0; s < n; ++s)
                if ((rc = launch_step(h))) return rc;
            CK(h, cudaEventRecord(h->ev1, h->st));
            CK(h, cudaEventSynchronize(h->ev1));
            CK(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
            run += n + 2;
            if (ms < best) { best = ms; best_cfg = c; best_pf = pfs[p]; }
        }
    }
    if ((rc = bgk_set_tile(h, best_cfg)) || (rc = bgk_set_prefetch(h, best_pf))) return rc;
    if (tile_cfg) *tile_cfg = best_cfg;
    if (steps_run) *steps_run = (int32_t)run;
    return BGK_OK;
}

int bgk_launch_count(bgk_handle *h, int64_t *launches)
{
    if (!h || !launches) return BGK_E_INVALID;
    *launches = h->launches;
    return BGK_OK;
}

int bgk_last_error(bgk_handle *h, char *buf, size_t len)
{
    if (!h || !buf || len == 0) return BGK_E_INVALID;
    std::snprintf(buf, len, "%s", h->err.c_str());
    return BGK_OK;
}

}  // extern "C"
