// bgk_batch.cu -- many independent lattices advanced by one persistent launch per time step.
//
// The reference advances one domain per run (SRC/bgk2d.F90:92-113).  A batch keeps any number
// of ping-pong handles of the same (storage, compute) kind resident; one kernel per time step
// covers a work list of row-segment tiles over all of them, either as one block per tile
// (batch_pp_flat_kernel, with an L2 prefetch of the tile a set distance ahead) or as a
// persistent grid walking contiguous chunks (batch_pp_kernel), and the step loop is replayed
// from CUDA graphs.  Tile shape, grid form, prefetch distance and steps per graph are chosen by
// bgk_batch_tune from timed trial steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "bgk_handle.h"

using namespace bgk;

struct bgk_batch {
    int storage = 0, compute = 0, dev = 0;
    KernelTable T{};
    std::vector<bgk_handle *> members;
    Lattice *d_lats = nullptr;
    int *d_cur = nullptr;
    int4 *d_tiles = nullptr;
    int ntiles = 0;
    size_t cap_lats = 0, cap_tiles = 0;
    int nles = 0;                   // LES members' tiles, stored after the ntiles others
    bool dirty = true;              // work list / device arrays need a rebuild
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr, ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_built_for = -1;       // generation the graph was captured for
    int generation = 0;
    int cfg = 2;                    // tile shape index (TILE_CFGS)
    int blocks_per_sm = 8;
    int graph_steps = 32;           // even
    int pf = 0;                     // one-block-per-tile kernel: L2 prefetch this many tiles ahead
    int sms = 152;
    int64_t launches = 0;
    int64_t steps = 0;
};

namespace {

int rebuild(bgk_batch *b)
{
    if (!b->dirty) return BGK_OK;
    const TileCfg tc = TILE_CFGS[b->cfg];
    std::vector<Lattice> lats;
    std::vector<int> cur;
    std::vector<int4> tiles, les_tiles;
    for (size_t i = 0; i < b->members.size(); ++i) {
        bgk_handle *h = b->members[i];
        lats.push_back(h->L);
        cur.push_back(h->cur);
        // LES members: the Smagorinsky kernel's own shape (128 x 1 threads, the cells per
        // thread of the single-domain LES step), in a list of their own
        const bool les = h->L.les != 0;
        const int txv = les ? 128 : tc.txv, ty = les ? 1 : tc.ty;
        const int n = les ? (b->T.elem_bytes == 2 ? b->T.vec / 2 : b->T.vec) : b->T.vec / tc.cdiv;
        const int nv = (h->L.lx + n - 1) / n;
        const int gx = (nv + txv - 1) / txv, gy = (h->L.ly + ty - 1) / ty;
        // the lattice's last tile row (boundary-rule cells) second, as tile_row() orders single
        // domains, so that it does not trail its lattice's work
        for (int b = 0; b < gy; ++b) {
            const int by = (gy < 2 || b == 0) ? b : (b == 1 ? gy - 1 : b - 1);
            for (int bx = 0; bx < gx; ++bx) (les ? les_tiles : tiles).push_back(make_int4((int)i, bx, by, 0));
        }
    }
    const size_t nplain = tiles.size();
    tiles.insert(tiles.end(), les_tiles.begin(), les_tiles.end());  // LES entries after the others
    // a failed allocation leaves the pointers null and the capacity 0, so a later rebuild retries
    // the allocation and never frees an array twice
    if (lats.size() > b->cap_lats) {
        if (b->d_lats) cudaFreeAsync(b->d_lats, b->st);
        if (b->d_cur) cudaFreeAsync(b->d_cur, b->st);
        b->d_lats = nullptr;
        b->d_cur = nullptr;
        b->cap_lats = std::max<size_t>(lats.size(), 2 * b->cap_lats);
        const cudaError_t e1 = cudaMallocAsync((void **)&b->d_lats, b->cap_lats * sizeof(Lattice), b->st);
        const cudaError_t e2 =
            e1 == cudaSuccess ? cudaMallocAsync((void **)&b->d_cur, b->cap_lats * sizeof(int), b->st) : e1;
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            cudaGetLastError();
            if (e1 == cudaSuccess) cudaFreeAsync(b->d_lats, b->st);
            b->d_lats = nullptr;
            b->d_cur = nullptr;
            b->cap_lats = 0;
            return BGK_E_NOMEM;
        }
    }
    if (tiles.size() > b->cap_tiles) {
        if (b->d_tiles) cudaFreeAsync(b->d_tiles, b->st);
        b->d_tiles = nullptr;
        b->cap_tiles = std::max<size_t>(tiles.size(), 2 * b->cap_tiles);
        if (cudaMallocAsync((void **)&b->d_tiles, b->cap_tiles * sizeof(int4), b->st) != cudaSuccess) {
            cudaGetLastError();
            b->d_tiles = nullptr;
            b->cap_tiles = 0;
            return BGK_E_NOMEM;
        }
    }
    if (!lats.empty()) {
        if (cudaMemcpyAsync(b->d_lats, lats.data(), lats.size() * sizeof(Lattice), cudaMemcpyHostToDevice, b->st) ||
            cudaMemcpyAsync(b->d_cur, cur.data(), cur.size() * sizeof(int), cudaMemcpyHostToDevice, b->st) ||
            cudaMemcpyAsync(b->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, b->st))
            return BGK_E_CUDA;
    }
    if (cudaStreamSynchronize(b->st) != cudaSuccess) return BGK_E_CUDA;
    b->ntiles = (int)nplain;
    b->nles = (int)les_tiles.size();
    b->dirty = false;
    b->generation++;
    return BGK_OK;
}

int sync_cur(bgk_batch *b)
{
    std::vector<int> cur;
    for (auto *h : b->members) cur.push_back(h->cur);
    if (cur.empty()) return BGK_OK;
    if (cudaMemcpyAsync(b->d_cur, cur.data(), cur.size() * sizeof(int), cudaMemcpyHostToDevice, b->st) != cudaSuccess)
        return BGK_E_CUDA;
    return cudaStreamSynchronize(b->st) == cudaSuccess ? BGK_OK : BGK_E_CUDA;
}

// blocks_per_sm == 0 selects one block per tile
int grid_of(const bgk_batch *b)
{
    if (b->blocks_per_sm == 0) return 0;
    return std::max(1, std::min(b->ntiles, b->blocks_per_sm * b->sms));
}

int launch_one(bgk_batch *b, int parity)
{
    if (b->ntiles == 0 && b->nles == 0) return BGK_OK;
    if (b->ntiles > 0) {
        if (b->T.batch_step(b->d_lats, b->d_cur, b->d_tiles, b->ntiles, parity, b->cfg, grid_of(b), b->pf, b->st) !=
            cudaSuccess)
            return BGK_E_CUDA;
        b->launches++;
    }
    if (b->nles > 0) {  // members with the Smagorinsky collision: their own launch of the same step
        if (b->T.batch_les(b->d_lats, b->d_cur, b->d_tiles + b->ntiles, b->nles, parity, b->st) != cudaSuccess)
            return BGK_E_CUDA;
        b->launches++;
    }
    return BGK_OK;
}

int capture(bgk_batch *b)
{
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return BGK_E_CUDA;
    const int64_t l0 = b->launches;
    int rc = BGK_OK;
    for (int s = 0; s < b->graph_steps && rc == BGK_OK; ++s) rc = launch_one(b, s & 1);
    b->launches = l0;
    cudaError_t e = cudaStreamEndCapture(b->st, &g);
    if (rc != BGK_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc != BGK_OK ? rc : BGK_E_CUDA;
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return BGK_E_CUDA;
    b->graph_built_for = b->generation;
    return BGK_OK;
}

void advance_members(bgk_batch *b, int n)
{
    for (auto *h : b->members) {
        h->itime += n;
        h->launches += n;
        if (n & 1) h->cur ^= 1;
    }
    b->steps += n;
}

int step_impl(bgk_batch *b, int n, bool use_graph)
{
    int rc = rebuild(b);
    if (rc) return rc;
    if (b->members.empty() || n <= 0) return BGK_OK;
    if (use_graph) {
        while (n >= b->graph_steps) {
            if (b->graph_built_for != b->generation && (rc = capture(b))) return rc;
            if (cudaGraphLaunch(b->graph, b->st) != cudaSuccess) return BGK_E_CUDA;
            b->launches += (int64_t)b->graph_steps * ((b->ntiles > 0) + (b->nles > 0));
            advance_members(b, b->graph_steps);  // graph_steps is even: buffers unchanged
            n -= b->graph_steps;
        }
    }
    for (int s = 0; s < n; ++s)
        if ((rc = launch_one(b, s & 1))) return rc;
    advance_members(b, n);
    if (n & 1) {
        // members flipped buffers: refresh the device copy before the next launch
        if (cudaStreamSynchronize(b->st) != cudaSuccess) return BGK_E_CUDA;
        if ((rc = sync_cur(b))) return rc;
    }
    if (cudaEventRecord(b->done, b->st) != cudaSuccess) return BGK_E_CUDA;
    return BGK_OK;
}

}  // namespace

extern "C" {

int bgk_batch_create(int32_t storage, int32_t compute, int32_t device, bgk_batch **out)
{
    if (!out) return BGK_E_INVALID;
    *out = nullptr;
    bgk_batch *b = new bgk_batch();
    b->storage = storage;
    b->compute = compute;
    b->dev = device;
    bgk_case_desc d;
    bgk_default_desc(&d);
    d.lx = d.ly = 8;
    d.storage = storage;
    d.compute = compute;
    d.device = device;
    // the kernel table comes from a probe handle of the same kind
    bgk_handle *probe = nullptr;
    if (enter_device(device) != cudaSuccess) { delete b; return BGK_E_CUDA; }
    int rc = bgk_create(&d, &probe);
    if (rc) { delete b; return rc; }
    b->T = probe->T;
    bgk_destroy(probe);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
        delete b;
        return BGK_E_CUDA;
    }
    *out = b;
    return BGK_OK;
}

int bgk_batch_destroy(bgk_batch *b)
{
    if (!b) return BGK_E_INVALID;
    enter_device(b->dev);
    cudaStreamSynchronize(b->st);
    for (auto *h : b->members) { h->batch = nullptr; h->wait_ev = nullptr; }
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->d_lats) cudaFreeAsync(b->d_lats, b->st);
    if (b->d_cur) cudaFreeAsync(b->d_cur, b->st);
    if (b->d_tiles) cudaFreeAsync(b->d_tiles, b->st);
    cudaStreamSynchronize(b->st);
    if (b->done) cudaEventDestroy(b->done);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return BGK_OK;
}

int bgk_batch_add(bgk_batch *b, bgk_handle *h)
{
    if (!b || !h) return BGK_E_INVALID;
    if (h->batch) return BGK_E_INVALID;
    if (h->desc.storage != b->storage || h->desc.compute != b->compute || h->dev != b->dev ||
        h->L.scheme != BGK_SCHEME_PINGPONG)
        return BGK_E_INVALID;
    // the batch kernels carry the fused one-pass step of deviations; a backward-facing step's
    // boundary routine and the Smagorinsky members' step run as batched launches of their own
    if (h->two_pass || h->L.noshift) return BGK_E_UNSUPPORTED;
    if (h->sticky) return h->sticky;
    enter_device(b->dev);
    if (cudaStreamSynchronize(h->st) != cudaSuccess || cudaStreamSynchronize(b->st) != cudaSuccess) return BGK_E_CUDA;
    b->members.push_back(h);
    h->batch = b;
    h->wait_ev = b->done;
    b->dirty = true;
    return BGK_OK;
}

int bgk_batch_remove(bgk_batch *b, bgk_handle *h)
{
    if (!b || !h) return BGK_E_INVALID;
    auto it = std::find(b->members.begin(), b->members.end(), h);
    if (it == b->members.end()) return BGK_E_NOTFOUND;
    enter_device(b->dev);
    // detached even when the batch's stream reports a failure: bgk_destroy frees the handle next,
    // and the batch must not keep a pointer to it
    const bool ok = cudaStreamSynchronize(b->st) == cudaSuccess;
    b->members.erase(it);
    h->batch = nullptr;
    h->wait_ev = nullptr;
    b->dirty = true;
    return ok ? BGK_OK : BGK_E_CUDA;
}

int bgk_batch_size(bgk_batch *b, int32_t *members, int64_t *cells)
{
    if (!b) return BGK_E_INVALID;
    int64_t c = 0;
    for (auto *h : b->members) c += (int64_t)h->desc.lx * h->desc.ly;
    if (members) *members = (int32_t)b->members.size();
    if (cells) *cells = c;
    return BGK_OK;
}

int bgk_batch_step(bgk_batch *b, int32_t nsteps)
{
    if (!b || nsteps < 0) return BGK_E_INVALID;
    if (enter_device(b->dev) != cudaSuccess) return BGK_E_CUDA;
    return step_impl(b, nsteps, true);
}

int bgk_batch_step_timed(bgk_batch *b, int32_t nsteps, float *ms)
{
    if (!b || !ms || nsteps < 0) return BGK_E_INVALID;
    if (enter_device(b->dev) != cudaSuccess) return BGK_E_CUDA;
    int rc = rebuild(b);
    if (rc) return rc;
    if (cudaEventRecord(b->ev0, b->st) != cudaSuccess) return BGK_E_CUDA;
    if ((rc = step_impl(b, nsteps, true))) return rc;
    if (cudaEventRecord(b->ev1, b->st) != cudaSuccess || cudaEventSynchronize(b->ev1) != cudaSuccess ||
        cudaEventElapsedTime(ms, b->ev0, b->ev1) != cudaSuccess)
        return BGK_E_CUDA;
    return BGK_OK;
}

int bgk_batch_sync(bgk_batch *b)
{
    if (!b) return BGK_E_INVALID;
    enter_device(b->dev);
    return cudaStreamSynchronize(b->st) == cudaSuccess ? BGK_OK : BGK_E_CUDA;
}

int bgk_batch_set_config(bgk_batch *b, int32_t tile_cfg, int32_t blocks_per_sm, int32_t graph_steps)
{
    if (!b || tile_cfg < 0 || tile_cfg >= NUM_CFG || blocks_per_sm < 0 || graph_steps < 2 || (graph_steps & 1))
        return BGK_E_INVALID;
    if (tile_cfg != b->cfg) b->dirty = true;
    if (tile_cfg != b->cfg || blocks_per_sm != b->blocks_per_sm || graph_steps != b->graph_steps) b->graph_built_for = -1;
    b->cfg = tile_cfg;
    b->blocks_per_sm = blocks_per_sm;
    b->graph_steps = graph_steps;
    return BGK_OK;
}

int bgk_batch_set_prefetch(bgk_batch *b, int32_t tiles_ahead)
{
    if (!b || tiles_ahead < 0) return BGK_E_INVALID;
    if (tiles_ahead != b->pf) b->graph_built_for = -1;
    b->pf = tiles_ahead;
    return BGK_OK;
}

int bgk_batch_get_config(bgk_batch *b, int32_t out[3])
{
    if (!b || !out) return BGK_E_INVALID;
    out[0] = b->cfg; out[1] = b->blocks_per_sm; out[2] = b->graph_steps;
    return BGK_OK;
}

// Autotuner: times `trial_steps` real steps (they advance the members) for every tile shape and
// persistent grid size (and, with one block per tile, L2 prefetch distance), then the
// steps-per-graph candidates, and keeps the fastest.
int bgk_batch_tune(bgk_batch *b, int32_t trial_steps, int32_t *steps_run)
{
    if (!b || trial_steps < 2) return BGK_E_INVALID;
    if (enter_device(b->dev) != cudaSuccess) return BGK_E_CUDA;
    int64_t run = 0;
    const int bps_opts[4] = {0, 4, 8, 16};
    float best = 1e30f;
    int best_cfg = b->cfg, best_bps = b->blocks_per_sm, best_pf = b->pf;
    const int n = trial_steps & ~1;
    const int pf_opts[3] = {0, 4 * b->sms, 8 * b->sms};
    for (int c = 0; c < NUM_CFG; ++c) {
        for (int bi = 0; bi < 6; ++bi) {
            const int bps = bps_opts[bi < 3 ? 0 : bi - 2], pf = bi < 3 ? pf_opts[bi] : 0;
            int rc = bgk_batch_set_config(b, c, bps, b->graph_steps);
            if (rc || (rc = bgk_batch_set_prefetch(b, pf))) return rc;
            if ((rc = rebuild(b))) return rc;
            if ((rc = step_impl(b, 2, false))) return rc;  // warm-up at this shape
            run += 2;
            if (cudaEventRecord(b->ev0, b->st) != cudaSuccess) return BGK_E_CUDA;
            if ((rc = step_impl(b, n, false))) return rc;
            run += n;
            float ms = 0;
            if (cudaEventRecord(b->ev1, b->st) != cudaSuccess || cudaEventSynchronize(b->ev1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, b->ev0, b->ev1) != cudaSuccess)
                return BGK_E_CUDA;
            if (ms < best) { best = ms; best_cfg = c; best_bps = bps; best_pf = pf; }
        }
    }
    const int g_opts[3] = {8, 32, 128};
    float gbest = 1e30f;
    int best_g = b->graph_steps;
    if (int rc = bgk_batch_set_prefetch(b, best_pf)) return rc;
    for (int gi = 0; gi < 3; ++gi) {
        int rc = bgk_batch_set_config(b, best_cfg, best_bps, g_opts[gi]);
        if (rc) return rc;
        const int m = std::max(g_opts[gi], n) / g_opts[gi] * g_opts[gi];
        if ((rc = step_impl(b, g_opts[gi], true))) return rc;  // capture + warm-up
        run += g_opts[gi];
        float ms = 0;
        if ((rc = bgk_batch_step_timed(b, m, &ms))) return rc;
        run += m;
        const float per = ms / m;
        if (per < gbest) { gbest = per; best_g = g_opts[gi]; }
    }
    int rc = bgk_batch_set_config(b, best_cfg, best_bps, best_g);
    if (rc) return rc;
    if (steps_run) *steps_run = (int32_t)run;
    return BGK_OK;
}

int bgk_batch_launch_count(bgk_batch *b, int64_t *launches)
{
    if (!b || !launches) return BGK_E_INVALID;
    *launches = b->launches;
    return BGK_OK;
}

}  // extern "C"
