// bgk_serve.cpp -- continuous-batching request loop over the C ABI.
//
// A scheduler thread admits submitted solves (FIFO) while slots and HBM allow, attaches each
// to the batch of its storage kind, and advances every batch in rounds of steps; batches of
// different kinds run on their own streams, so their work overlaps.  A round never crosses a
// request's next residual check or its step budget, so every request is checked at the same
// step counts (multiples of its check_every) whatever else is resident, and its result is the
// same alone and in a mix.  Finished requests are detached, reduced, and freed.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bgk2d_gb300.h"

namespace {

using clk = std::chrono::steady_clock;

struct Job {
    int64_t id;
    bgk_request req;
    bgk_result res;
    bgk_handle *h = nullptr;
    int64_t bytes = 0;
    int64_t charged = 0;  // bytes counted in the server's `used` while the job holds them
    int32_t steps = 0;
    int32_t lx = 0, ly = 0;
    bool res_started = false;
    std::vector<double> rho, u, v;
};

int store_bytes(int storage) { return storage == BGK_STORE_F64 ? 8 : (storage == BGK_STORE_F32 ? 4 : 2); }

void geometry(const bgk_request &r, int32_t &lx, int32_t &ly)
{
    if (r.kind == BGK_REQ_CYLINDER) { lx = 16 * r.n; ly = 4 * r.n; }
    else { lx = r.n; ly = r.n; }
}

// device bytes a request will hold: ping-pong planes, staging plane, residual snapshot, mask
int64_t estimate_bytes(const bgk_request &r)
{
    int32_t lx, ly;
    geometry(r, lx, ly);
    const int64_t eb = store_bytes(r.storage);
    const int64_t pitch = ((lx + 32) * eb + 127) / 128 * 128;
    const int64_t planes = 18 * pitch * (ly + 2);
    const int64_t stage = (int64_t)(lx + 2) * (ly + 2) * 4;
    const int64_t snap = (int64_t)lx * ly * 16;
    return planes + stage + snap + (int64_t)(ly + 2) * ((lx + 33) / 32) * 4 + (1 << 20);
}

}  // namespace

struct bgk_server {
    bgk_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::deque<std::unique_ptr<Job>> pending;
    std::vector<std::unique_ptr<Job>> active;
    std::vector<std::unique_ptr<Job>> prepared;    // created, not yet attached to a batch
    std::deque<bgk_result> finished;
    std::map<int64_t, std::unique_ptr<Job>> kept;  // finished jobs holding fields
    std::map<int, bgk_batch *> batches;            // storage kind -> batch
    std::thread worker;
    std::atomic<bool> stop{false};
    int64_t next_id = 1;
    int64_t used = 0, budget = 0;
    clk::time_point t0;
    // stats
    int64_t submitted = 0, admitted = 0, completed = 0, failed = 0, cell_updates = 0, launches = 0;
    double busy_s = 0, queue_s_sum = 0, first_admit = -1, last_done = 0;
    int64_t rounds = 0, round_steps = 0;
    int32_t peak = 0;
    std::vector<double> latencies;

    double now() const { return std::chrono::duration<double>(clk::now() - t0).count(); }
};

namespace {

int make_handle(bgk_server *S, Job &j)
{
    const bgk_request &r = j.req;
    bgk_case_desc d;
    bgk_default_desc(&d);
    geometry(r, j.lx, j.ly);
    d.lx = j.lx;
    d.ly = j.ly;
    d.storage = r.storage;
    d.compute = r.storage == BGK_STORE_F64 ? BGK_COMPUTE_F64 : BGK_COMPUTE_F32;
    d.device = S->cfg.device;
    if (r.kind == BGK_REQ_LDC) {
        d.tcase = BGK_CASE_LDC;
        d.u0 = r.u;
        d.svisc = r.u * r.n / r.re;
    } else if (r.kind == BGK_REQ_TGV) {
        d.tcase = BGK_CASE_TGV;
        d.u0 = 0.0;
        d.svisc = r.u * r.n / r.re;
        d.init_v = BGK_INIT_TGV;
        d.tgv_u0 = r.u;
    } else {
        d.tcase = BGK_CASE_CUSTOM;
        d.faces[0] = BGK_FACE_INFLOW;
        d.faces[1] = BGK_FACE_OUTFLOW_ZG;
        d.faces[2] = BGK_FACE_WALL;
        d.faces[3] = BGK_FACE_WALL;
        d.u0 = 0.0;
        d.u_inflow = r.u;
        d.inflow_profile = 1;
        d.svisc = r.u * r.n / r.re;
        d.obstacle = BGK_OBS_CIRCLE;
        d.radius = r.n / 2;
        d.obs_icoord = 4 * r.n;
        d.obs_jcoord = 2 * r.n + 1;
    }
    return bgk_create(&d, &j.h);
}

bgk_batch *batch_for(bgk_server *S, int storage)
{
    auto it = S->batches.find(storage);
    if (it != S->batches.end()) return it->second;
    bgk_batch *b = nullptr;
    const int compute = storage == BGK_STORE_F64 ? BGK_COMPUTE_F64 : BGK_COMPUTE_F32;
    if (bgk_batch_create(storage, compute, S->cfg.device, &b) != BGK_OK) return nullptr;
    // one block per work-list tile with an L2 prefetch of the tile half a wave (FP32) or a wave
    // (16-bit, 8 bytes per thread) ahead: on a mixed cavity / cylinder / Taylor-Green batch FP32
    // 90.7 GLUPS and FP16 148.6, against 54 and 62 with the persistent grid
    const bool half = storage == BGK_STORE_F16 || storage == BGK_STORE_BF16;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, S->cfg.device);
    bgk_batch_set_config(b, S->cfg.tile_cfg >= 0 ? S->cfg.tile_cfg : (half ? 5 : 1), 0, 32);
    bgk_batch_set_prefetch(b, (half ? 8 : 4) * sms);
    S->batches[storage] = b;
    return b;
}

void finish(bgk_server *S, std::unique_ptr<Job> j, int status)
{
    j->res.status = status;
    j->res.steps = j->steps;
    j->res.lx = j->lx;
    j->res.ly = j->ly;
    if (j->h) {
        if (status == BGK_OK || status == BGK_E_NUMERIC) {
            // a request without a residual check learns of a blow-up here: non-finite means
            const int rc = bgk_diagno(j->h, 0, j->res.diagno);
            if (status == BGK_OK && rc != BGK_OK) j->res.status = status = rc;
            if (j->req.kind == BGK_REQ_CYLINDER) bgk_draglift(j->h, j->res.draglift);
            if (j->req.keep_fields && status == BGK_OK) {
                const size_t n = (size_t)j->lx * j->ly;
                j->rho.resize(n);
                j->u.resize(n);
                j->v.resize(n);
                bgk_fields(j->h, j->rho.data(), j->u.data(), j->v.data());
            }
        }
        int64_t l = 0;
        bgk_launch_count(j->h, &l);
        bgk_destroy(j->h);  // detaches from its batch
        j->h = nullptr;
    }
    j->res.t_done = S->now();
    std::lock_guard<std::mutex> g(S->mu);
    S->used -= j->charged;
    if (status == BGK_OK) S->completed++;
    else S->failed++;
    S->latencies.push_back(j->res.t_done - j->res.t_submit);
    S->last_done = std::max(S->last_done, j->res.t_done);
    S->finished.push_back(j->res);
    if (j->req.keep_fields && status == BGK_OK) S->kept[j->id] = std::move(j);
    S->done_cv.notify_all();
}

// HBM left free on the device, less the headroom kept for the runtime and other users
constexpr int64_t HEADROOM = (int64_t)4 << 30;

int64_t free_hbm()
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        (void)cudaGetLastError();
        return INT64_MAX;  // unknown: the budget alone decides
    }
    return (int64_t)fr - HEADROOM;
}

// Create device state for queued requests (FIFO) while slots and HBM allow.  Each new case
// lives on its own stream, so this overlaps with the batches' kernels.  A request is admitted
// when it fits in the server's budget (fixed at creation) and in the HBM free right now: memory
// that other processes took, or gave back, since the server started counts at every admission.
void prepare(bgk_server *S)
{
    int64_t avail = -1;  // free HBM, read once per call and reduced by what this call admits
    for (;;) {
        std::unique_ptr<Job> j;
        {
            std::lock_guard<std::mutex> g(S->mu);
            if (S->pending.empty()) return;
            if ((int)(S->active.size() + S->prepared.size()) >= S->cfg.max_slots) return;
            Job &head = *S->pending.front();
            if (head.bytes <= S->budget && avail < 0) avail = std::max<int64_t>(free_hbm(), 0);
            if (head.bytes > S->budget) {  // can never fit: reject now
                j = std::move(S->pending.front());
                S->pending.pop_front();
            } else if (S->used + head.bytes > S->budget || head.bytes > avail) {
                return;  // wait for memory to free up (FIFO)
            } else {
                avail -= head.bytes;
                j = std::move(S->pending.front());
                S->pending.pop_front();
                S->used += j->bytes;
                j->charged = j->bytes;
            }
        }
        if (j->bytes > S->budget) {
            finish(S, std::move(j), BGK_E_NOMEM);
            continue;
        }
        int rc = make_handle(S, *j);
        if (rc != BGK_OK) {
            finish(S, std::move(j), rc);
            continue;
        }
        S->prepared.push_back(std::move(j));
    }
}

// attach prepared cases to the batch of their storage kind (between rounds)
void attach(bgk_server *S)
{
    for (auto &j : S->prepared) {
        bgk_batch *b = batch_for(S, j->req.storage);
        int rc = b ? bgk_batch_add(b, j->h) : BGK_E_CUDA;
        if (rc != BGK_OK) {
            finish(S, std::move(j), rc);
            continue;
        }
        j->res.t_admit = S->now();
        std::lock_guard<std::mutex> g(S->mu);
        S->admitted++;
        if (S->first_admit < 0) S->first_admit = j->res.t_admit;
        S->queue_s_sum += j->res.t_admit - j->res.t_submit;
        S->active.push_back(std::move(j));
        S->peak = std::max<int32_t>(S->peak, (int32_t)S->active.size());
    }
    S->prepared.clear();
}

int32_t next_event(const Job &j)
{
    int32_t e = j.req.max_steps - j.steps;
    if (j.req.tol > 0 && j.req.check_every > 0) e = std::min(e, j.req.check_every - j.steps % j.req.check_every);
    return std::max(e, 1);
}

void round_once(bgk_server *S)
{
    int32_t n = std::max(1, S->cfg.chunk_steps);
    for (auto &j : S->active) n = std::min(n, next_event(*j));
    const auto t = clk::now();
    int64_t launches = 0, cells = 0;
    std::map<int, int> failed;  // storage kind -> status of a batch whose step or sync failed
    for (auto &kv : S->batches) {
        int32_t members = 0;
        bgk_batch_size(kv.second, &members, nullptr);
        if (members == 0) continue;
        int64_t l0 = 0, l1 = 0;
        bgk_batch_launch_count(kv.second, &l0);
        if (int rc = bgk_batch_step(kv.second, n)) failed[kv.first] = rc;  // asynchronous
        bgk_batch_launch_count(kv.second, &l1);
        launches += l1 - l0;
    }
    prepare(S);  // new cases are created while the round runs
    for (auto &kv : S->batches)
        if (int rc = bgk_batch_sync(kv.second)) failed.emplace(kv.first, rc);
    for (auto &j : S->active) cells += (int64_t)n * j->lx * j->ly;
    {
        std::lock_guard<std::mutex> g(S->mu);  // the statistics are read by other threads
        S->launches += launches;
        S->busy_s += std::chrono::duration<double>(clk::now() - t).count();
        S->rounds++;
        S->round_steps += n;
        S->cell_updates += cells;
    }
    std::vector<std::unique_ptr<Job>> keep;
    for (auto &j : S->active) {
        j->steps += n;
        int status = -1;
        auto f = failed.find(j->req.storage);
        if (f != failed.end()) status = f->second;
        if (status < 0 && j->req.tol > 0 && j->req.check_every > 0 && j->steps % j->req.check_every == 0) {
            double r = 0;
            int rc = bgk_residual(j->h, &r);
            if (!j->res_started) { j->res_started = true; r = 1.0; }  // first check sets the snapshot
            j->res.residual = r;
            if (rc == BGK_E_NUMERIC) status = BGK_E_NUMERIC;
            else if (rc != BGK_OK) status = rc;
            else if (r < j->req.tol) status = BGK_OK;
        }
        if (status < 0 && j->steps >= j->req.max_steps) status = BGK_OK;
        if (status >= 0) finish(S, std::move(j), status);
        else keep.push_back(std::move(j));
    }
    S->active = std::move(keep);
    attach(S);
}

void worker_main(bgk_server *S)
{
    cudaSetDevice(S->cfg.device);
    while (!S->stop.load()) {
        if (S->active.empty()) {
            prepare(S);
            attach(S);
        }
        if (S->active.empty()) {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait_for(lk, std::chrono::milliseconds(2), [&] { return S->stop.load() || !S->pending.empty(); });
            continue;
        }
        round_once(S);
    }
}

}  // namespace

extern "C" {

int bgk_server_create(const bgk_server_config *cfg, bgk_server **out)
{
    if (!cfg || !out || cfg->max_slots < 1 || cfg->chunk_steps < 1) return BGK_E_INVALID;
    *out = nullptr;
    bgk_server *S = new bgk_server();
    S->cfg = *cfg;
    size_t fr = 0, tot = 0;
    if (cudaSetDevice(cfg->device) != cudaSuccess || cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        (void)cudaGetLastError();  // reported here; later calls must not see it
        delete S;
        return BGK_E_CUDA;
    }
    const int64_t avail = (int64_t)fr - HEADROOM;
    S->budget = cfg->hbm_budget > 0 ? std::min<int64_t>(cfg->hbm_budget, avail) : avail;
    if (S->budget <= 0) { delete S; return BGK_E_NOMEM; }
    S->t0 = clk::now();
    S->worker = std::thread(worker_main, S);
    *out = S;
    return BGK_OK;
}

int bgk_server_destroy(bgk_server *S)
{
    if (!S) return BGK_E_INVALID;
    S->stop.store(true);
    S->cv.notify_all();
    if (S->worker.joinable()) S->worker.join();
    for (auto &j : S->active)
        if (j->h) bgk_destroy(j->h);
    for (auto &j : S->prepared)
        if (j->h) bgk_destroy(j->h);
    for (auto &kv : S->batches) bgk_batch_destroy(kv.second);
    delete S;
    return BGK_OK;
}

int bgk_server_submit(bgk_server *S, const bgk_request *req, int64_t *id)
{
    if (!S || !req) return BGK_E_INVALID;
    const bgk_request &r = *req;
    if (r.kind < BGK_REQ_LDC || r.kind > BGK_REQ_TGV || r.n < 8 || r.re <= 0 || r.u <= 0 || r.max_steps < 1)
        return BGK_E_INVALID;
    if (r.storage != BGK_STORE_F32 && r.storage != BGK_STORE_F16 && r.storage != BGK_STORE_BF16 &&
        r.storage != BGK_STORE_F64)
        return BGK_E_INVALID;
    if (r.tol > 0 && r.check_every < 1) return BGK_E_INVALID;
    auto j = std::make_unique<Job>();
    j->req = r;
    j->bytes = estimate_bytes(r);
    std::memset(&j->res, 0, sizeof(j->res));
    std::lock_guard<std::mutex> g(S->mu);
    j->id = S->next_id++;
    j->res.id = j->id;
    j->res.t_submit = S->now();
    if (id) *id = j->id;
    S->pending.push_back(std::move(j));
    S->submitted++;
    S->cv.notify_all();
    return BGK_OK;
}

int bgk_server_poll(bgk_server *S, bgk_result *out, int32_t max, int32_t *n)
{
    if (!S || !n || (max > 0 && !out)) return BGK_E_INVALID;
    std::lock_guard<std::mutex> g(S->mu);
    int32_t k = 0;
    while (k < max && !S->finished.empty()) {
        out[k++] = S->finished.front();
        S->finished.pop_front();
    }
    *n = k;
    return BGK_OK;
}

int bgk_server_drain(bgk_server *S, double timeout_s)
{
    if (!S) return BGK_E_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    const bool ok = S->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return S->completed + S->failed >= S->submitted; });
    return ok ? BGK_OK : BGK_E_TIMEOUT;
}

int bgk_server_fields(bgk_server *S, int64_t id, double *rho, double *u, double *v, int64_t capacity)
{
    if (!S || !rho || !u || !v) return BGK_E_INVALID;
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->kept.find(id);
    if (it == S->kept.end()) return BGK_E_NOTFOUND;
    Job &j = *it->second;
    if (capacity < (int64_t)j.rho.size()) return BGK_E_INVALID;  // kept for a call with room
    std::memcpy(rho, j.rho.data(), j.rho.size() * sizeof(double));
    std::memcpy(u, j.u.data(), j.u.size() * sizeof(double));
    std::memcpy(v, j.v.data(), j.v.size() * sizeof(double));
    S->kept.erase(it);
    return BGK_OK;
}

int bgk_server_get_stats(bgk_server *S, bgk_server_stats *o)
{
    if (!S || !o) return BGK_E_INVALID;
    std::lock_guard<std::mutex> g(S->mu);
    std::memset(o, 0, sizeof(*o));
    o->submitted = S->submitted;
    o->admitted = S->admitted;
    o->completed = S->completed;
    o->failed = S->failed;
    o->cell_updates = S->cell_updates;
    o->busy_s = S->busy_s;
    o->wall_s = S->first_admit >= 0 ? S->last_done - S->first_admit : 0.0;
    o->glups = o->wall_s > 0 ? (double)S->cell_updates / o->wall_s / 1e9 : 0.0;
    std::vector<double> lat = S->latencies;
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double p) -> double {
        if (lat.empty()) return 0.0;
        const size_t k = std::min(lat.size() - 1, (size_t)(p * (lat.size() - 1) + 0.5));
        return lat[k];
    };
    o->p50_s = pct(0.50);
    o->p99_s = pct(0.99);
    o->mean_queue_s = S->admitted ? S->queue_s_sum / (double)S->admitted : 0.0;
    o->peak_resident = S->peak;
    o->launches = S->launches;
    o->rounds = S->rounds;
    o->mean_round_steps = S->rounds ? (double)S->round_steps / (double)S->rounds : 0.0;
    return BGK_OK;
}

}  // extern "C"
