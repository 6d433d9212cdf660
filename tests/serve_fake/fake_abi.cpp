// Host-only fake of the handle and batch entry points that bgk_serve.cpp calls, so that the
// serving scheduler (admission, HBM accounting, rounds, residual stops, failure statuses) runs
// on a machine without a GPU.  A "step" only counts: each member of a stepped batch adds n to
// its step counter.  The observable quantities are chosen so a test can predict them:
//   residual after s steps        = 1 / s
//   diagno                        = {s, lx, ly, 0}; non-finite (BGK_E_NUMERIC) for u0 == nan_u0
//   fields                        = rho filled with s
//   bgk_batch_step on fail_storage = BGK_E_CUDA, nothing stepped
// fake_counts reports live handles, the most that were alive at once, and creations.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/bgk2d_gb300.h"

struct bgk_handle {
    bgk_case_desc d;
    int64_t steps = 0;
    bgk_batch *batch = nullptr;
};

struct bgk_batch {
    int32_t storage = 0;
    std::vector<bgk_handle *> members;
    int64_t launches = 0;
};

size_t g_fake_free_bytes = (size_t)64 << 30;  // what the fake cudaMemGetInfo reports as free

namespace {
std::mutex mu;
int fail_storage = -1;
double nan_u0 = -1.0;
int64_t live = 0, max_live = 0, created = 0;
}  // namespace

extern "C" {

void fake_configure(int32_t storage_that_fails, double u0_that_blows_up)
{
    std::lock_guard<std::mutex> g(mu);
    fail_storage = storage_that_fails;
    nan_u0 = u0_that_blows_up;
    live = max_live = created = 0;
}

// free device memory as the next cudaMemGetInfo sees it (another process taking or giving back HBM)
void fake_set_free_bytes(int64_t bytes)
{
    std::lock_guard<std::mutex> g(mu);
    g_fake_free_bytes = (size_t)bytes;
}

void fake_counts(int64_t out[3])
{
    std::lock_guard<std::mutex> g(mu);
    out[0] = live;
    out[1] = max_live;
    out[2] = created;
}

int bgk_default_desc(bgk_case_desc *d)
{
    std::memset(d, 0, sizeof(*d));
    d->lx = d->ly = 256;
    return BGK_OK;
}

int bgk_create(const bgk_case_desc *d, bgk_handle **out)
{
    bgk_handle *h = new bgk_handle();
    h->d = *d;
    *out = h;
    std::lock_guard<std::mutex> g(mu);
    ++created;
    ++live;
    if (live > max_live) max_live = live;
    return BGK_OK;
}

int bgk_destroy(bgk_handle *h)
{
    if (h->batch) {
        auto &m = h->batch->members;
        for (size_t i = 0; i < m.size(); ++i)
            if (m[i] == h) { m.erase(m.begin() + (long)i); break; }
    }
    delete h;
    std::lock_guard<std::mutex> g(mu);
    --live;
    return BGK_OK;
}

int bgk_diagno(bgk_handle *h, int32_t, double out[4])
{
    out[0] = (double)h->steps;
    out[1] = h->d.lx;
    out[2] = h->d.ly;
    out[3] = 0.0;
    if (h->d.u0 == nan_u0) {
        out[0] = std::nan("");
        return BGK_E_NUMERIC;
    }
    return BGK_OK;
}

int bgk_draglift(bgk_handle *, double out[2])
{
    out[0] = 1.0;
    out[1] = 2.0;
    return BGK_OK;
}

int bgk_fields(bgk_handle *h, double *rho, double *u, double *v)
{
    const size_t n = (size_t)h->d.lx * h->d.ly;
    for (size_t i = 0; i < n; ++i) {
        rho[i] = (double)h->steps;
        u[i] = v[i] = 0.0;
    }
    return BGK_OK;
}

int bgk_residual(bgk_handle *h, double *out)
{
    *out = h->steps > 0 ? 1.0 / (double)h->steps : 1.0;
    return BGK_OK;
}

int bgk_launch_count(bgk_handle *h, int64_t *l)
{
    *l = h->steps;
    return BGK_OK;
}

int bgk_batch_create(int32_t storage, int32_t, int32_t, bgk_batch **out)
{
    bgk_batch *b = new bgk_batch();
    b->storage = storage;
    *out = b;
    return BGK_OK;
}

int bgk_batch_destroy(bgk_batch *b)
{
    for (auto *h : b->members) h->batch = nullptr;
    delete b;
    return BGK_OK;
}

int bgk_batch_set_config(bgk_batch *, int32_t, int32_t, int32_t) { return BGK_OK; }
int bgk_batch_set_prefetch(bgk_batch *, int32_t) { return BGK_OK; }

int bgk_batch_add(bgk_batch *b, bgk_handle *h)
{
    if (h->d.storage != b->storage || h->batch) return BGK_E_INVALID;
    b->members.push_back(h);
    h->batch = b;
    return BGK_OK;
}

int bgk_batch_size(bgk_batch *b, int32_t *members, int64_t *cells)
{
    int64_t c = 0;
    for (auto *h : b->members) c += (int64_t)h->d.lx * h->d.ly;
    if (members) *members = (int32_t)b->members.size();
    if (cells) *cells = c;
    return BGK_OK;
}

int bgk_batch_launch_count(bgk_batch *b, int64_t *l)
{
    *l = b->launches;
    return BGK_OK;
}

int bgk_batch_step(bgk_batch *b, int32_t n)
{
    if (b->storage == fail_storage) return BGK_E_CUDA;
    for (auto *h : b->members) h->steps += n;
    b->launches += n;
    return BGK_OK;
}

int bgk_batch_sync(bgk_batch *) { return BGK_OK; }

}  // extern "C"
