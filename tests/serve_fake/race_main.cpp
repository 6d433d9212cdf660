// Concurrency check of the serving scheduler, built with -fsanitize=thread against the fake ABI
// (tests/test_serve_host.py::test_scheduler_has_no_data_races).  Client threads submit requests
// and read statistics and results while the scheduler thread runs its rounds; the sanitizer
// reports any unsynchronised access to shared server state.  Exit status 0 when every request
// finished with BGK_OK.
#include <cstdio>
#include <thread>
#include <vector>

#include "../../include/bgk2d_gb300.h"

extern "C" void fake_configure(int32_t storage_that_fails, double u0_that_blows_up);

int main()
{
    fake_configure(-1, -1.0);
    bgk_server_config cfg{};
    cfg.device = 0;
    cfg.max_slots = 4;
    cfg.chunk_steps = 50;
    cfg.tile_cfg = -1;
    bgk_server *s = nullptr;
    if (bgk_server_create(&cfg, &s) != BGK_OK) return 2;
    std::vector<std::thread> clients;
    for (int t = 0; t < 3; ++t)
        clients.emplace_back([s, t] {
            for (int k = 0; k < 8; ++k) {
                bgk_request r{};
                r.kind = BGK_REQ_LDC;
                r.n = 32 + 8 * t;
                r.re = 100;
                r.u = 0.1;
                r.storage = (k & 1) ? BGK_STORE_F16 : BGK_STORE_F32;
                r.max_steps = 400;
                r.tol = (k % 3 == 0) ? 1e-3 : 0.0;
                r.check_every = 100;
                int64_t id = 0;
                bgk_server_submit(s, &r, &id);
                bgk_server_stats st;
                bgk_server_get_stats(s, &st);
            }
        });
    std::thread watcher([s] {
        for (int k = 0; k < 200; ++k) {
            bgk_server_stats st;
            bgk_server_get_stats(s, &st);
            bgk_result res[8];
            int32_t n = 0;
            bgk_server_poll(s, res, 0, &n);
        }
    });
    for (auto &c : clients) c.join();
    watcher.join();
    if (bgk_server_drain(s, 60.0) != BGK_OK) return 3;
    bgk_result res[64];
    int32_t n = 0;
    bgk_server_poll(s, res, 64, &n);
    int bad = 0;
    for (int i = 0; i < n; ++i) bad += res[i].status != BGK_OK;
    bgk_server_stats st;
    bgk_server_get_stats(s, &st);
    bgk_server_destroy(s);
    std::printf("results %d failed %d completed %lld\n", n, bad, (long long)st.completed);
    return (n == 24 && bad == 0 && st.completed == 24) ? 0 : 4;
}
