// serve_tsan_main.cpp -- the request server's threads under ThreadSanitizer, on the CPU (tests/test_serve_tsan.py).
//
// The server (final184_gb300/csrc/serve.cpp, compiled unchanged) runs against serve_fake_device.cpp.  Four host
// threads submit requests to three scenes (moves, views, host-buffer requests, injected update failures) while
// another cancels and a third polls statistics; every ticket must finish with OK, CANCELLED or the injected failure.
// Then the worker-loss hook: the scheduler thread exits between admission and issue, the queued requests fail with
// F184GI_ERR_WORKER and later submissions are refused.  Exit status 0 when every check holds (ThreadSanitizer's own
// exit code marks a race).
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <random>
#include <thread>
#include <vector>

#include "f184gi.h"

#define CHECK(c)                                                              \
    do {                                                                      \
        if (!(c)) {                                                           \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            std::exit(2);                                                     \
        }                                                                     \
    } while (0)

int main(int argc, char** argv) {
    const char* log_path = argc > 1 ? argv[1] : nullptr;
    f184gi_server_config cfg{};
    cfg.slots = 2;
    cfg.max_batch_views = 16;
    f184gi_server* S = nullptr;
    CHECK(f184gi_server_create(&cfg, &S) == F184GI_OK);
    if (log_path) CHECK(f184gi_server_set_log(S, log_path) == F184GI_OK);
    const uint64_t ntris = 64;
    std::vector<float> tri(ntris * 9, 0.5f);
    std::vector<uint32_t> alb(ntris, 0xff808080u);
    f184gi_bounds b{};
    b.max.x = b.max.y = b.max.z = 1.0f;
    f184gi_light light{{1.f, 1.f, 1.f}, {0.f, -1.f, 0.f}};
    for (uint32_t id = 0; id < 3; ++id) {
        f184gi_grid_desc d{16, 4, F184GI_FMT_F16, 0, 256, 0};
        CHECK(f184gi_server_add_scene(S, id, &d, tri.data(), alb.data(), ntris, &b, &light) == F184GI_OK);
    }
    // view buffers (host memory stands for device memory in the fake)
    const uint32_t W = 16, H = 8;
    std::vector<float> depth(W * H, 0.5f);
    std::vector<uint32_t> normal(W * H, 0);
    std::vector<uint16_t> rough(W * H, 0);
    std::vector<std::vector<float>> outs(64, std::vector<float>(2 * W * H * 4));
    auto make_view = [&](int k) {
        f184gi_view v{};
        for (int i = 0; i < 16; ++i) v.view[i] = v.proj[i] = (i % 5 == 0) ? 1.f : 0.f;
        v.width = W, v.height = H;
        v.depth = depth.data(), v.normal = normal.data(), v.roughness = rough.data();
        v.out = outs[k % 64].data();
        v.out_format = F184GI_FMT_F32;
        return v;
    };
    std::mutex tmu;
    std::vector<std::pair<uint64_t, uint32_t>> tickets;  // (ticket, flags)
    std::atomic<bool> done{false};
    auto submitter = [&](int seed) {
        std::mt19937 rng(seed);
        for (int i = 0; i < 40; ++i) {
            f184gi_view views[4];
            const uint32_t nv = 1 + rng() % 4;
            for (uint32_t k = 0; k < nv; ++k) views[k] = make_view(int(rng() % 64));
            f184gi_move mv[2] = {{uint32_t(rng() % 32), 4u, {0.01f, 0.f, 0.f}}, {40u, 8u, {0.f, -0.02f, 0.f}}};
            f184gi_request r{};
            r.scene_id = rng() % 3;
            r.flags = (rng() % 7 == 0) ? F184GI_REQ_INJECT_FAIL : ((rng() % 5 == 0) ? F184GI_REQ_HOST_BUFFERS : 0u);
            r.moves = mv;
            r.nmoves = rng() % 3;
            r.nviews = nv;
            r.views = views;
            uint64_t t = 0;
            CHECK(f184gi_server_submit(S, &r, &t) == F184GI_OK);
            std::lock_guard<std::mutex> lk(tmu);
            tickets.push_back({t, r.flags});
        }
    };
    auto canceller = [&]() {
        std::mt19937 rng(99);
        while (!done.load()) {
            uint64_t t = 0;
            {
                std::lock_guard<std::mutex> lk(tmu);
                if (!tickets.empty()) t = tickets[rng() % tickets.size()].first;
            }
            if (t) f184gi_server_cancel(S, t);  // OK, or INVALID once running
            std::this_thread::sleep_for(std::chrono::microseconds(300));
        }
    };
    auto poller = [&]() {
        while (!done.load()) {
            f184gi_server_stats st{};
            CHECK(f184gi_server_get_stats(S, &st) == F184GI_OK);
            std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
    };
    std::vector<std::thread> th;
    for (int k = 0; k < 4; ++k) th.emplace_back(submitter, 1000 + k);
    std::thread tc(canceller), tp(poller);
    for (auto& t : th) t.join();
    int ok = 0, cancelled = 0, injected = 0;
    for (auto& tf : tickets) {
        f184gi_request_result res{};
        const int rc = f184gi_server_wait(S, tf.first, 20000, &res);
        if (tf.second & F184GI_REQ_INJECT_FAIL) {
            CHECK(rc == F184GI_ERR_CUDA || res.status == F184GI_ERR_CANCELLED);
            injected += rc == F184GI_ERR_CUDA;
        } else {
            CHECK(rc == F184GI_OK);
            CHECK(res.status == F184GI_OK || res.status == F184GI_ERR_CANCELLED);
            (res.status == F184GI_OK ? ok : cancelled) += 1;
        }
    }
    done = true;
    tc.join();
    tp.join();
    CHECK(ok > 0 && injected > 0);
    // worker lost between stages: the scheduler exits after admitting this request's batch
    f184gi_view v = make_view(0);
    f184gi_request r{};
    r.scene_id = 1;
    r.nviews = 1;
    r.views = &v;
    r.flags = F184GI_REQ_INJECT_WORKER_EXIT;
    uint64_t t = 0;
    CHECK(f184gi_server_submit(S, &r, &t) == F184GI_OK);
    f184gi_request_result res{};
    CHECK(f184gi_server_wait(S, t, 20000, &res) == F184GI_ERR_WORKER);
    r.flags = 0;
    CHECK(f184gi_server_submit(S, &r, &t) == F184GI_ERR_WORKER);
    CHECK(f184gi_server_destroy(S) == F184GI_OK);
    std::printf("served %d, cancelled %d, injected failures %d; worker loss reported\n", ok, cancelled, injected);
    return 0;
}
