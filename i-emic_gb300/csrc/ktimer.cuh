// Per-kernel-class device timing: CUDA events recorded on the launching
// stream around each launch of the instrumented kernels, drained (elapsed
// times summed) at points where the host synchronises anyway. Off by
// default; each record also carries the launch's algorithmic bytes and flops.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/iemic_gb300.h"

namespace iemic {

struct KTimer {
    struct Rec {
        cudaEvent_t a, b;
        int cls;
        double bytes, flops;
    };
    bool on = false;
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double ms[IEMIC_KC_COUNT] = {}, bytes[IEMIC_KC_COUNT] = {}, flops[IEMIC_KC_COUNT] = {};
    long long launches[IEMIC_KC_COUNT] = {};

    cudaEvent_t get() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    // Returns the start event (or null when off); pass it to stop().
    cudaEvent_t start(cudaStream_t s) {
        if (!on) return nullptr;
        cudaEvent_t a = get();
        cudaEventRecord(a, s);
        return a;
    }
    void stop(cudaEvent_t a, cudaStream_t s, int cls, double nbytes, double nflops) {
        if (!a) return;
        cudaEvent_t b = get();
        cudaEventRecord(b, s);
        pending.push_back({a, b, cls, nbytes, nflops});
    }
    void drain() {
        for (const Rec& r : pending) {
            float t = 0.f;
            cudaEventSynchronize(r.b);
            cudaEventElapsedTime(&t, r.a, r.b);
            ms[r.cls] += t;
            bytes[r.cls] += r.bytes;
            flops[r.cls] += r.flops;
            launches[r.cls] += 1;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        pending.clear();
    }
    void reset() {
        drain();
        for (int c = 0; c < IEMIC_KC_COUNT; ++c) ms[c] = bytes[c] = flops[c] = 0.0, launches[c] = 0;
    }
    ~KTimer() {
        for (const Rec& r : pending) {
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

}  // namespace iemic
