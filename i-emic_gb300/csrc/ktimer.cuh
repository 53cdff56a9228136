// Per-kernel-class device timing: CUDA events recorded on the launching
// stream around each launch of the instrumented kernels, drained (elapsed
// times summed) at points where the host synchronises anyway. Off by
// default; each record also carries the launch's algorithmic bytes and flops.
// Inside a stream capture the records go to a template (`sink`): their
// events become event nodes of the graph, and after every replay the
// template's records are queued again, so graph-launched work is timed as it
// runs in production.
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
        bool owned_by_template = false;   // events of a captured graph: not recycled
    };
    bool on = false;
    std::vector<Rec> pending;
    std::vector<Rec>* sink = nullptr;     // template being captured
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
        if (cudaEventCreate(&e) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        return e;
    }
    // Inside a capture a plain record only orders the captured work; the
    // external flag makes it an event-record node that runs on every replay.
    cudaError_t record(cudaEvent_t ev, cudaStream_t s) const {
        return sink ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaEventRecord(ev, s);
    }
    // Returns the start event (or null when off); pass it to stop().
    cudaEvent_t start(cudaStream_t s) {
        if (!on && !sink) return nullptr;
        cudaEvent_t a = get();
        if (a && record(a, s) != cudaSuccess) {
            (void)cudaGetLastError();
            ++failed;
            return nullptr;
        }
        return a;
    }
    void stop(cudaEvent_t a, cudaStream_t s, int cls, double nbytes, double nflops) {
        if (!a) return;
        cudaEvent_t b = get();
        if (!b || record(b, s) != cudaSuccess) {
            (void)cudaGetLastError();
            ++failed;
            return;
        }
        if (sink)
            sink->push_back({a, b, cls, nbytes, nflops, true});
        else
            pending.push_back({a, b, cls, nbytes, nflops, false});
    }
    // after a replay of a graph captured with `sink = &tmpl`
    void replayed(const std::vector<Rec>& tmpl) { pending.insert(pending.end(), tmpl.begin(), tmpl.end()); }
    long long failed = 0;   // records whose elapsed time the runtime refused
    // per-launch trace in completion order (class, device ms, algorithmic bytes)
    struct Trace {
        int cls;
        float ms;
        double bytes;
    };
    static constexpr size_t kTraceCap = size_t(1) << 20;
    std::vector<Trace> trace;
    void drain() {
        for (const Rec& r : pending) {
            float t = 0.f;
            cudaEventSynchronize(r.b);
            if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) {
                (void)cudaGetLastError();   // not sticky: clear it so it is not reported later
                ++failed;
                t = 0.f;
            }
            if (trace.size() < kTraceCap) trace.push_back({r.cls, t, r.bytes});
            ms[r.cls] += t;
            bytes[r.cls] += r.bytes;
            flops[r.cls] += r.flops;
            launches[r.cls] += 1;
            if (!r.owned_by_template) {
                pool.push_back(r.a);
                pool.push_back(r.b);
            }
        }
        pending.clear();
    }
    void reset() {
        drain();
        failed = 0;
        trace.clear();
        for (int c = 0; c < IEMIC_KC_COUNT; ++c) ms[c] = bytes[c] = flops[c] = 0.0, launches[c] = 0;
    }
    ~KTimer() {
        for (const Rec& r : pending) {
            if (r.owned_by_template) continue;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
    }
};

}  // namespace iemic
