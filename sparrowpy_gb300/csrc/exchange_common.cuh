// Internal declarations shared by the exchange translation units.
#pragma once
#include <cuda_runtime.h>

#include <vector>
#include <stddef.h>

#include "../../include/sparrow_gb300.h"

inline size_t sp_align(size_t bytes) { return (bytes + 255) & ~(size_t)255; }

// CUDA-event timing of a region of work enqueued on one stream (optional).
struct SpEventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    bool on = false;
    SpEventTimer(bool enable, cudaStream_t st) : on(enable) {
        if (!on) return;
        if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
            on = false;
            return;
        }
        cudaEventRecord(a, st);
    }
    void stop(cudaStream_t st) {
        if (on) cudaEventRecord(b, st);
    }
    // call after the stream was synchronised
    float elapsed_ms() {
        float ms = -1.0f;
        if (on) cudaEventElapsedTime(&ms, a, b);
        return ms;
    }
    ~SpEventTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// CUDA-event time of a series of intervals (one per order: the scatter
// launches alone), summed after the stream has been synchronised.
struct SpIntervalTimer {
    std::vector<cudaEvent_t> ev;
    int used = 0;
    bool on = false;
    SpIntervalTimer(bool enable, int max_intervals) : on(enable && max_intervals > 0) {
        if (!on) return;
        ev.assign((size_t)2 * max_intervals, nullptr);
        for (auto& e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) {
                e = nullptr;
                on = false;
            }
    }
    void start(cudaStream_t st) {
        if (on && 2 * used + 1 < (int)ev.size()) cudaEventRecord(ev[(size_t)2 * used], st);
    }
    void stop(cudaStream_t st) {
        if (on && 2 * used + 1 < (int)ev.size()) cudaEventRecord(ev[(size_t)2 * used++ + 1], st);
    }
    float total_ms() {  // call after the stream was synchronised
        float sum = 0.0f;
        for (int k = 0; on && k < used; ++k) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, ev[(size_t)2 * k], ev[(size_t)2 * k + 1]) == cudaSuccess) sum += ms;
        }
        return on ? sum : -1.0f;
    }
    ~SpIntervalTimer() {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
    SpIntervalTimer(const SpIntervalTimer&) = delete;
    SpIntervalTimer& operator=(const SpIntervalTimer&) = delete;
};

size_t sp_structured_workspace(int precision, int algorithm, int n_patches, int n_dirs, int n_bins, int n_samples,
                               long long n_dir_pairs, int n_class);
int sp_run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st);
