// Internal declarations shared by the exchange translation units.
#pragma once
#include <cuda_runtime.h>
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

size_t sp_structured_workspace(int precision, int algorithm, int n_patches, int n_dirs, int n_bins, int n_samples,
                               long long n_dir_pairs, int n_class);
int sp_run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st);
