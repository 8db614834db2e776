// Internal declarations shared by the exchange translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/sparrow_gb300.h"

inline size_t sp_align(size_t bytes) { return (bytes + 255) & ~(size_t)255; }

size_t sp_structured_workspace(int precision, int n_patches, int n_dirs, int n_bins, int n_samples,
                               long long n_dir_pairs, int n_class);
int sp_run_structured(const sp_exchange_args* a, void* ws, size_t ws_bytes, cudaStream_t st);
