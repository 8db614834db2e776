// Library identification, the kernel launch counter and the sizes of the argument structs.
#include <atomic>

#include "common.cuh"

static std::atomic<long long> g_launches{0};

void sp_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

extern "C" const char* sp_version(void) { return "sparrowpy_gb300 0.1.0 (sm_103a)"; }

extern "C" long long sp_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" size_t sp_exchange_args_size(void) { return sizeof(sp_exchange_args); }
extern "C" size_t sp_adjoint_args_size(void) { return sizeof(sp_adjoint_args); }
extern "C" size_t sp_batch_args_size(void) { return sizeof(sp_batch_args); }
