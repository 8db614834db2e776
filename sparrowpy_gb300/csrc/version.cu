// Library identification and the kernel launch counter.
#include <atomic>

#include "common.cuh"

static std::atomic<long long> g_launches{0};

void sp_note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

extern "C" const char* sp_version(void) { return "sparrowpy_gb300 0.1.0 (sm_103a)"; }

extern "C" long long sp_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }
