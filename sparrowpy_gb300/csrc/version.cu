// Library identification.
#include "common.cuh"

extern "C" const char* sp_version(void) { return "sparrowpy_gb300 0.1.0 (sm_103a)"; }
