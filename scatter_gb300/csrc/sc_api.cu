// Library-wide entry points: version, status strings, last CUDA error text.
#include <stdio.h>

#include "sc_common.cuh"

namespace sc {
static thread_local char g_last_error[256] = "";
void set_last_error(const char* where, cudaError_t e) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, cudaGetErrorString(e));
}
void set_last_message(const char* text) { snprintf(g_last_error, sizeof(g_last_error), "%s", text); }
}  // namespace sc

extern "C" int sc_version(void) { return 1; }

extern "C" const char* sc_status_string(int status) {
  switch (status) {
    case SC_OK: return "ok";
    case SC_BAD_ARG: return "bad argument";
    case SC_NOT_CONVERGED: return "iterative solve not converged";
    case SC_BREAKDOWN: return "iterative solve breakdown (matrix not positive definite)";
    case SC_CAPACITY: return "capacity exceeded";
    case SC_CUDA_ERROR: return "CUDA error";
    default: return "unknown status";
  }
}

extern "C" const char* sc_last_error(void) { return sc::g_last_error; }
