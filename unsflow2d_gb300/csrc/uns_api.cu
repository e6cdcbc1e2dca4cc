// uns_api.cu -- library-wide entry points of libunsflow_gpu.so.
#include <string>

#include "uns_common.cuh"
#include "unsflow_gpu.h"

namespace uns {
thread_local std::string g_last_error;
void set_last_error(const std::string& s) { g_last_error = s; }
}  // namespace uns

extern "C" {
const char* uns_last_error(void) { return uns::g_last_error.c_str(); }
const char* uns_version(void) { return "unsflow_gpu 0.1 (sm_103a)"; }
}
