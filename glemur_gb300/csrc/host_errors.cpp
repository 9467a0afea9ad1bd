// host_errors.cpp -- per-thread error message of the C-ABI.
#include <string>

#include "gm_internal.h"

namespace {
thread_local std::string g_last_error;
}

namespace gm {
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}
}  // namespace gm

extern "C" const char* gm_last_error(void) { return g_last_error.c_str(); }
extern "C" const char* gm_version(void) { return "glemur_gb300 0.1 (sm_103a)"; }
