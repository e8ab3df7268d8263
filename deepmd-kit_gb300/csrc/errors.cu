// Error text plumbing and version of the dpgb library.
#include <string>

#include "common.cuh"

namespace dpgb {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
}  // namespace dpgb

extern "C" {
const char* dpgb_last_error(void) { return dpgb::g_last_error.c_str(); }
const char* dpgb_version(void) { return "dpgb 0.1 (sm_103a)"; }
}
