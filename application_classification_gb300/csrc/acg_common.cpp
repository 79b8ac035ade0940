// acg_common.cpp -- thread-local error message and status strings.
#include "acg_common.h"

namespace acg {

static thread_local std::string g_last_error;

acg_status set_error(acg_status s, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

void clear_error() { g_last_error.clear(); }

}  // namespace acg

extern "C" const char* acg_last_error(void) { return acg::g_last_error.c_str(); }

extern "C" const char* acg_status_string(acg_status s) {
  switch (s) {
    case ACG_OK: return "ok";
    case ACG_ERR_INVALID_ARGUMENT: return "invalid argument";
    case ACG_ERR_OUT_OF_MEMORY: return "out of memory";
    case ACG_ERR_INDEX_OUT_OF_RANGE: return "index out of range";
    case ACG_ERR_CUDA: return "CUDA error";
    case ACG_ERR_UNSUPPORTED: return "unsupported";
    case ACG_ERR_IO: return "I/O error";
    case ACG_ERR_DEVICE_TIMEOUT: return "device timeout";
  }
  return "unknown status";
}

extern "C" const char* acg_version(void) { return "acg 0.1.0 sm_103a"; }
