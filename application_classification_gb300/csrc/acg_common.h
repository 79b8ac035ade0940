// acg_common.h -- internal helpers shared by the host and CUDA sources.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "acg.h"

namespace acg {

// Record a message for acg_last_error() on this thread and return `s`.
acg_status set_error(acg_status s, const char* fmt, ...)
#if defined(__GNUC__)
    __attribute__((format(printf, 2, 3)))
#endif
    ;
void clear_error();

}  // namespace acg

#define ACG_TRY(expr)                          \
  do {                                         \
    acg_status acg_try_s_ = (expr);            \
    if (acg_try_s_ != ACG_OK) return acg_try_s_; \
  } while (0)
