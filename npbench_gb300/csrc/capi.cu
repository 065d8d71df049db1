// Library-wide C ABI helpers: version, status strings, per-thread last error.
#include <cstdarg>
#include <cstdio>

#include "npbgb_common.cuh"

namespace npbgb {

static thread_local char g_last_error[512] = "";

int32_t set_error(int32_t code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

}  // namespace npbgb

extern "C" {

const char* npbgb_version(void) { return "npbgb 0.1.0 sm_103a"; }

const char* npbgb_last_error(void) { return npbgb::g_last_error; }

const char* npbgb_status_string(int32_t status) {
  switch (status) {
    case NPBGB_OK: return "ok";
    case NPBGB_ERR_ARG: return "invalid argument";
    case NPBGB_ERR_DTYPE: return "unsupported dtype";
    case NPBGB_ERR_CUDA: return "CUDA error";
    case NPBGB_ERR_TIMEOUT: return "device wait timed out";
    case NPBGB_ERR_NOMEM: return "capacity or budget exceeded";
    case NPBGB_ERR_STATE: return "invalid state";
    default: return "unknown status";
  }
}

}  // extern "C"
