// Library-level entry points: version and status strings.
#include "common.cuh"

ODIL_API int odil_version(void) { return 100; }

ODIL_API const char* odil_status_string(int status) {
    switch (status) {
        case ODIL_OK: return "ok";
        case ODIL_ERR_SHAPE: return "sizes out of range or inconsistent";
        case ODIL_ERR_DTYPE: return "unsupported precision combination";
        case ODIL_ERR_ALIGN: return "pointer misaligned for vector access";
        case ODIL_ERR_LAUNCH: return "CUDA launch or runtime failure";
        case ODIL_ERR_TIMEOUT: return "a bounded device-side wait gave up";
        case ODIL_ERR_NONFINITE: return "NaN or Inf detected";
        case ODIL_ERR_WORKSPACE: return "workspace missing or too small";
        case ODIL_ERR_ARG: return "null pointer or invalid argument";
        default: return "unknown status";
    }
}
