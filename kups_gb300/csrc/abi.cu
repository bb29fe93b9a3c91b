// Library identity and error strings of the kups_gb300 C ABI.
#include "common.cuh"

extern "C" const char *kups_version(void) { return "kups_gb300 0.1.0 sm_103a"; }

extern "C" const char *kups_error_string(int32_t code) {
  switch (code) {
    case KUPS_OK: return "ok";
    case KUPS_ERR_CAPACITY: return "capacity exceeded (status.required holds the size that suffices)";
    case KUPS_ERR_NONFINITE: return "non-finite value encountered";
    case KUPS_ERR_INVALID: return "invalid argument";
    case KUPS_ERR_CUDA: return "CUDA launch or runtime error";
    case KUPS_ERR_UNSUPPORTED: return "unsupported configuration";
    default: return "unknown error";
  }
}
