// Library-wide entry points of the C ABI (version and status strings).
#include "pwd_common.cuh"

extern "C" int pwd_version(void) { return 100; }  // 0.1.0

extern "C" const char* pwd_status_string(int status) {
  switch (status) {
    case PWD_OK: return "ok";
    case PWD_EINVAL: return "invalid size or parameter";
    case PWD_EWORKSPACE: return "workspace missing, too small or not 256-byte aligned";
    case PWD_ECUDA: return "CUDA launch or runtime error";
    case PWD_ENOTSUP: return "parameter outside what this build supports";
  }
  return "unknown status";
}
