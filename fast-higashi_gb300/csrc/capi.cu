// Library-level entry points: status strings and version.
#include "fh_common.cuh"

extern "C" const char* fh_status_string(int status) {
  switch (status) {
    case FH_OK: return "ok";
    case FH_ERR_ARG: return "bad argument (pointer, shape or count)";
    case FH_ERR_UNSUPPORTED: return "size or option outside what the kernels handle";
    case FH_ERR_NONFINITE: return "non-finite value";
    case FH_ERR_ILLCOND: return "zero or non-positive pivot in a factorisation";
    case FH_ERR_LAUNCH: return "CUDA launch or runtime failure";
    case FH_ERR_INDEX: return "contact index outside its tile";
    case FH_ERR_TIMEOUT: return "bounded device wait ran out";
    default: return "unknown status";
  }
}

extern "C" int fh_version(void) { return 100; }
