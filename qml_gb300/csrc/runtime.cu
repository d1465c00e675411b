// Library-level entry points: version and the last CUDA error string.
#include <cstring>
#include <string>

#include "common.cuh"

namespace {
thread_local std::string g_last_error;
}

namespace qmlg {

int set_cuda_error(cudaError_t e)
{
    g_last_error = cudaGetErrorString(e);
    return QMLG_E_CUDA;
}

}  // namespace qmlg

extern "C" const char *qmlg_version(void) { return "qmlg 0.1.0 (sm_103a)"; }

extern "C" const char *qmlg_last_error(void) { return g_last_error.c_str(); }
