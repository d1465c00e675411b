// Library-level entry points: version and the last CUDA error string.
#include <atomic>
#include <cstring>
#include <string>

#include "common.cuh"

namespace {
thread_local std::string g_last_error;
std::atomic<unsigned long long> g_launches{0};
}

namespace qmlg {

int set_cuda_error(cudaError_t e)
{
    g_last_error = cudaGetErrorString(e);
    return QMLG_E_CUDA;
}

void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace qmlg

extern "C" uint64_t qmlg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" const char *qmlg_version(void) { return "qmlg 0.1.0 (sm_103a)"; }

extern "C" const char *qmlg_last_error(void) { return g_last_error.c_str(); }
