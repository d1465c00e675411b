// Library-level entry points: version and the last CUDA error string.
#include <atomic>
#include <cstring>
#include <string>

#include "common.cuh"

namespace {
thread_local std::string g_last_error;
thread_local int t_sm_limit = 0;
thread_local int t_persistent = 1;
thread_local int t_cooperative = 1;
std::atomic<unsigned long long> g_launches{0};
}

namespace qmlg {

int set_cuda_error(cudaError_t e)
{
    g_last_error = cudaGetErrorString(e);
    return QMLG_E_CUDA;
}

void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

int read_back(void *host, const void *dev, size_t bytes, cudaStream_t s)
{
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? QMLG_OK : set_cuda_error(e);
}

int sm_limit(int full) { return (t_sm_limit > 0 && t_sm_limit < full) ? t_sm_limit : full; }

bool persistent_tiles() { return t_persistent != 0; }

bool cooperative_on() { return t_cooperative != 0; }

}  // namespace qmlg

extern "C" uint64_t qmlg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" const char *qmlg_version(void) { return "qmlg 0.1.0 (sm_103a)"; }

extern "C" const char *qmlg_last_error(void) { return g_last_error.c_str(); }

extern "C" void qmlg_set_thread_sm_limit(int n) { t_sm_limit = n > 0 ? n : 0; }

extern "C" void qmlg_set_thread_persistent(int on) { t_persistent = on ? 1 : 0; }

extern "C" void qmlg_set_thread_cooperative(int on) { t_cooperative = on ? 1 : 0; }
