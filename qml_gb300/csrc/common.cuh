// Shared helpers for the qmlg CUDA sources (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qmlg.h"

namespace qmlg {

// Records the CUDA error for qmlg_last_error() and maps it to a status code.
int set_cuda_error(cudaError_t e);

// Adds to the process-wide count of kernels this library has launched.
void count_launches(unsigned n);

// Small device-to-host read of a result the stream is still producing: waits for
// the stream first, then copies.  A pageable copy issued behind pending work keeps
// other host threads' CUDA calls waiting until that work finishes; a copy issued
// on an idle stream returns at once.
int read_back(void *host, const void *dev, size_t bytes, cudaStream_t s);

// Grid cap for persistent and cooperative kernels launched from this host thread
// (qmlg_set_thread_sm_limit); returns `full` when no cap is set.
int sm_limit(int full);

// False when the calling host thread asked for one CTA per tile instead of
// persistent CTAs (qmlg_set_thread_persistent).
bool persistent_tiles();

// False when the calling host thread turned cooperative (grid-synchronised)
// kernels off (qmlg_set_thread_cooperative).
bool cooperative_on();

inline int check_launch()
{
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? QMLG_OK : set_cuda_error(e);
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Simple bump allocator over a caller-provided workspace.
struct Workspace {
    char *base;
    size_t size;
    size_t used;
    Workspace(void *p, size_t n) : base(static_cast<char *>(p)), size(n), used(0) {}
    template <class T> T *take(size_t count)
    {
        size_t off = align_up(used, 256);
        size_t bytes = count * sizeof(T);
        if (base == nullptr || off + bytes > size) return nullptr;
        used = off + bytes;
        return reinterpret_cast<T *>(base + off);
    }
};

// Workspace size helper: sums aligned chunk sizes the same way Workspace::take does.
struct WorkspacePlan {
    size_t used = 0;
    template <class T> void add(size_t count) { used = align_up(used, 256) + count * sizeof(T); }
    size_t total() const { return align_up(used, 256) + 256; }
};

}  // namespace qmlg

// Error-free transformations for double-double accumulation (Knuth two-sum and
// the FMA two-product).  Written without contraction-sensitive shortcuts.
__device__ __forceinline__ void qmlg_two_sum(double a, double b, double &s, double &e)
{
    s = __dadd_rn(a, b);
    double bv = __dsub_rn(s, a);
    double av = __dsub_rn(s, bv);
    e = __dadd_rn(__dsub_rn(a, av), __dsub_rn(b, bv));
}

// (hi, lo) += a * b
__device__ __forceinline__ void qmlg_dd_fma(double &hi, double &lo, double a, double b)
{
    double p = __dmul_rn(a, b);
    double pe = __fma_rn(a, b, -p);
    double s, e;
    qmlg_two_sum(hi, p, s, e);
    e = __dadd_rn(e, __dadd_rn(pe, lo));
    qmlg_two_sum(s, e, hi, lo);
}

// (hi, lo) += (bh, bl)
__device__ __forceinline__ void qmlg_dd_add(double &hi, double &lo, double bh, double bl)
{
    double s, e;
    qmlg_two_sum(hi, bh, s, e);
    e = __dadd_rn(e, __dadd_rn(lo, bl));
    qmlg_two_sum(s, e, hi, lo);
}
