// Local (atomic) kernels: for every pair of molecules (a, b) and every sigma s,
//   K[s + ns*(a + nm1*b)] = sum_{i in a} sum_{j in b} exp(dist(q1_i, q2_j) * inv_s)
// with dist = |.|^2, inv_s = -0.5/sigma_s^2 (Gaussian) or dist = |.|_1,
// inv_s = -1/sigma_s (Laplacian).  Restates fget_local_kernels_gaussian /
// fget_local_kernels_laplacian (qml/fkernels.f90:23-196), bound by
// qml.kernels.get_local_kernels_* (qml/kernels.py:218-299).  FP64 arithmetic; the
// atom-pair sums run in a different order than Fortran's sum(), so entries agree to
// rounding (relative 1e-12), not bit for bit.
//
// One CTA per molecule pair: the atom-pair distances of a 256-pair chunk go to
// shared memory, then every thread accumulates exp() of its share for a chunk of up
// to 8 sigmas; a block reduction per sigma writes the entry.  Symmetric mode (the
// same atoms on both sides) computes b >= a and writes the mirror as well, so K is
// exactly symmetric.
#include <cmath>

#include "common.cuh"

namespace {

constexpr int LT = 256;      // threads per CTA
constexpr int LCHUNK = 256;  // atom pairs per distance chunk
constexpr int LSIG = 8;      // sigmas per pass

template <int KIND>
__global__ void __launch_bounds__(LT)
local_kernels_kernel(const double *__restrict__ A, int64_t lda, const int64_t *__restrict__ offa,
                     int nm1, const double *__restrict__ B, int64_t ldb,
                     const int64_t *__restrict__ offb, int nm2, int d,
                     const double *__restrict__ sigmas, int ns, double *__restrict__ K,
                     int symmetric)
{
    __shared__ double sdist[LCHUNK];
    __shared__ double sred[LSIG][LT / 32];
    int a, b;
    if (symmetric) {
        // triangular enumeration: block t -> (a, b) with b >= a
        const int64_t t = blockIdx.x;
        int64_t r = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
        while (r * (r + 1) / 2 > t) --r;
        while ((r + 1) * (r + 2) / 2 <= t) ++r;
        b = (int)r;
        a = (int)(t - r * (r + 1) / 2);
    } else {
        a = (int)(blockIdx.x % (unsigned)nm1);
        b = (int)(blockIdx.x / (unsigned)nm1);
    }
    const int64_t ia = offa[a], ib = offb[b];
    const int ni = (int)(offa[a + 1] - ia), nj = (int)(offb[b + 1] - ib);
    const int np = ni * nj;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int s0 = 0; s0 < ns; s0 += LSIG) {
        const int sc = min(LSIG, ns - s0);
        double inv[LSIG], acc[LSIG];
#pragma unroll
        for (int u = 0; u < LSIG; ++u) {
            acc[u] = 0.0;
            const double sg = u < sc ? sigmas[s0 + u] : 1.0;
            inv[u] = KIND == 0 ? -0.5 / (sg * sg) : -1.0 / sg;
        }
        for (int p0 = 0; p0 < np; p0 += LCHUNK) {
            const int p = p0 + tid;
            if (tid < LCHUNK) {
                double dd = 0.0;
                if (p < np) {
                    const int i = p % ni, j = p / ni;
                    const double *x = A + (ia + i) * lda, *y = B + (ib + j) * ldb;
                    for (int t = 0; t < d; ++t) {
                        const double u = x[t] - y[t];
                        dd = KIND == 0 ? fma(u, u, dd) : dd + fabs(u);
                    }
                }
                sdist[tid] = dd;
            }
            __syncthreads();
            if (tid < LCHUNK && p < np) {
                const double dd = sdist[tid];
#pragma unroll
                for (int u = 0; u < LSIG; ++u)
                    if (u < sc) acc[u] += exp(dd * inv[u]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int u = 0; u < LSIG; ++u) {
            double v = acc[u];
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) sred[u][warp] = v;
        }
        __syncthreads();
        if (tid < sc) {
            double v = 0.0;
            for (int w = 0; w < LT / 32; ++w) v += sred[tid][w];
            K[(int64_t)(s0 + tid) + (int64_t)ns * ((int64_t)a + (int64_t)nm1 * b)] = v;
            if (symmetric && a != b)
                K[(int64_t)(s0 + tid) + (int64_t)ns * ((int64_t)b + (int64_t)nm1 * a)] = v;
        }
        __syncthreads();
    }
}

}  // namespace

extern "C" int qmlg_local_kernels(int kind, const double *A, int64_t lda, const int64_t *offsets_a,
                                  int nm1, const double *B, int64_t ldb, const int64_t *offsets_b,
                                  int nm2, int d, const double *sigmas, int nsigmas, double *K,
                                  int flags, void *stream)
{
    if ((kind != 0 && kind != 1) || nm1 < 0 || nm2 < 0 || d < 0 || nsigmas < 0) return QMLG_E_ARG;
    if (nm1 == 0 || nm2 == 0 || nsigmas == 0) return QMLG_OK;
    if (A == nullptr || B == nullptr || offsets_a == nullptr || offsets_b == nullptr ||
        sigmas == nullptr || K == nullptr || lda < d || ldb < d)
        return QMLG_E_ARG;
    const bool symmetric = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (symmetric && (nm1 != nm2 || A != B || lda != ldb || offsets_a != offsets_b)) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    const int64_t blocks = symmetric ? (int64_t)nm1 * (nm1 + 1) / 2 : (int64_t)nm1 * nm2;
    if (blocks > 0x7fffffffll) return QMLG_E_TOO_LARGE;
    const dim3 grid((unsigned)blocks);
    if (kind == 0)
        local_kernels_kernel<0><<<grid, LT, 0, s>>>(A, lda, offsets_a, nm1, B, ldb, offsets_b, nm2, d,
                                                    sigmas, nsigmas, K, symmetric ? 1 : 0);
    else
        local_kernels_kernel<1><<<grid, LT, 0, s>>>(A, lda, offsets_a, nm1, B, ldb, offsets_b, nm2, d,
                                                    sigmas, nsigmas, K, symmetric ? 1 : 0);
    qmlg::count_launches(1);
    return qmlg::check_launch();
}
