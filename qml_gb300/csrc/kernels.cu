// FP64 kernel matrices and the prediction that uses them.
//
// Restates the global kernels of qml/fkernels.f90, K in Fortran order like the
// reference (K[j + i*ldk] for A row j, B row i):
//   Gaussian  (:340-372)  exp(-0.5/sigma^2 * |A_j - B_i|^2)
//   Laplacian (:374-400)  exp(-1/sigma * |A_j - B_i|_1)
//   linear    (:403-423)  A_j . B_i
//   Matern L2 (:426-484)  d = |A_j - B_i|_2, order 0: exp(-d/s), 1: exp(-r3 d/s)(1 + r3 d/s),
//                         2: exp(-r5 d/s)(1 + r5 d/s + 5 d^2 / (3 s^2))  (r3 = sqrt 3, r5 = sqrt 5)
//   Sargan    (:487-531)  d = |A_j - B_i|_1, exp(-d/s) (1 + sum_m gamma_m (d/s)^m)
// The Gaussian distance is formed as |a|^2 + |b|^2 - 2 a.b (norms in FP64); the
// other distances keep the reference's direct difference form.
//
// Tiling: a CTA computes a 64 (j, rows of A) x 64 (i, rows of B) tile with 256
// threads, 4x4 outputs per thread, the feature dimension streamed through shared
// memory 16 columns at a time.  Symmetric mode computes only tiles on or below the
// diagonal and writes the mirror through a shared-memory transpose, so K is
// exactly symmetric.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace {

constexpr int TJ = 64;   // tile rows (A side, contiguous in K)
constexpr int TI = 64;   // tile cols (B side)
constexpr int TK = 16;   // feature chunk
constexpr int NT = 256;  // threads

enum Kind { kGauss = 0, kLaplace = 1, kLinear = 2, kMaternL2 = 3, kSargan = 4 };

// Epilogue constants: s1 the exponent's factor (Matern: -sqrt(2 order + 1)/sigma),
// s2 the Matern order-2 quadratic factor 5/(3 sigma^2), gammas[0..ng) the Sargan
// polynomial (device memory).
struct EpiParams {
    double s1 = 0.0, s2 = 0.0;
    int order = 0;
    const double *gammas = nullptr;
    int ng = 0;
};

// Maps a linear block id onto a lower-triangular tile pair (bi >= bj).
__device__ __forceinline__ void tri_index(int64_t t, int &bi, int &bj)
{
    int64_t r = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = (int)r;
    bj = (int)(t - r * (r + 1) / 2);
}

// Maps a linear block id onto a rectangular tile pair: bj (A side, fastest, tj
// tiles) and bi (B side).  One grid dimension takes up to 2^31 - 1 blocks, where a
// second one would stop at 65535 tiles (4.19M rows).
__device__ __forceinline__ void rect_index(int tj, int &bj, int &bi)
{
    bj = (int)(blockIdx.x % (unsigned)tj);
    bi = (int)(blockIdx.x / (unsigned)tj);
}

// One-dimensional grid over a tile list: tj * ti rectangular tiles, or the
// tj (tj + 1) / 2 tiles on and below the diagonal; false when the list is longer
// than one grid dimension takes.
inline bool tile_list_grid(int tj, int ti, bool symmetric, dim3 &grid)
{
    const int64_t t = symmetric ? (int64_t)tj * (tj + 1) / 2 : (int64_t)tj * ti;
    if (t > 0x7fffffffLL) return false;
    grid = dim3((unsigned)t);
    return true;
}

// Accumulates the 4x4 micro-tile over the feature dimension.
template <int KIND>
__device__ __forceinline__ void tile_accumulate(const double *__restrict__ A, int64_t lda, int na,
                                                const double *__restrict__ B, int64_t ldb, int nb,
                                                int d, int j0, int i0, double (&acc)[4][4],
                                                double (*As)[TJ + 1], double (*Bs)[TI + 1],
                                                double *a2s, double *b2s)
{
    // Gaussian: threads 0..63 accumulate |A_j|^2 and 64..127 |B_i|^2 of the tile rows
    double nrm = 0.0;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

    for (int t0 = 0; t0 < d; t0 += TK) {
        // 64 rows x 16 features of each operand: 1024 values, 4 per thread.
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * NT;
            const int r = e >> 4, c = e & 15;
            const int t = t0 + c;
            const int ja = j0 + r, ib = i0 + r;
            As[c][r] = (ja < na && t < d) ? A[(int64_t)ja * lda + t] : 0.0;
            Bs[c][r] = (ib < nb && t < d) ? B[(int64_t)ib * ldb + t] : 0.0;
        }
        __syncthreads();
        if (KIND == kGauss && tid < TJ + TI) {
            const int r = tid & (TJ - 1);
            if (tid < TJ) {
#pragma unroll
                for (int c = 0; c < TK; ++c) nrm = fma(As[c][r], As[c][r], nrm);
            } else {
#pragma unroll
                for (int c = 0; c < TK; ++c) nrm = fma(Bs[c][r], Bs[c][r], nrm);
            }
        }
#pragma unroll
        for (int c = 0; c < TK; ++c) {
            double av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[c][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[c][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    if (KIND == kGauss || KIND == kLinear) {
                        acc[a][b] = fma(av[a], bv[b], acc[a][b]);
                    } else if (KIND == kMaternL2) {
                        const double t = av[a] - bv[b];
                        acc[a][b] = fma(t, t, acc[a][b]);
                    } else {
                        acc[a][b] += fabs(av[a] - bv[b]);
                    }
                }
        }
        __syncthreads();
    }
    if (KIND == kGauss && tid < TJ + TI) {
        if (tid < TJ) a2s[tid] = nrm;
        else b2s[tid - TJ] = nrm;
    }
    __syncthreads();
}

template <int KIND>
__global__ void __launch_bounds__(NT)
kernel_matrix_kernel(const double *__restrict__ A, int64_t lda, int na,
                     const double *__restrict__ B, int64_t ldb, int nb, int d,
                     EpiParams ep, double *__restrict__ K, int64_t ldk, int symmetric,
                     double diag_shift, const int *__restrict__ skip)
{
    // skip (may be null): *skip != 0 means another kernel of the same launch
    // sequence writes K (the fixed-point Laplacian when its grid is fine enough)
    if (skip != nullptr && *skip != 0) return;
    // operand chunks during accumulation, the output tile (for the mirror) after
    __shared__ double smem[TI * (TJ + 1)];
    __shared__ double a2s[TJ], b2s[TI];
    double(*As)[TJ + 1] = reinterpret_cast<double(*)[TJ + 1]>(smem);
    double(*Bs)[TI + 1] = reinterpret_cast<double(*)[TI + 1]>(smem + TK * (TJ + 1));
    double(*T)[TJ + 1] = reinterpret_cast<double(*)[TJ + 1]>(smem);

    int bj, bi;
    if (symmetric) {
        tri_index(blockIdx.x, bi, bj);  // bi >= bj: B-tile index >= A-tile index
    } else {
        rect_index((na + TJ - 1) / TJ, bj, bi);
    }
    const int j0 = bj * TJ, i0 = bi * TI;
    double acc[4][4];
    tile_accumulate<KIND>(A, lda, na, B, ldb, nb, d, j0, i0, acc, As, Bs, a2s, b2s);

    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int j = j0 + tx + 16 * a, i = i0 + ty + 16 * b;
            double v;
            if (KIND == kGauss) {
                double d2 = 0.0;
                if (j < na && i < nb)
                    d2 = fmax(a2s[tx + 16 * a] + b2s[ty + 16 * b] - 2.0 * acc[a][b], 0.0);
                if (symmetric && i == j) d2 = 0.0;
                v = exp(ep.s1 * d2);
            } else if (KIND == kLaplace) {
                v = exp(ep.s1 * acc[a][b]);
            } else if (KIND == kLinear) {
                v = acc[a][b];
            } else if (KIND == kMaternL2) {
                const double d2 = acc[a][b], dd = sqrt(d2);
                v = exp(ep.s1 * dd);
                if (ep.order == 1) v *= 1.0 - ep.s1 * dd;
                else if (ep.order == 2) v *= 1.0 - ep.s1 * dd + ep.s2 * d2;
            } else {
                // exp(-d/s) (1 + sum_m gamma_m t^m), t = d/s
                const double dd = acc[a][b], t = -ep.s1 * dd;
                double pw = 1.0, sum = 0.0;
                for (int m = 0; m < ep.ng; ++m) {
                    pw *= t;
                    sum += ep.gammas[m] * pw;
                }
                v = exp(ep.s1 * dd) * (1.0 + sum);
            }
            if (symmetric && i == j) v += diag_shift;
            if (j < na && i < nb) K[(int64_t)i * ldk + j] = v;
            T[ty + 16 * b][tx + 16 * a] = v;
        }
    if (symmetric && bi != bj) {
        // mirror: K[i + j*ldk] for the same (j, i), coalesced along i
        __syncthreads();
        for (int e = tid; e < TI * TJ; e += NT) {
            const int ii = e & (TI - 1), jj = e / TI;
            const int i = i0 + ii, j = j0 + jj;
            if (i < nb && j < na) K[(int64_t)j * ldk + i] = T[ii][jj];
        }
    }
}

// Fused prediction: per (training tile, test tile) partial sums of k * alpha.
template <int KIND>
__global__ void __launch_bounds__(NT)
predict_partial_kernel(const double *__restrict__ Xtr, int64_t ldtr, int ntr,
                       const double *__restrict__ Xte, int64_t ldte, int nte, int d,
                       double scale, const double *__restrict__ alpha,
                       double *__restrict__ partial, const int *__restrict__ skip)
{
    if (skip != nullptr && *skip != 0) return;  // as in kernel_matrix_kernel
    __shared__ double As[TK][TJ + 1];
    __shared__ double Bs[TK][TI + 1];
    __shared__ double a2s[TJ], b2s[TI];
    __shared__ double red[16][TI + 1];
    int bj, bi;
    rect_index((ntr + TJ - 1) / TJ, bj, bi);
    const int j0 = bj * TJ, i0 = bi * TI;
    double acc[4][4];
    tile_accumulate<KIND>(Xtr, ldtr, ntr, Xte, ldte, nte, d, j0, i0, acc, As, Bs, a2s, b2s);
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int i = i0 + ty + 16 * b;
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int j = j0 + tx + 16 * a;
            if (j < ntr && i < nte) {
                double v;
                if (KIND == kGauss) {
                    const double d2 =
                        fmax(a2s[tx + 16 * a] + b2s[ty + 16 * b] - 2.0 * acc[a][b], 0.0);
                    v = exp(scale * d2);
                } else {
                    v = exp(scale * acc[a][b]);
                }
                s = fma(v, alpha[j], s);
            }
        }
        red[tx][ty + 16 * b] = s;
    }
    __syncthreads();
    if (tid < TI) {
        double s = 0.0;
        for (int q = 0; q < 16; ++q) s += red[q][tid];
        const int i = i0 + tid;
        if (i < nte) partial[(int64_t)bj * nte + i] = s;
    }
}

__global__ void reduce_partial_kernel(const double *__restrict__ partial, int nparts, int n,
                                      double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += partial[(int64_t)p * n + i];
    y[i] = s;
}

// yhat[i] = sum_j Ks[j + i*ldk] alpha[j]: one warp per column of Ks.
__global__ void gemv_t_kernel(const double *__restrict__ Ks, int64_t ldk, int ntr, int nte,
                              const double *__restrict__ alpha, double *__restrict__ y)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nte) return;
    const double *col = Ks + (int64_t)warp * ldk;
    double s = 0.0;
    for (int j = lane; j < ntr; j += 32) s = fma(col[j], alpha[j], s);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) y[warp] = s;
}

int check_common(const double *A, int64_t lda, int na, const double *B, int64_t ldb, int nb,
                 int d, double sigma)
{
    if (na < 0 || nb < 0 || d < 0) return QMLG_E_ARG;
    if ((na > 0 && (A == nullptr || lda < d)) || (nb > 0 && (B == nullptr || ldb < d)))
        return QMLG_E_ARG;
    if (!(sigma > 0.0) || !std::isfinite(sigma)) return QMLG_E_ARG;
    return QMLG_OK;
}

template <int KIND>
void launch_kernel_matrix(dim3 grid, cudaStream_t s, const double *A, int64_t lda, int na,
                          const double *B, int64_t ldb, int nb, int d, const EpiParams &ep,
                          double *K, int64_t ldk, int symmetric, double diag_shift)
{
    kernel_matrix_kernel<KIND><<<grid, NT, 0, s>>>(A, lda, na, B, ldb, nb, d, ep, K, ldk, symmetric,
                                                   diag_shift, nullptr);
    qmlg::count_launches(1);
}

int kernel_matrix(int kind, const double *A, int64_t lda, int na, const double *B,
                  int64_t ldb, int nb, int d, double sigma, double *K, int64_t ldk, int flags,
                  double diag_shift, void *stream, EpiParams ep = EpiParams())
{
    int st = check_common(A, lda, na, B, ldb, nb, d, sigma);
    if (st != QMLG_OK) return st;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    const bool symmetric = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (symmetric && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    cudaStream_t s = qmlg::as_stream(stream);

    if (kind == kGauss) ep.s1 = -0.5 / (sigma * sigma);
    else if (kind == kLaplace || kind == kSargan) ep.s1 = -1.0 / sigma;
    const int tj = (int)qmlg::ceil_div(na, TJ), ti = (int)qmlg::ceil_div(nb, TI);
    dim3 grid;
    if (!tile_list_grid(tj, ti, symmetric, grid)) return QMLG_E_ARG;
    const int sym = symmetric ? 1 : 0;
    switch (kind) {
    case kGauss: launch_kernel_matrix<kGauss>(grid, s, A, lda, na, B, ldb, nb, d, ep, K, ldk, sym, diag_shift); break;
    case kLaplace: launch_kernel_matrix<kLaplace>(grid, s, A, lda, na, B, ldb, nb, d, ep, K, ldk, sym, diag_shift); break;
    case kLinear: launch_kernel_matrix<kLinear>(grid, s, A, lda, na, B, ldb, nb, d, ep, K, ldk, sym, diag_shift); break;
    case kMaternL2: launch_kernel_matrix<kMaternL2>(grid, s, A, lda, na, B, ldb, nb, d, ep, K, ldk, sym, diag_shift); break;
    default: launch_kernel_matrix<kSargan>(grid, s, A, lda, na, B, ldb, nb, d, ep, K, ldk, sym, diag_shift); break;
    }
    return qmlg::check_launch();
}

}  // namespace

extern "C" int qmlg_gaussian_kernel(const double *A, int64_t lda, int na, const double *B,
                                    int64_t ldb, int nb, int d, double sigma, double *K,
                                    int64_t ldk, int flags, double diag_shift, void *stream)
{
    return kernel_matrix(kGauss, A, lda, na, B, ldb, nb, d, sigma, K, ldk, flags, diag_shift,
                         stream);
}

extern "C" int qmlg_laplacian_kernel(const double *A, int64_t lda, int na, const double *B,
                                     int64_t ldb, int nb, int d, double sigma, double *K,
                                     int64_t ldk, int flags, double diag_shift, void *stream)
{
    return kernel_matrix(kLaplace, A, lda, na, B, ldb, nb, d, sigma, K, ldk, flags, diag_shift,
                         stream);
}

extern "C" int qmlg_linear_kernel(const double *A, int64_t lda, int na, const double *B,
                                  int64_t ldb, int nb, int d, double *K, int64_t ldk, int flags,
                                  double diag_shift, void *stream)
{
    return kernel_matrix(kLinear, A, lda, na, B, ldb, nb, d, 1.0, K, ldk, flags, diag_shift,
                         stream);
}

extern "C" int qmlg_matern_kernel_l2(const double *A, int64_t lda, int na, const double *B,
                                     int64_t ldb, int nb, int d, double sigma, int order,
                                     double *K, int64_t ldk, int flags, double diag_shift,
                                     void *stream)
{
    if (order < 0 || order > 2) return QMLG_E_ARG;
    EpiParams ep;
    ep.order = order;
    // the reference's inv_sigma and inv_sigma2 (qml/fkernels.f90:446-479)
    ep.s1 = -std::sqrt((double)(2 * order + 1)) / sigma;
    if (order == 0) ep.s1 = -1.0 / sigma;
    ep.s2 = 5.0 / (3.0 * sigma * sigma);
    return kernel_matrix(kMaternL2, A, lda, na, B, ldb, nb, d, sigma, K, ldk, flags, diag_shift,
                         stream, ep);
}

extern "C" int qmlg_sargan_kernel(const double *A, int64_t lda, int na, const double *B,
                                  int64_t ldb, int nb, int d, double sigma, const double *gammas,
                                  int ngammas, double *K, int64_t ldk, int flags,
                                  double diag_shift, void *stream)
{
    if (ngammas < 0 || (ngammas > 0 && gammas == nullptr)) return QMLG_E_ARG;
    EpiParams ep;
    ep.gammas = gammas;
    ep.ng = ngammas;
    return kernel_matrix(kSargan, A, lda, na, B, ldb, nb, d, sigma, K, ldk, flags, diag_shift,
                         stream, ep);
}

extern "C" int qmlg_predict_gemv(const double *Ks, int64_t ldk, int ntrain, int ntest,
                                 const double *alpha, double *yhat, void *stream)
{
    if (ntrain < 0 || ntest < 0 || ldk < ntrain) return QMLG_E_ARG;
    if (ntest == 0) return QMLG_OK;
    if (Ks == nullptr || alpha == nullptr || yhat == nullptr) return QMLG_E_ARG;
    { gemv_t_kernel<<<(int)qmlg::ceil_div((int64_t)ntest * 32, 256), 256, 0,
                    qmlg::as_stream(stream)>>>(Ks, ldk, ntrain, ntest, alpha, yhat); qmlg::count_launches(1); }
    return qmlg::check_launch();
}

extern "C" size_t qmlg_predict_workspace_size(int ntrain, int ntest)
{
    qmlg::WorkspacePlan p;
    p.add<double>((size_t)qmlg::ceil_div(ntrain < 1 ? 1 : ntrain, TJ) * (size_t)ntest);  // partials
    return p.total();
}

extern "C" int qmlg_predict_fused(int kind, const double *Xtrain, int64_t ldtrain, int ntrain,
                                  const double *Xtest, int64_t ldtest, int ntest, int d,
                                  double sigma, const double *alpha, double *yhat,
                                  void *workspace, size_t ws_bytes, void *stream)
{
    if (kind != QMLG_KIND_GAUSSIAN && kind != QMLG_KIND_LAPLACIAN) return QMLG_E_ARG;
    int st = check_common(Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, sigma);
    if (st != QMLG_OK) return st;
    if (ntest == 0) return QMLG_OK;
    if (yhat == nullptr || (ntrain > 0 && alpha == nullptr)) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    if (ntrain == 0) {
        cudaError_t e = cudaMemsetAsync(yhat, 0, sizeof(double) * (size_t)ntest, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    if (ws_bytes < qmlg_predict_workspace_size(ntrain, ntest)) return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    const int tj = (int)qmlg::ceil_div(ntrain, TJ), ti = (int)qmlg::ceil_div(ntest, TI);
    dim3 grid;
    if (!tile_list_grid(tj, ti, false, grid)) return QMLG_E_ARG;
    double *partial = ws.take<double>((size_t)tj * ntest);
    if (partial == nullptr) return QMLG_E_WORKSPACE;
    const double scale = kind == QMLG_KIND_GAUSSIAN ? -0.5 / (sigma * sigma) : -1.0 / sigma;
    if (kind == QMLG_KIND_GAUSSIAN)
        { predict_partial_kernel<kGauss><<<grid, NT, 0, s>>>(
            Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, scale, alpha, partial, nullptr); qmlg::count_launches(1); }
    else
        { predict_partial_kernel<kLaplace><<<grid, NT, 0, s>>>(
            Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, scale, alpha, partial, nullptr); qmlg::count_launches(1); }
    { reduce_partial_kernel<<<(int)qmlg::ceil_div(ntest, 256), 256, 0, s>>>(partial, tj, ntest, yhat); qmlg::count_launches(1); }
    return qmlg::check_launch();
}

// ---------------------------------------------------------------------------
// Fused prediction for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at all.  An example is a serving process
// whose memory manager reserves its whole HBM budget at start-up and forbids later
// allocations, because cudaMalloc synchronises the device and can fail mid-request
// once memory is fragmented.  Such a caller may also be unable to size and hand
// over a workspace.  This variant keeps its scratch (the per-training-tile partial
// sums) in a fixed array compiled into the library, so the call allocates nothing.
//
// The array holds kNoAllocPartials doubles (32 MiB).  Every GPU that loads the
// library keeps it reserved until the process exits.  A call needs
// ceil(ntrain / 64) * ntest partial sums and is rejected with QMLG_E_TOO_LARGE
// beyond that.  Every partial sum is written before it is read, so nothing has
// to be cleared between calls.  All calls share the one array, so calls whose
// work overlaps on the GPU (different streams, or different host threads) race
// on it and must be serialised by the caller.
// ---------------------------------------------------------------------------

namespace {

constexpr size_t kNoAllocPartials = (size_t)4 << 20;  // doubles: 32 MiB
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) double g_noalloc_partials[kNoAllocPartials];

std::mutex g_noalloc_mutex;
double *g_noalloc_address[kNoAllocMaxDevices] = {};

// Device address of the array on the current device.  The host-side symbol is
// only a stand-in, so the address is looked up once per device (with that device
// current) and cached.
int noalloc_scratch(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    if (dev < 0 || dev >= kNoAllocMaxDevices) return QMLG_E_ARG;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_address[dev] == nullptr) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
        g_noalloc_address[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_address[dev];
    return QMLG_OK;
}

}  // namespace

extern "C" int qmlg_predict_fused_noalloc(int kind, const double *Xtrain, int64_t ldtrain,
                                          int ntrain, const double *Xtest, int64_t ldtest,
                                          int ntest, int d, double sigma, const double *alpha,
                                          double *yhat, void *stream)
{
    if (kind != QMLG_KIND_GAUSSIAN && kind != QMLG_KIND_LAPLACIAN) return QMLG_E_ARG;
    int st = check_common(Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, sigma);
    if (st != QMLG_OK) return st;
    if (ntest == 0) return QMLG_OK;
    if (yhat == nullptr || (ntrain > 0 && alpha == nullptr)) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    if (ntrain == 0) {
        cudaError_t e = cudaMemsetAsync(yhat, 0, sizeof(double) * (size_t)ntest, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    const int tj = (int)qmlg::ceil_div(ntrain, TJ), ti = (int)qmlg::ceil_div(ntest, TI);
    if ((size_t)tj * (size_t)ntest > kNoAllocPartials) return QMLG_E_TOO_LARGE;
    dim3 grid;  // tj * ti <= tj * ntest, far below the one-dimensional grid limit
    if (!tile_list_grid(tj, ti, false, grid)) return QMLG_E_TOO_LARGE;
    double *partial = nullptr;
    st = noalloc_scratch(&partial);
    if (st != QMLG_OK) return st;
    const double scale = kind == QMLG_KIND_GAUSSIAN ? -0.5 / (sigma * sigma) : -1.0 / sigma;
    if (kind == QMLG_KIND_GAUSSIAN) {
        predict_partial_kernel<kGauss><<<grid, NT, 0, s>>>(
            Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, scale, alpha, partial, nullptr);
    } else {
        predict_partial_kernel<kLaplace><<<grid, NT, 0, s>>>(
            Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, scale, alpha, partial, nullptr);
    }
    qmlg::count_launches(1);
    reduce_partial_kernel<<<(int)qmlg::ceil_div(ntest, 256), 256, 0, s>>>(partial, tj, ntest, yhat);
    qmlg::count_launches(1);
    return qmlg::check_launch();
}

// ---------------------------------------------------------------------------
// Laplacian kernel in exact fixed-point integer arithmetic.
//
// Every feature is rounded once to q = round(x * 2^F) (int64).  The L1 distance is
// then an exact integer sum of |q_a - q_b| (no rounding, so the result does not
// depend on the summation order and K is exactly symmetric), converted to FP64
// once: L1 = sum * 2^-F.  F is the largest scale with d * 2 * max|x| * 2^F < 2^62
// (no overflow); the rounding of the inputs moves L1 by at most d * 2^-F, i.e. K
// by at most d * 2^-F / sigma relative, which must stay below 0.5e-12 or the FP64
// kernel runs instead.  The sums run on the integer pipes, not the FP64 ones.
// ---------------------------------------------------------------------------

namespace {

__global__ void max_abs_rows_kernel(const double *__restrict__ X, int64_t ldx, int rows, int cols,
                                    unsigned long long *__restrict__ out)
{
    unsigned long long m = 0;
    const int64_t total = (int64_t)rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long b =
            (unsigned long long)__double_as_longlong(fabs(X[(e / cols) * ldx + e % cols]));
        m = b > m ? b : m;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, off);
        m = o > m ? o : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Fixed-point grid decided on the device, for the entry points that take no host
// decision: the same rule as the host code below, ok = 0 when the bound fails.
struct FixedPlan {
    double scale, inv_scale;
    int ok, pad;
};

// plan->{scale, inv_scale, ok} from the largest |x| of the operands (the bits in
// maxbits[0 .. nmax-1], as max_abs_rows_kernel leaves them); a failed bound ORs 8
// into *flag (may be null).
__global__ void fixed_plan_kernel(const unsigned long long *__restrict__ maxbits, int nmax, int d,
                                  double sigma, FixedPlan *__restrict__ plan, int *__restrict__ flag)
{
    // the largest |x| bit pattern: NaN sorts above +inf, so any NaN makes m non-finite
    // (an fmax would drop it)
    unsigned long long mbits = 0;
    for (int k = 0; k < nmax; ++k) mbits = maxbits[k] > mbits ? maxbits[k] : mbits;
    const double m = __longlong_as_double((long long)mbits);
    bool ok = isfinite(m);
    int F = 0;
    if (ok) {
        int em = 0, ed = 0;
        if (m > 0.0) frexp(m, &em);
        frexp((double)(2 * (long long)(d < 1 ? 1 : d)), &ed);
        F = min(62 - ed - em, 1000);
        ok = ldexp((double)d, -F) / sigma <= 0.5e-12;
    }
    plan->scale = ok ? ldexp(1.0, F) : 0.0;
    plan->inv_scale = ok ? ldexp(1.0, -F) : 0.0;
    plan->ok = ok ? 1 : 0;
    if (!ok && flag != nullptr) atomicOr(flag, 8);
}

// Q = round(X * scale); with a plan the scale is the plan's, and nothing is done
// when the plan failed.
__global__ void to_fixed_kernel(const double *__restrict__ X, int64_t ldx, int rows, int cols,
                                double scale, long long *__restrict__ Q,
                                const FixedPlan *__restrict__ plan)
{
    if (plan != nullptr) {
        if (!plan->ok) return;
        scale = plan->scale;
    }
    const int64_t total = (int64_t)rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = e / cols, c = e % cols;
        Q[e] = __double2ll_rn(X[r * ldx + c] * scale);
    }
}

__device__ __forceinline__ long long iabs64(long long v) { return v < 0 ? -v : v; }

// EPI 0: Laplacian exp(-d / sigma); 1: Sargan exp(-d / sigma) (1 + sum_m gamma_m t^m).
template <int EPI>
__global__ void __launch_bounds__(NT)
laplace_fixed_kernel(const long long *__restrict__ A, int na, const long long *__restrict__ B,
                     int nb, int d, double inv_scale, double neg_inv_sigma,
                     double *__restrict__ K, int64_t ldk, int symmetric, double diag_shift,
                     const FixedPlan *__restrict__ plan, const double *__restrict__ gammas, int ng)
{
    if (plan != nullptr) {  // the device-side grid: nothing to do when it failed
        if (!plan->ok) return;
        inv_scale = plan->inv_scale;
    }
    // operand chunks during the sums, the output tile (for the mirror) after
    __shared__ double smem[TI * (TJ + 1)];
    long long(*As)[TJ + 1] = reinterpret_cast<long long(*)[TJ + 1]>(smem);
    long long(*Bs)[TI + 1] = reinterpret_cast<long long(*)[TI + 1]>(smem + TK * (TJ + 1));
    double(*T)[TJ + 1] = reinterpret_cast<double(*)[TJ + 1]>(smem);
    int bj, bi;
    if (symmetric) {
        tri_index(blockIdx.x, bi, bj);
    } else {
        rect_index((na + TJ - 1) / TJ, bj, bi);
    }
    const int j0 = bj * TJ, i0 = bi * TI;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    long long acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0;
    for (int t0 = 0; t0 < d; t0 += TK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * NT;
            const int r = e >> 4, c = e & 15;
            const int t = t0 + c;
            As[c][r] = (j0 + r < na && t < d) ? A[(int64_t)(j0 + r) * d + t] : 0;
            Bs[c][r] = (i0 + r < nb && t < d) ? B[(int64_t)(i0 + r) * d + t] : 0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < TK; ++c) {
            long long av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[c][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[c][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += iabs64(av[a] - bv[b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int j = j0 + tx + 16 * a, i = i0 + ty + 16 * b;
            const double dist = (double)acc[a][b] * inv_scale;
            double v = exp(neg_inv_sigma * dist);
            if (EPI == 1) {
                // Sargan, as kernel_matrix_kernel forms it: t = d / sigma
                const double t = -neg_inv_sigma * dist;
                double pw = 1.0, sum = 0.0;
                for (int m = 0; m < ng; ++m) {
                    pw *= t;
                    sum += gammas[m] * pw;
                }
                v *= 1.0 + sum;
            }
            if (symmetric && i == j) v = 1.0 + diag_shift;
            if (j < na && i < nb) K[(int64_t)i * ldk + j] = v;
            T[ty + 16 * b][tx + 16 * a] = v;
        }
    if (symmetric && bi != bj) {
        __syncthreads();
        for (int e = tid; e < TI * TJ; e += NT) {
            const int ii = e & (TI - 1), jj = e / TI;
            const int i = i0 + ii, j = j0 + jj;
            if (i < nb && j < na) K[(int64_t)j * ldk + i] = T[ii][jj];
        }
    }
}

// Fused Laplacian prediction in fixed point: the L1 sums of laplace_fixed_kernel for
// a (training tile, test tile), then the per-test-column partial sums of k * alpha
// over the tile's training rows (in the same fixed order as predict_partial_kernel).
__global__ void __launch_bounds__(NT)
laplace_fixed_predict_kernel(const long long *__restrict__ A, int na, const long long *__restrict__ B,
                             int nb, int d, double inv_scale, double neg_inv_sigma,
                             const double *__restrict__ alpha, double *__restrict__ partial,
                             const FixedPlan *__restrict__ plan)
{
    if (plan != nullptr) {
        if (!plan->ok) return;
        inv_scale = plan->inv_scale;
    }
    __shared__ double smem[TI * (TJ + 1)];
    long long(*As)[TJ + 1] = reinterpret_cast<long long(*)[TJ + 1]>(smem);
    long long(*Bs)[TI + 1] = reinterpret_cast<long long(*)[TI + 1]>(smem + TK * (TJ + 1));
    double(*red)[TI + 1] = reinterpret_cast<double(*)[TI + 1]>(smem);
    int bj, bi;
    rect_index((na + TJ - 1) / TJ, bj, bi);
    const int j0 = bj * TJ, i0 = bi * TI;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    long long acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0;
    for (int t0 = 0; t0 < d; t0 += TK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * NT;
            const int r = e >> 4, c = e & 15;
            const int t = t0 + c;
            As[c][r] = (j0 + r < na && t < d) ? A[(int64_t)(j0 + r) * d + t] : 0;
            Bs[c][r] = (i0 + r < nb && t < d) ? B[(int64_t)(i0 + r) * d + t] : 0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < TK; ++c) {
            long long av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[c][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[c][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] += iabs64(av[a] - bv[b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int i = i0 + ty + 16 * b;
        double sum = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int j = j0 + tx + 16 * a;
            if (j < na && i < nb)
                sum = fma(exp(neg_inv_sigma * ((double)acc[a][b] * inv_scale)), alpha[j], sum);
        }
        red[tx][ty + 16 * b] = sum;
    }
    __syncthreads();
    if (tid < TI) {
        double sum = 0.0;
        for (int q = 0; q < 16; ++q) sum += red[q][tid];
        const int i = i0 + tid;
        if (i < nb) partial[(int64_t)bj * nb + i] = sum;
    }
}

}  // namespace

extern "C" size_t qmlg_laplacian_kernel_fixed_workspace_size(int na, int nb, int d, int flags)
{
    qmlg::WorkspacePlan p;
    p.add<long long>((size_t)na * d);
    if (!(flags & QMLG_KERNEL_SYMMETRIC)) p.add<long long>((size_t)nb * d);
    p.add<unsigned long long>(2);
    p.add<FixedPlan>(1);
    return p.total();
}

namespace {

// The FP64 kernel behind a fixed-point call that cannot meet its bound.
int l1_fp64(const double *A, int64_t lda, int na, const double *B, int64_t ldb, int nb, int d,
            double sigma, const double *gammas, int ng, double *K, int64_t ldk, int flags,
            double diag_shift, void *stream)
{
    return gammas == nullptr
               ? qmlg_laplacian_kernel(A, lda, na, B, ldb, nb, d, sigma, K, ldk, flags, diag_shift,
                                       stream)
               : qmlg_sargan_kernel(A, lda, na, B, ldb, nb, d, sigma, gammas, ng, K, ldk, flags,
                                    diag_shift, stream);
}

// L1 kernel matrices from exact fixed-point sums: the Laplacian (gammas == nullptr)
// or the Sargan kernel.  gain multiplies the grid's bound on t = d / sigma, for an
// epilogue that passes an error in t into K amplified.
int fixed_l1_matrix(const double *A, int64_t lda, int na, const double *B, int64_t ldb, int nb,
                    int d, double sigma, const double *gammas, int ng, double gain, double *K,
                    int64_t ldk, int flags, double diag_shift, void *workspace, size_t ws_bytes,
                    void *stream)
{
    int st = check_common(A, lda, na, B, ldb, nb, d, sigma);
    if (st != QMLG_OK) return st;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    const bool symmetric = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (symmetric && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    const int tj = (int)qmlg::ceil_div(na, TJ), ti = (int)qmlg::ceil_div(nb, TI);
    dim3 grid;
    if (!tile_list_grid(tj, ti, symmetric, grid)) return QMLG_E_ARG;
    if (ws_bytes < qmlg_laplacian_kernel_fixed_workspace_size(na, nb, d, flags))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    long long *qa = ws.take<long long>((size_t)na * d);
    long long *qb = symmetric ? qa : ws.take<long long>((size_t)nb * d);
    unsigned long long *mx = ws.take<unsigned long long>(2);
    if (qa == nullptr || qb == nullptr || mx == nullptr) return QMLG_E_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    auto blocks = [](int64_t total) { return (int)std::min<int64_t>(qmlg::ceil_div(total, 256), 2432); };
    max_abs_rows_kernel<<<blocks((int64_t)na * d), 256, 0, s>>>(A, lda, na, d, mx);
    if (!symmetric) max_abs_rows_kernel<<<blocks((int64_t)nb * d), 256, 0, s>>>(B, ldb, nb, d, mx + 1);
    qmlg::count_launches(symmetric ? 1 : 2);
    unsigned long long h[2] = {0, 0};
    st = qmlg::read_back(h, mx, sizeof(h), s);
    if (st != QMLG_OK) return st;
    // the larger |x| bit pattern: a NaN in either operand makes m non-finite
    const unsigned long long hb = symmetric ? h[0] : std::max(h[0], h[1]);
    double m;
    std::memcpy(&m, &hb, sizeof(double));
    if (!std::isfinite(m))
        return l1_fp64(A, lda, na, B, ldb, nb, d, sigma, gammas, ng, K, ldk, flags, diag_shift,
                       stream);
    int em = 0;
    if (m > 0.0) std::frexp(m, &em);  // m < 2^em
    int ed = 0;
    std::frexp((double)(2 * (int64_t)(d < 1 ? 1 : d)), &ed);  // 2d <= 2^ed
    const int F = std::min(62 - ed - em, 1000);
    const double bound = std::ldexp((double)d, -F) / sigma;
    if (gain * bound > 0.5e-12)  // not representable finely enough: the FP64 kernel
        return l1_fp64(A, lda, na, B, ldb, nb, d, sigma, gammas, ng, K, ldk, flags, diag_shift,
                       stream);
    const double scale = std::ldexp(1.0, F), inv_scale = std::ldexp(1.0, -F);
    to_fixed_kernel<<<blocks((int64_t)na * d), 256, 0, s>>>(A, lda, na, d, scale, qa, nullptr);
    if (!symmetric)
        to_fixed_kernel<<<blocks((int64_t)nb * d), 256, 0, s>>>(B, ldb, nb, d, scale, qb, nullptr);
    qmlg::count_launches(symmetric ? 1 : 2);
    if (gammas == nullptr)
        laplace_fixed_kernel<0><<<grid, NT, 0, s>>>(qa, na, qb, nb, d, inv_scale, -1.0 / sigma, K,
                                                    ldk, symmetric ? 1 : 0, diag_shift, nullptr,
                                                    nullptr, 0);
    else
        laplace_fixed_kernel<1><<<grid, NT, 0, s>>>(qa, na, qb, nb, d, inv_scale, -1.0 / sigma, K,
                                                    ldk, symmetric ? 1 : 0, diag_shift, nullptr,
                                                    gammas, ng);
    qmlg::count_launches(1);
    return qmlg::check_launch();
}

}  // namespace

extern "C" int qmlg_laplacian_kernel_fixed(const double *A, int64_t lda, int na, const double *B,
                                           int64_t ldb, int nb, int d, double sigma, double *K,
                                           int64_t ldk, int flags, double diag_shift,
                                           void *workspace, size_t ws_bytes, void *stream)
{
    return fixed_l1_matrix(A, lda, na, B, ldb, nb, d, sigma, nullptr, 0, 1.0, K, ldk, flags,
                           diag_shift, workspace, ws_bytes, stream);
}

extern "C" size_t qmlg_sargan_kernel_fixed_workspace_size(int na, int nb, int d, int flags)
{
    return qmlg_laplacian_kernel_fixed_workspace_size(na, nb, d, flags);
}

// With t = d / sigma, ln K = -t + ln(1 + sum_m gamma_m t^m).  For gamma_m >= 0 the
// polynomial is >= 1 and its log-derivative is at most ng max(1, sum gamma), so an
// error in t reaches K relative at most (1 + ng max(1, sum gamma)) times; that factor
// tightens the grid's bound.  A negative gamma takes the FP64 kernel.
extern "C" int qmlg_sargan_kernel_fixed(const double *A, int64_t lda, int na, const double *B,
                                        int64_t ldb, int nb, int d, double sigma,
                                        const double *gammas, int ng, double *K, int64_t ldk,
                                        int flags, double diag_shift, void *workspace,
                                        size_t ws_bytes, void *stream)
{
    if (ng < 0 || (ng > 0 && gammas == nullptr)) return QMLG_E_ARG;
    if (ng == 0)
        return fixed_l1_matrix(A, lda, na, B, ldb, nb, d, sigma, nullptr, 0, 1.0, K, ldk, flags,
                               diag_shift, workspace, ws_bytes, stream);
    std::vector<double> g(ng);
    cudaStream_t s = qmlg::as_stream(stream);
    int st = qmlg::read_back(g.data(), gammas, sizeof(double) * ng, s);
    if (st != QMLG_OK) return st;
    double sum = 0.0;
    bool nonneg = true;
    for (double v : g) {
        nonneg = nonneg && v >= 0.0 && std::isfinite(v);
        sum += v;
    }
    if (!nonneg)
        return qmlg_sargan_kernel(A, lda, na, B, ldb, nb, d, sigma, gammas, ng, K, ldk, flags,
                                  diag_shift, stream);
    const double gain = 1.0 + ng * std::fmax(1.0, sum);
    return fixed_l1_matrix(A, lda, na, B, ldb, nb, d, sigma, gammas, ng, gain, K, ldk, flags,
                           diag_shift, workspace, ws_bytes, stream);
}

extern "C" size_t qmlg_predict_laplacian_fixed_workspace_size(int ntrain, int ntest, int d)
{
    qmlg::WorkspacePlan p;
    p.add<double>((size_t)qmlg::ceil_div(ntrain < 1 ? 1 : ntrain, TJ) * (size_t)ntest);  // partials
    p.add<long long>((size_t)ntrain * d);
    p.add<long long>((size_t)ntest * d);
    p.add<unsigned long long>(2);
    p.add<FixedPlan>(1);
    return p.total();
}

extern "C" int qmlg_predict_laplacian_fixed(const double *Xtrain, int64_t ldtrain, int ntrain,
                                            const double *Xtest, int64_t ldtest, int ntest, int d,
                                            double sigma, const double *alpha, double *yhat,
                                            void *workspace, size_t ws_bytes, void *stream)
{
    int st = check_common(Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, sigma);
    if (st != QMLG_OK) return st;
    if (ntest == 0) return QMLG_OK;
    if (yhat == nullptr || (ntrain > 0 && alpha == nullptr)) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    if (ntrain == 0) {
        cudaError_t e = cudaMemsetAsync(yhat, 0, sizeof(double) * (size_t)ntest, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    if (ws_bytes < qmlg_predict_laplacian_fixed_workspace_size(ntrain, ntest, d))
        return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    const int tj = (int)qmlg::ceil_div(ntrain, TJ), ti = (int)qmlg::ceil_div(ntest, TI);
    dim3 grid;
    if (!tile_list_grid(tj, ti, false, grid)) return QMLG_E_ARG;
    double *partial = ws.take<double>((size_t)tj * ntest);
    long long *qa = ws.take<long long>((size_t)ntrain * d);
    long long *qb = ws.take<long long>((size_t)ntest * d);
    unsigned long long *mx = ws.take<unsigned long long>(2);
    if (partial == nullptr || qa == nullptr || qb == nullptr || mx == nullptr)
        return QMLG_E_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    auto blocks = [](int64_t total) { return (int)std::min<int64_t>(qmlg::ceil_div(total, 256), 2432); };
    max_abs_rows_kernel<<<blocks((int64_t)ntrain * d), 256, 0, s>>>(Xtrain, ldtrain, ntrain, d, mx);
    max_abs_rows_kernel<<<blocks((int64_t)ntest * d), 256, 0, s>>>(Xtest, ldtest, ntest, d, mx + 1);
    qmlg::count_launches(2);
    unsigned long long h[2] = {0, 0};
    if ((st = qmlg::read_back(h, mx, sizeof(h), s)) != QMLG_OK) return st;
    // the larger |x| bit pattern: a NaN in either operand makes m non-finite
    const unsigned long long hb = std::max(h[0], h[1]);
    double m;
    std::memcpy(&m, &hb, sizeof(double));
    // the same fixed-point grid and 1e-12 bound as qmlg_laplacian_kernel_fixed
    int F = 0;
    bool fixed = std::isfinite(m);
    if (fixed) {
        int em = 0;
        if (m > 0.0) std::frexp(m, &em);
        int ed = 0;
        std::frexp((double)(2 * (int64_t)(d < 1 ? 1 : d)), &ed);
        F = std::min(62 - ed - em, 1000);
        fixed = std::ldexp((double)d, -F) / sigma <= 0.5e-12;
    }
    if (fixed) {
        const double scale = std::ldexp(1.0, F), inv_scale = std::ldexp(1.0, -F);
        to_fixed_kernel<<<blocks((int64_t)ntrain * d), 256, 0, s>>>(Xtrain, ldtrain, ntrain, d,
                                                                    scale, qa, nullptr);
        to_fixed_kernel<<<blocks((int64_t)ntest * d), 256, 0, s>>>(Xtest, ldtest, ntest, d, scale,
                                                                   qb, nullptr);
        laplace_fixed_predict_kernel<<<grid, NT, 0, s>>>(qa, ntrain, qb, ntest, d, inv_scale,
                                                         -1.0 / sigma, alpha, partial, nullptr);
        qmlg::count_launches(3);
    } else {
        predict_partial_kernel<kLaplace><<<grid, NT, 0, s>>>(
            Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, -1.0 / sigma, alpha, partial, nullptr);
        qmlg::count_launches(1);
    }
    { reduce_partial_kernel<<<(int)qmlg::ceil_div(ntest, 256), 256, 0, s>>>(partial, tj, ntest, yhat); qmlg::count_launches(1); }
    return qmlg::check_launch();
}

// ---------------------------------------------------------------------------
// Capture-safe fixed-point Laplacian entry points.
//
// They take no host decision and read nothing back, so they can be recorded into a
// CUDA graph and issued by serving threads that keep several streams busy.  The
// fixed-point grid is decided on the device by the host rule above
// (fixed_plan_kernel).  The FP64 kernel is launched beside the fixed-point one:
// whichever of the two the plan does not select returns at once, so the result is
// always written, and a failed bound ORs 8 into *d_flag (may be null) to record
// that the FP64 kernel produced it.
// ---------------------------------------------------------------------------

extern "C" int qmlg_laplacian_kernel_fixed_async(const double *A, int64_t lda, int na,
                                                 const double *B, int64_t ldb, int nb, int d,
                                                 double sigma, double *K, int64_t ldk, int flags,
                                                 double diag_shift, int *d_flag, void *workspace,
                                                 size_t ws_bytes, void *stream)
{
    int st = check_common(A, lda, na, B, ldb, nb, d, sigma);
    if (st != QMLG_OK) return st;
    if (K == nullptr || ldk < na) return QMLG_E_ARG;
    const bool symmetric = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (symmetric && (na != nb || A != B || lda != ldb)) return QMLG_E_ARG;
    if (na == 0 || nb == 0) return QMLG_OK;
    const int tj = (int)qmlg::ceil_div(na, TJ), ti = (int)qmlg::ceil_div(nb, TI);
    dim3 grid;
    if (!tile_list_grid(tj, ti, symmetric, grid)) return QMLG_E_ARG;
    if (ws_bytes < qmlg_laplacian_kernel_fixed_workspace_size(na, nb, d, flags))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    long long *qa = ws.take<long long>((size_t)na * d);
    long long *qb = symmetric ? qa : ws.take<long long>((size_t)nb * d);
    unsigned long long *mx = ws.take<unsigned long long>(2);
    FixedPlan *plan = ws.take<FixedPlan>(1);
    if (qa == nullptr || qb == nullptr || mx == nullptr || plan == nullptr) return QMLG_E_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    auto blocks = [](int64_t total) { return (int)std::min<int64_t>(qmlg::ceil_div(total, 256), 2432); };
    max_abs_rows_kernel<<<blocks((int64_t)na * d), 256, 0, s>>>(A, lda, na, d, mx);
    if (!symmetric) max_abs_rows_kernel<<<blocks((int64_t)nb * d), 256, 0, s>>>(B, ldb, nb, d, mx + 1);
    fixed_plan_kernel<<<1, 1, 0, s>>>(mx, symmetric ? 1 : 2, d, sigma, plan, d_flag);
    to_fixed_kernel<<<blocks((int64_t)na * d), 256, 0, s>>>(A, lda, na, d, 0.0, qa, plan);
    if (!symmetric)
        to_fixed_kernel<<<blocks((int64_t)nb * d), 256, 0, s>>>(B, ldb, nb, d, 0.0, qb, plan);
    laplace_fixed_kernel<0><<<grid, NT, 0, s>>>(qa, na, qb, nb, d, 0.0, -1.0 / sigma, K, ldk,
                                             symmetric ? 1 : 0, diag_shift, plan, nullptr, 0);
    EpiParams ep;
    ep.s1 = -1.0 / sigma;
    kernel_matrix_kernel<kLaplace><<<grid, NT, 0, s>>>(A, lda, na, B, ldb, nb, d, ep, K, ldk,
                                                       symmetric ? 1 : 0, diag_shift, &plan->ok);
    qmlg::count_launches(symmetric ? 5 : 7);
    return qmlg::check_launch();
}

extern "C" int qmlg_predict_laplacian_fixed_async(const double *Xtrain, int64_t ldtrain, int ntrain,
                                                  const double *Xtest, int64_t ldtest, int ntest,
                                                  int d, double sigma, const double *alpha,
                                                  double *yhat, int *d_flag, void *workspace,
                                                  size_t ws_bytes, void *stream)
{
    int st = check_common(Xtrain, ldtrain, ntrain, Xtest, ldtest, ntest, d, sigma);
    if (st != QMLG_OK) return st;
    if (ntest == 0) return QMLG_OK;
    if (yhat == nullptr || (ntrain > 0 && alpha == nullptr)) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    if (ntrain == 0) {
        cudaError_t e = cudaMemsetAsync(yhat, 0, sizeof(double) * (size_t)ntest, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    if (ws_bytes < qmlg_predict_laplacian_fixed_workspace_size(ntrain, ntest, d))
        return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    const int tj = (int)qmlg::ceil_div(ntrain, TJ), ti = (int)qmlg::ceil_div(ntest, TI);
    dim3 grid;
    if (!tile_list_grid(tj, ti, false, grid)) return QMLG_E_ARG;
    double *partial = ws.take<double>((size_t)tj * ntest);
    long long *qa = ws.take<long long>((size_t)ntrain * d);
    long long *qb = ws.take<long long>((size_t)ntest * d);
    unsigned long long *mx = ws.take<unsigned long long>(2);
    FixedPlan *plan = ws.take<FixedPlan>(1);
    if (partial == nullptr || qa == nullptr || qb == nullptr || mx == nullptr || plan == nullptr)
        return QMLG_E_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    auto blocks = [](int64_t total) { return (int)std::min<int64_t>(qmlg::ceil_div(total, 256), 2432); };
    max_abs_rows_kernel<<<blocks((int64_t)ntrain * d), 256, 0, s>>>(Xtrain, ldtrain, ntrain, d, mx);
    max_abs_rows_kernel<<<blocks((int64_t)ntest * d), 256, 0, s>>>(Xtest, ldtest, ntest, d, mx + 1);
    fixed_plan_kernel<<<1, 1, 0, s>>>(mx, 2, d, sigma, plan, d_flag);
    to_fixed_kernel<<<blocks((int64_t)ntrain * d), 256, 0, s>>>(Xtrain, ldtrain, ntrain, d, 0.0, qa,
                                                                plan);
    to_fixed_kernel<<<blocks((int64_t)ntest * d), 256, 0, s>>>(Xtest, ldtest, ntest, d, 0.0, qb, plan);
    laplace_fixed_predict_kernel<<<grid, NT, 0, s>>>(qa, ntrain, qb, ntest, d, 0.0, -1.0 / sigma,
                                                     alpha, partial, plan);
    predict_partial_kernel<kLaplace><<<grid, NT, 0, s>>>(Xtrain, ldtrain, ntrain, Xtest, ldtest,
                                                         ntest, d, -1.0 / sigma, alpha, partial,
                                                         &plan->ok);
    reduce_partial_kernel<<<(int)qmlg::ceil_div(ntest, 256), 256, 0, s>>>(partial, tj, ntest, yhat);
    qmlg::count_launches(9);
    return qmlg::check_launch();
}
