// Symmetric indefinite solve and inverse by Bunch-Kaufman diagonal pivoting.
//
// Restates LAPACK's dsytf2 (lower, the unblocked form of the dsytrf that fbkf_solve /
// fbkf_invert call, qml/fcho_solve.f90:76-150) and dsytrs:
//   alpha = (1 + sqrt 17)/8; at step k, colmax = max_{i>k} |a_ik| (first index imax);
//   |a_kk| >= alpha colmax: 1x1 pivot k; else rowmax = max_{j != imax} |a_imax,j| over
//   the trailing matrix; |a_kk| >= alpha colmax (colmax/rowmax): 1x1 pivot k;
//   |a_imax,imax| >= alpha rowmax: 1x1 pivot imax; else 2x2 pivot (k, imax);
//   the pivot row/column is swapped into place (symmetric interchange of the trailing
//   matrix), then the rank-1 or rank-2 trailing update and the L columns;
//   ipiv as LAPACK's (1-based; negative for both columns of a 2x2 block); a zero
//   column sets info = k+1 and is skipped, as dsytf2 does.
// Storage: the row-major lower triangle W[i][j], i >= j (the column-major lower
// triangle dsytrf("L") works on, seen transposed).
//
// One cooperative kernel runs the whole factorisation, four grid barriers per
// pivot step: CTA 0 decides the pivot (block reductions), the grid swaps, copies
// the pivot columns and multipliers, then updates the trailing triangle one row per
// warp (four independent elements per lane in flight) while writing the L columns.
// Everything another CTA wrote since the last barrier is read through L2
// (ld.global.cg), never through a possibly stale L1 line.  The inverse is the Schur complement left by
// the first n steps on [[A, I], [I, 0]] with the pivot search confined to A's rows
// (a symmetric permutation inside A's block leaves that complement -A^-1).
#include <algorithm>
#include <cmath>

#include <cooperative_groups.h>

#include "common.cuh"
#include "emulated_gemm.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int BK_THREADS = 1024;

struct BkArgs {
    double *W;
    int64_t ld;
    int N;        // matrix size (trailing updates run over [k, N))
    int nsearch;  // pivots are taken, and searched for, among indices < nsearch
    int *ipiv;    // [nsearch]
    int *info;
    double *x0, *x1;  // [N] copies of the pivot columns / 2x2 multipliers
    int *dec;         // [4] the step's decision: kp, kstep, zero column
};

__device__ __forceinline__ void bk_sync(cg::grid_group &g)
{
    if (gridDim.x == 1) __syncthreads();
    else g.sync();
}

// Block-wide (max |value|, first index) reduction; every thread gets the result.
__device__ void block_argmax(double &v, int &idx, double *sv, int *si)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, v, off);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ov > v || (ov == v && oi < idx)) {
            v = ov;
            idx = oi;
        }
    }
    if (lane == 0) {
        sv[warp] = v;
        si[warp] = idx;
    }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < BK_THREADS / 32; ++w)
            if (sv[w] > sv[0] || (sv[w] == sv[0] && si[w] < si[0])) {
                sv[0] = sv[w];
                si[0] = si[w];
            }
    }
    __syncthreads();
    v = sv[0];
    idx = si[0];
    __syncthreads();
}

__global__ void __launch_bounds__(BK_THREADS) bk_factor_kernel(BkArgs a)
{
    cg::grid_group g = cg::this_grid();
    __shared__ double sv[BK_THREADS / 32];
    __shared__ int si[BK_THREADS / 32];
    const double alpha = (1.0 + sqrt(17.0)) / 8.0;
    double *W = a.W;
    const int64_t ld = a.ld;
    const int N = a.N, ns = a.nsearch;
    const int tid = threadIdx.x;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + tid, gsz = (int64_t)gridDim.x * blockDim.x;
    const int warp_g = (int)(gt >> 5), nwarps = (int)(gsz >> 5), lane = tid & 31;
    int k = 0;
    while (k < ns) {
        // ---- decide the pivot (CTA 0)
        if (blockIdx.x == 0) {
            double cm = 0.0;
            int imax = k;
            for (int i = k + 1 + tid; i < ns; i += BK_THREADS) {
                const double v = fabs(__ldcg(W + (int64_t)i * ld + k));
                if (v > cm) {
                    cm = v;
                    imax = i;
                }
            }
            block_argmax(cm, imax, sv, si);
            const double absakk = fabs(__ldcg(W + (int64_t)k * ld + k));
            int kp = k, kstep = 1, zero = 0;
            if (fmax(absakk, cm) == 0.0) {
                zero = 1;
            } else if (!(absakk >= alpha * cm)) {
                // rowmax over row/column imax of the trailing block
                double rm = 0.0;
                int jdummy = 0;
                for (int j = k + tid; j < imax; j += BK_THREADS)
                    rm = fmax(rm, fabs(__ldcg(W + (int64_t)imax * ld + j)));
                for (int i = imax + 1 + tid; i < ns; i += BK_THREADS)
                    rm = fmax(rm, fabs(__ldcg(W + (int64_t)i * ld + imax)));
                block_argmax(rm, jdummy, sv, si);
                if (absakk >= alpha * cm * (cm / rm)) {
                    kp = k;
                } else if (fabs(__ldcg(W + (int64_t)imax * ld + imax)) >= alpha * rm) {
                    kp = imax;
                } else {
                    kp = imax;
                    kstep = 2;
                }
            }
            if (tid == 0) {
                a.dec[0] = kp;
                a.dec[1] = kstep;
                a.dec[2] = zero;
                if (zero && *a.info == 0) *a.info = k + 1;
            }
        }
        bk_sync(g);
        const int kp = __ldcg(a.dec), kstep = __ldcg(a.dec + 1), zero = __ldcg(a.dec + 2);
        const int kk = k + kstep - 1;
        // ---- symmetric interchange of kk and kp in the trailing block
        if (!zero && kp != kk) {
            // items: [0] the diagonal, (k..kk) row entries, (kk..kp) the middle,
            // (kp..N) the columns below kp
            const int nleft = kk - k, nmid = kp - kk - 1, nbelow = N - kp - 1;
            const int64_t total = 1 + nleft + nmid + nbelow;
            for (int64_t t = gt; t < total; t += gsz) {
                double *p, *q;
                if (t == 0) {
                    p = W + (int64_t)kk * ld + kk;
                    q = W + (int64_t)kp * ld + kp;
                } else if (t <= nleft) {
                    const int j = k + (int)(t - 1);
                    p = W + (int64_t)kk * ld + j;
                    q = W + (int64_t)kp * ld + j;
                } else if (t <= nleft + nmid) {
                    const int m = kk + 1 + (int)(t - 1 - nleft);
                    p = W + (int64_t)m * ld + kk;
                    q = W + (int64_t)kp * ld + m;
                } else {
                    const int i = kp + 1 + (int)(t - 1 - nleft - nmid);
                    p = W + (int64_t)i * ld + kk;
                    q = W + (int64_t)i * ld + kp;
                }
                const double tmp = __ldcg(p);
                *p = __ldcg(q);
                *q = tmp;
            }
        }
        bk_sync(g);
        // ---- pivot columns (copies) and 2x2 multipliers
        if (!zero) {
            if (kstep == 1) {
                for (int64_t i = k + 1 + gt; i < N; i += gsz) a.x0[i] = __ldcg(W + i * ld + k);
            } else {
                const double d21 = __ldcg(W + (int64_t)(k + 1) * ld + k);
                const double d11 = __ldcg(W + (int64_t)(k + 1) * ld + k + 1) / d21;
                const double d22 = __ldcg(W + (int64_t)k * ld + k) / d21;
                const double t = 1.0 / (d11 * d22 - 1.0);
                const double e21 = t / d21;
                for (int64_t j = k + 2 + gt; j < N; j += gsz) {
                    const double ajk = __ldcg(W + j * ld + k), ajk1 = __ldcg(W + j * ld + k + 1);
                    a.x0[j] = e21 * (d11 * ajk - ajk1);   // wk
                    a.x1[j] = e21 * (d22 * ajk1 - ajk);   // wkp1
                }
            }
        }
        bk_sync(g);
        // ---- trailing update (one row per warp) and the L columns
        if (!zero) {
            const double *x0 = a.x0, *x1 = a.x1;
            if (kstep == 1) {
                const double r = 1.0 / __ldcg(W + (int64_t)k * ld + k);
                for (int i = k + 1 + warp_g; i < N; i += nwarps) {
                    const double xi = __ldcg(x0 + i);
                    const double f = -xi * r;
                    double *row = W + (int64_t)i * ld;
                    int j = k + 1 + lane;
                    for (; j + 96 <= i; j += 128) {  // loads of four elements, then their FMAs
                        const double r0 = __ldcg(row + j), r1 = __ldcg(row + j + 32);
                        const double r2 = __ldcg(row + j + 64), r3 = __ldcg(row + j + 96);
                        const double y0 = __ldcg(x0 + j), y1 = __ldcg(x0 + j + 32);
                        const double y2 = __ldcg(x0 + j + 64), y3 = __ldcg(x0 + j + 96);
                        row[j] = fma(f, y0, r0);
                        row[j + 32] = fma(f, y1, r1);
                        row[j + 64] = fma(f, y2, r2);
                        row[j + 96] = fma(f, y3, r3);
                    }
                    for (; j <= i; j += 32) row[j] = fma(f, __ldcg(x0 + j), __ldcg(row + j));
                    if (lane == 0) row[k] = xi * r;
                }
            } else {
                for (int i = k + 2 + warp_g; i < N; i += nwarps) {
                    double *row = W + (int64_t)i * ld;
                    const double aik = __ldcg(row + k), aik1 = __ldcg(row + k + 1);
                    int j = k + 2 + lane;
                    for (; j + 96 <= i; j += 128) {
                        double rv[4], u[4], v[4];
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            rv[t] = __ldcg(row + j + 32 * t);
                            u[t] = __ldcg(x0 + j + 32 * t);
                            v[t] = __ldcg(x1 + j + 32 * t);
                        }
#pragma unroll
                        for (int t = 0; t < 4; ++t) row[j + 32 * t] = rv[t] - (aik * u[t] + aik1 * v[t]);
                    }
                    for (; j <= i; j += 32)
                        row[j] = __ldcg(row + j) - (aik * __ldcg(x0 + j) + aik1 * __ldcg(x1 + j));
                }
            }
        }
        bk_sync(g);
        if (!zero && kstep == 2) {
            for (int64_t j = k + 2 + gt; j < N; j += gsz) {
                W[j * ld + k] = a.x0[j];
                W[j * ld + k + 1] = a.x1[j];
            }
        }
        if (gt == 0) {
            if (kstep == 1) {
                a.ipiv[k] = kp + 1;
            } else {
                a.ipiv[k] = -(kp + 1);
                a.ipiv[k + 1] = -(kp + 1);
            }
        }
        bk_sync(g);
        k += kstep;
    }
}

// dsytrs (lower, one right-hand side) with the factor above, in one CTA.
__global__ void __launch_bounds__(1024)
bk_solve_kernel(const double *__restrict__ W, int64_t ld, int n, const int *__restrict__ ipiv,
                double *__restrict__ b)
{
    __shared__ double red[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    auto block_sum = [&](double v) -> double {
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[warp] = v;
        __syncthreads();
        double s = 0.0;
        if (tid == 0)
            for (int w = 0; w < (nt + 31) / 32; ++w) s += red[w];
        __syncthreads();
        return s;  // valid in thread 0
    };
    // L D x = b
    int k = 0;
    while (k < n) {
        if (ipiv[k] > 0) {
            const int kp = ipiv[k] - 1;
            if (tid == 0 && kp != k) {
                const double t = b[k];
                b[k] = b[kp];
                b[kp] = t;
            }
            __syncthreads();
            const double bk = b[k];
            for (int i = k + 1 + tid; i < n; i += nt) b[i] -= W[(int64_t)i * ld + k] * bk;
            __syncthreads();
            if (tid == 0) b[k] = bk / W[(int64_t)k * ld + k];
            __syncthreads();
            k += 1;
        } else {
            const int kp = -ipiv[k] - 1;
            if (tid == 0 && kp != k + 1) {
                const double t = b[k + 1];
                b[k + 1] = b[kp];
                b[kp] = t;
            }
            __syncthreads();
            const double b0 = b[k], b1 = b[k + 1];
            for (int i = k + 2 + tid; i < n; i += nt)
                b[i] -= W[(int64_t)i * ld + k] * b0 + W[(int64_t)i * ld + k + 1] * b1;
            __syncthreads();
            if (tid == 0) {
                const double akm1k = W[(int64_t)(k + 1) * ld + k];
                const double akm1 = W[(int64_t)k * ld + k] / akm1k;
                const double ak = W[(int64_t)(k + 1) * ld + k + 1] / akm1k;
                const double denom = akm1 * ak - 1.0;
                const double bkm1 = b0 / akm1k, bk = b1 / akm1k;
                b[k] = (ak * bkm1 - bk) / denom;
                b[k + 1] = (akm1 * bk - bkm1) / denom;
            }
            __syncthreads();
            k += 2;
        }
    }
    // L^T x = b
    k = n - 1;
    while (k >= 0) {
        if (ipiv[k] > 0) {
            double s = 0.0;
            for (int i = k + 1 + tid; i < n; i += nt) s += W[(int64_t)i * ld + k] * b[i];
            s = block_sum(s);
            if (tid == 0) {
                b[k] -= s;
                const int kp = ipiv[k] - 1;
                if (kp != k) {
                    const double t = b[k];
                    b[k] = b[kp];
                    b[kp] = t;
                }
            }
            __syncthreads();
            k -= 1;
        } else {
            // the 2x2 block (k-1, k)
            double s0 = 0.0, s1 = 0.0;
            for (int i = k + 1 + tid; i < n; i += nt) {
                s1 += W[(int64_t)i * ld + k] * b[i];
                s0 += W[(int64_t)i * ld + k - 1] * b[i];
            }
            s1 = block_sum(s1);
            s0 = block_sum(s0);
            if (tid == 0) {
                b[k] -= s1;
                b[k - 1] -= s0;
                const int kp = -ipiv[k] - 1;
                if (kp != k) {
                    const double t = b[k];
                    b[k] = b[kp];
                    b[kp] = t;
                }
            }
            __syncthreads();
            k -= 2;
        }
    }
}

// W's lower triangle (ldw = N): A's column-major lower triangle, and for the inverse
// (N = 2n) the identity coupling block below it.
__global__ void bk_build_kernel(const double *__restrict__ A, int64_t lda, int n, int N,
                                double *__restrict__ W)
{
    const int64_t total = (int64_t)N * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / N), c = (int)(e % N);
        if (c > r) continue;
        double v = 0.0;
        if (r < n) v = A[(int64_t)r + (int64_t)c * lda];
        else if (c < n) v = (c == r - n) ? 1.0 : 0.0;
        W[(int64_t)r * N + c] = v;
    }
}

__global__ void bk_extract_kernel(const double *__restrict__ W, int n, double *__restrict__ Ainv,
                                  int64_t ldi)
{
    const int N = 2 * n;
    const int64_t total = (int64_t)n * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const int hi = i > j ? i : j, lo = i > j ? j : i;
        Ainv[(int64_t)i + (int64_t)j * ldi] = -W[(int64_t)(n + hi) * N + (n + lo)];
    }
}

struct BkBufs {
    int *info, *dec, *ipiv;
    double *W, *x0, *x1;
};

size_t bk_ws(int n, int N)
{
    qmlg::WorkspacePlan p;
    p.add<int>(4);
    p.add<int>(4);
    p.add<int>((size_t)std::max(n, 1));
    p.add<double>((size_t)N * N);
    p.add<double>((size_t)N);
    p.add<double>((size_t)N);
    return p.total();
}

int bk_factor(const double *A, int64_t lda, int n, int N, void *workspace, size_t ws_bytes,
              BkBufs &b, cudaStream_t s)
{
    if (ws_bytes < bk_ws(n, N)) return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    b.info = ws.take<int>(4);
    b.dec = ws.take<int>(4);
    b.ipiv = ws.take<int>((size_t)std::max(n, 1));
    b.W = ws.take<double>((size_t)N * N);
    b.x0 = ws.take<double>((size_t)N);
    b.x1 = ws.take<double>((size_t)N);
    cudaError_t e = cudaMemsetAsync(b.info, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const int blocks = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)N * N, 256), 152 * 64);
    { bk_build_kernel<<<blocks, 256, 0, s>>>(A, lda, n, N, b.W); qmlg::count_launches(1); }
    BkArgs a{b.W, (int64_t)N, N, n, b.ipiv, b.info, b.x0, b.x1, b.dec};
    int grid = 1;
    if (N > 256 && qmlg::cooperative_allowed_on(s)) {
        int dev = 0, sms = 0, per = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, bk_factor_kernel, BK_THREADS, 0)) !=
                cudaSuccess)
            return qmlg::set_cuda_error(e);
        grid = std::max(1, std::min(qmlg::sm_limit(sms), sms * std::max(per, 1)));
    }
    if (grid > 1) {
        void *args[] = {(void *)&a};
        return qmlg::launch_cooperative_serialised((const void *)bk_factor_kernel, grid, BK_THREADS,
                                                   args, s);
    }
    bk_factor_kernel<<<1, BK_THREADS, 0, s>>>(a);
    qmlg::count_launches(1);
    return qmlg::check_launch();
}

}  // namespace

extern "C" size_t qmlg_bkf_solve_workspace_size(int n) { return bk_ws(n, n); }

extern "C" int qmlg_bkf_solve(const double *A, int n, int64_t lda, const double *y, double *x,
                              void *workspace, size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    if (A == nullptr || y == nullptr || x == nullptr) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    BkBufs b;
    int st = bk_factor(A, lda, n, n, workspace, ws_bytes, b, s);
    if (st != QMLG_OK) return st;
    cudaError_t e = cudaMemcpyAsync(x, y, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    { bk_solve_kernel<<<1, 1024, 0, s>>>(b.W, n, n, b.ipiv, x); qmlg::count_launches(1); }
    if ((st = qmlg::check_launch()) != QMLG_OK) return st;
    int info = 0;
    st = qmlg::read_back(&info, b.info, sizeof(int), s);
    return st != QMLG_OK ? st : info;
}

extern "C" size_t qmlg_bkf_invert_workspace_size(int n) { return bk_ws(n, 2 * std::max(n, 1)); }

extern "C" int qmlg_bkf_invert(const double *A, int n, int64_t lda, double *Ainv, int64_t ldi,
                               void *workspace, size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n || ldi < n) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    if (A == nullptr || Ainv == nullptr) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    BkBufs b;
    int st = bk_factor(A, lda, n, 2 * n, workspace, ws_bytes, b, s);
    if (st != QMLG_OK) return st;
    const int eb = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)n * n, 256), 152 * 64);
    { bk_extract_kernel<<<eb, 256, 0, s>>>(b.W, n, Ainv, ldi); qmlg::count_launches(1); }
    if ((st = qmlg::check_launch()) != QMLG_OK) return st;
    int info = 0;
    st = qmlg::read_back(&info, b.info, sizeof(int), s);
    return st != QMLG_OK ? st : info;
}
