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
// Two forms.  Above N = 256 (outside stream capture) the blocked form below (LAPACK's
// dlasyf, "blocked form").  Otherwise one CTA runs the unblocked dsytf2 kernel
// bk_factor_kernel, written for a cooperative grid, two barriers per pivot step:
//   1. CTA 0 decides the pivot.  Column k comes from a contiguous copy and its
//      maximum from per-CTA partials, both left by the previous step's update; only
//      the row-max search reads the matrix (row imax, and column imax, which it
//      keeps).  CTA 0 then writes the pivot column(s) as they will be after the
//      interchange and the 2x2 multipliers, all read from before it.
//   2. The grid applies the interchange, the trailing update and the L columns in
//      one pass.  Each moved element is read from the copy of row/column kk.  The
//      trailing triangle is cut into 128-element row segments spread over all
//      warps, four independent elements per lane.  The segments at the diagonal's
//      left end also copy out columns k+kstep and k+kstep+1 and the partial maxima
//      for the next step.
// Its arithmetic is dsytf2's, operation for operation.
// Everything another CTA wrote since the last barrier is read through L2
// (ld.global.cg, never a possibly stale L1 line) by loads that the compiler may not
// move across the barrier; the step's decision is read once per CTA, by the thread
// that took part in the barrier's handshake, and shared through shared memory.
// The inverse is the Schur complement left by the first n steps on [[A, I], [I, 0]]
// with the pivot search confined to A's rows (a symmetric permutation inside A's
// block leaves that complement -A^-1).
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
    double *col;      // [2][2][N] columns k and k+1 of the current matrix, two generations
    double *ci;       // [N] column imax below imax, saved by the row-max search
    double *p0, *p1;  // [N] the pivot column(s) after the interchange
    double *w0, *w1;  // [N] the 2x2 pivot's multipliers
    double *sc;       // [4] the pivot block after the interchange
    double *pv;       // [grid] per-CTA partial column maxima (value, first index)
    int *pi;
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

__device__ __forceinline__ int ld_relaxed_gpu(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Loads through L2 (never a possibly stale L1 line) of what other CTAs wrote before
// the last grid barrier.  The memory clobber keeps the compiler from moving them
// above the barrier.
__device__ __forceinline__ double ld_l2(const double *p)
{
    double v;
    asm volatile("ld.global.cg.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_l2(const int *p)
{
    int v;
    asm volatile("ld.global.cg.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The panel kernel's maxima compare |v| as integer keys (the bits of a non-negative
// double order as its value), which keeps them off the FP64 pipe; a NaN gets key 0
// and so never wins, as it never compares greater.
__device__ __forceinline__ unsigned long long abs_key(double v)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return u > 0x7ff0000000000000ull ? 0ull : u;
}

__device__ __forceinline__ void key_step(double v, int i, unsigned long long &bk, int &bi)
{
    const unsigned long long kv = abs_key(v);
    if (kv > bk || (kv == bk && i < bi)) {
        bk = kv;
        bi = i;
    }
}

__device__ __forceinline__ void warp_argmax_key(unsigned long long &key, int &idx)
{
    for (int off = 16; off > 0; off >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, off);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ok > key || (ok == key && oi < idx)) {
            key = ok;
            idx = oi;
        }
    }
}

// This CTA's (max, first index) to pv/pi[blockIdx.x] (pv as the double |v|).
__device__ void publish_partial_key(double *pv, int *pi, unsigned long long key, int idx,
                                    unsigned long long *sk, int *si)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_argmax_key(key, idx);
    if (lane == 0) {
        sk[warp] = key;
        si[warp] = idx;
    }
    __syncthreads();
    if (warp == 0) {
        key = lane < (int)(blockDim.x >> 5) ? sk[lane] : 0ull;
        idx = lane < (int)(blockDim.x >> 5) ? si[lane] : 0x7fffffff;
        warp_argmax_key(key, idx);
        if (lane == 0) {
            pv[blockIdx.x] = __longlong_as_double((long long)key);
            if (pi != nullptr) pi[blockIdx.x] = idx;
        }
    }
}

// Keeps (max |v|, first index) over the values a thread sees.
__device__ __forceinline__ void argmax_step(double v, int i, double &bv, int &bi)
{
    const double av = fabs(v);
    if (av > bv || (av == bv && i < bi)) {
        bv = av;
        bi = i;
    }
}

// Writes this CTA's (max, first index) to the partials (all threads take part).
__device__ void publish_partial(double *pv, int *pi, double bv, int bi, double *sv, int *si)
{
    block_argmax(bv, bi, sv, si);
    if (threadIdx.x == 0) {
        pv[blockIdx.x] = bv;
        if (pi != nullptr) pi[blockIdx.x] = bi;
    }
}

// Copies columns c and c+1 (rows >= c, resp. c+1) of W into column generation g and
// publishes the partial maxima of column c over rows (c, ns).
__device__ void load_columns(const BkArgs &a, int c, int gen, double *sv, int *si)
{
    const int N = a.N;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gsz = (int64_t)gridDim.x * blockDim.x;
    double *cA = a.col + (int64_t)(2 * gen) * N, *cB = cA + N;
    double bv = 0.0;
    int bi = c;
    for (int64_t i = c + gt; i < N; i += gsz) {
        const double v = ld_l2(a.W + i * a.ld + c);
        cA[i] = v;
        if (i > c && i < a.nsearch) argmax_step(v, (int)i, bv, bi);
        if (i > c) cB[i] = ld_l2(a.W + i * a.ld + c + 1);
    }
    publish_partial(a.pv, a.pi, bv, bi, sv, si);
}

__global__ void __launch_bounds__(BK_THREADS) bk_factor_kernel(BkArgs a)
{
    cg::grid_group g = cg::this_grid();
    __shared__ double sv[BK_THREADS / 32];
    __shared__ int si[BK_THREADS / 32];
    __shared__ int sdec[3];
    const double alpha = (1.0 + sqrt(17.0)) / 8.0;
    double *W = a.W;
    const int64_t ld = a.ld;
    const int N = a.N, ns = a.nsearch;
    const int tid = threadIdx.x;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + tid;
    const unsigned warp_g = (unsigned)(gt >> 5), nwarps = (unsigned)((int64_t)gridDim.x * blockDim.x >> 5);
    const int lane = tid & 31;
    int k = 0, gen = 0;
    load_columns(a, 0, 0, sv, si);
    bk_sync(g);
    while (k < ns) {
        const double *cA = a.col + (int64_t)(2 * gen) * N, *cB = cA + N;
        // ---- decide the pivot (CTA 0) from the partial maxima of column k
        if (blockIdx.x == 0) {
            double cm = 0.0;
            int imax = k;
            for (int b = tid; b < (int)gridDim.x; b += BK_THREADS) {
                const double v = ld_l2(a.pv + b);
                const int i = ld_l2(a.pi + b);
                if (v > cm || (v == cm && i < imax)) {
                    cm = v;
                    imax = i;
                }
            }
            block_argmax(cm, imax, sv, si);
            const double absakk = fabs(ld_l2(cA + k));
            int kp = k, kstep = 1, zero = 0;
            if (fmax(absakk, cm) == 0.0) {
                zero = 1;
            } else if (!(absakk >= alpha * cm)) {
                // rowmax over row/column imax of the trailing block; column imax
                // below imax is kept for the interchange
                double rm = 0.0;
                int jdummy = 0;
                for (int j = k + tid; j < imax; j += BK_THREADS)
                    rm = fmax(rm, fabs(ld_l2(W + (int64_t)imax * ld + j)));
                for (int i = imax + 1 + tid; i < N; i += BK_THREADS) {
                    const double v = ld_l2(W + (int64_t)i * ld + imax);
                    a.ci[i] = v;
                    if (i < ns) rm = fmax(rm, fabs(v));
                }
                block_argmax(rm, jdummy, sv, si);
                if (absakk >= alpha * cm * (cm / rm)) {
                    kp = k;
                } else if (fabs(ld_l2(W + (int64_t)imax * ld + imax)) >= alpha * rm) {
                    kp = imax;
                } else {
                    kp = imax;
                    kstep = 2;
                }
            }
            if (!zero) {
                // The symmetric interchange of kk = k + kstep - 1 and kp, read from
                // the matrix before it: new (i, j) = old (sig i, sig j).  Column k
                // (and k+1) come from the column copies, row kp from W, column kp
                // below kp from the copy the search made.
                const double *rowp = W + (int64_t)kp * ld;
                const double *ci = a.ci;
                if (kstep == 1) {
                    if (kp != k) {
                        for (int i = k + 1 + tid; i < N; i += BK_THREADS)
                            a.p0[i] = i < kp ? ld_l2(rowp + i) : (i == kp ? ld_l2(cA + kp) : ld_l2(ci + i));
                        if (tid == 0) a.sc[0] = ld_l2(rowp + kp);
                    } else if (tid == 0) {
                        a.sc[0] = ld_l2(cA + k);
                    }
                } else {
                    const double d21 = ld_l2(cA + kp);
                    const double d11 = ld_l2(rowp + kp) / d21;
                    const double d22 = ld_l2(cA + k) / d21;
                    const double t = 1.0 / (d11 * d22 - 1.0);
                    const double e21 = t / d21;
                    for (int j = k + 2 + tid; j < N; j += BK_THREADS) {
                        const double ajk = ld_l2(cA + (j == kp ? k + 1 : j));
                        const double ajk1 = j < kp ? ld_l2(rowp + j) : (j == kp ? ld_l2(rowp + k + 1) : ld_l2(ci + j));
                        a.p0[j] = ajk;
                        a.p1[j] = ajk1;
                        a.w0[j] = e21 * (d11 * ajk - ajk1);   // wk
                        a.w1[j] = e21 * (d22 * ajk1 - ajk);   // wkp1
                    }
                    if (tid == 0) {
                        a.sc[0] = ld_l2(cA + k);
                        a.sc[1] = d21;
                        a.sc[2] = ld_l2(rowp + kp);
                    }
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
        // the decision, read once per CTA by the thread that took part in the grid
        // barrier's handshake and handed to the others through shared memory
        if (tid == 0) {
            sdec[0] = ld_relaxed_gpu(a.dec);
            sdec[1] = ld_relaxed_gpu(a.dec + 1);
            sdec[2] = ld_relaxed_gpu(a.dec + 2);
        }
        __syncthreads();
        const int kp = sdec[0], kstep = sdec[1], zero = sdec[2];
        const int kk = k + kstep - 1, kn = k + kstep;
        const int ngen = gen ^ 1;
        double *nA = a.col + (int64_t)(2 * ngen) * N, *nB = nA + N;
        if (zero) {
            // nothing to update: the next step's columns straight from W
            load_columns(a, kn, ngen, sv, si);
        } else {
            // ---- the interchange, the trailing update and the L columns, the
            // trailing triangle cut into 128-element row segments spread over all
            // warps (four independent elements per lane); the segment at the
            // diagonal's left end also saves columns kn and kn+1 for the next step
            const bool swap = kp != kk;
            // row/column kk before the interchange: column k or k+1 of the copy
            const double *rkk = kstep == 1 ? cA : cB;
            const double okk = swap ? ld_l2(rkk + kk) : 0.0;
            const double *x0 = kstep == 1 ? (swap ? a.p0 : cA) : a.w0;
            const double *x1 = a.w1;
            const double *q0 = kstep == 1 ? x0 : a.p0, *q1 = a.p1;
            double r = 0.0;
            if (kstep == 1) {
                const double akk = ld_l2(a.sc);
                r = 1.0 / akk;
                if (gt == 0) W[(int64_t)k * ld + k] = akk;
            } else if (gt == 0) {
                W[(int64_t)k * ld + k] = ld_l2(a.sc);
                W[(int64_t)(k + 1) * ld + k] = ld_l2(a.sc + 1);
                W[(int64_t)(k + 1) * ld + k + 1] = ld_l2(a.sc + 2);
            }
            double bv = 0.0;
            int bi = kn;
            const int m = N - kn;
            const unsigned nseg = (unsigned)(m + 127) >> 7;
            const unsigned items = (unsigned)m * nseg;
            for (unsigned t = warp_g; t < items; t += nwarps) {
                const unsigned c = t / (unsigned)m, rr = t - c * (unsigned)m;
                const int i = kn + (int)rr, j0 = kn + (int)(c << 7);
                if (j0 > i) continue;
                double *row = W + (int64_t)i * ld;
                const bool rowkp = swap && i == kp;
                double ov[4], u[4], v[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = j0 + lane + 32 * e;
                    ov[e] = u[e] = v[e] = 0.0;
                    if (j <= i) {
                        // the value of new (i, j) before the update
                        ov[e] = rowkp ? (j == i ? okk : ld_l2(rkk + j))
                                      : (swap && j == kp ? ld_l2(rkk + i) : ld_l2(row + j));
                        u[e] = ld_l2(x0 + j);
                        if (kstep == 2) v[e] = ld_l2(x1 + j);
                    }
                }
                double nv[4];
                if (kstep == 1) {
                    const double xi = ld_l2(q0 + i);
                    const double f = -xi * r;
#pragma unroll
                    for (int e = 0; e < 4; ++e) nv[e] = fma(f, u[e], ov[e]);
                    if (c == 0 && lane == 0) row[k] = xi * r;
                } else {
                    const double aik = ld_l2(q0 + i), aik1 = ld_l2(q1 + i);
#pragma unroll
                    for (int e = 0; e < 4; ++e) nv[e] = ov[e] - (aik * u[e] + aik1 * v[e]);
                    if (c == 0 && lane == 0) {
                        row[k] = ld_l2(x0 + i);
                        row[k + 1] = ld_l2(x1 + i);
                    }
                }
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int j = j0 + lane + 32 * e;
                    if (j <= i) row[j] = nv[e];
                }
                if (c == 0) {
                    if (lane == 0) {
                        nA[i] = nv[0];
                        if (i > kn && i < ns) argmax_step(nv[0], i, bv, bi);
                    } else if (lane == 1 && i > kn) {
                        nB[i] = nv[0];
                    }
                }
            }
            publish_partial(a.pv, a.pi, bv, bi, sv, si);
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
        k = kn;
        gen = ngen;
    }
}

// ---------------------------------------------------------------- blocked form --
//
// LAPACK's dsytrf with dlasyf (lower, qml/fcho_solve.f90:76-150 calls dsytrf):
// panels of up to BK_NB columns are factorised with their trailing updates delayed
// (each column of the panel is brought up to date on the fly from the panel's L
// columns and the W = L D columns before it), then the trailing triangle takes the
// whole panel at once, A22 -= L21 W21^T: an emulated-FP64 product on the tensor
// cores (emu_tc_update) for the solve, FP64 for the inverse (bk_factor_blocked).
// As in dlasyf a panel stops one column early unless its last pivot is 2x2 (the
// row-max search needs a spare W column), and the interchanges that a panel applied
// to its own earlier L columns are undone afterwards, which leaves the factor in
// dsytf2's form.
//
// The panel kernel is cooperative, one thread block per SM, two grid barriers per
// column (three when the row-max search runs, one when a step without interchange
// shares its phase with the next column's update).  Every CTA takes the pivot decision
// itself from per-CTA partial maxima, so no barrier waits on one CTA's decision.
// The W rows that an interchange swaps are written to a two-row stage and put in
// place during the next column's update, because every CTA still reads them while
// the interchange is applied.

constexpr int BK_NB = 64;

struct BkPanelArgs {
    double *W;         // the matrix, row-major lower triangle
    int64_t ld;
    int N, nsearch;
    int k0;            // the panel's first column
    double *Wp;        // [N][BK_NB] the panel's W = L D columns, by matrix row
    double *stage;     // [2][BK_NB] rows kk and kp of Wp after the last interchange
    int *ipiv, *info;
    double *pv, *pv2;  // [grid] partial column maxima and row maxima
    int *pi;
    int *kb_out;       // columns this panel factorised
    // the inverse (N > nsearch), else null: perm[p] is the original index at position
    // p, kept through the interchanges (the coupling rows are ordered by it)
    int *perm;
};

// A row's dot product over the lanes of a warp: lane l holds the products of columns
// l (l0 r0) and l + 32 (l1 r1); lanes at or above m (the number of columns) hold
// zeros, and the levels of the reduction that would only add those zeros to lane 0
// are skipped (the FP64 pipe is the scarce one).  The sum is valid in lane 0.
__device__ __forceinline__ double row_dot(double l0, double r0, double l1, double r1, int m)
{
    double dot = m > 32 ? fma(l1, r1, l0 * r0) : l0 * r0;
    const int top = m > 16 ? 16 : (m > 8 ? 8 : (m > 4 ? 4 : (m > 2 ? 2 : (m > 1 ? 1 : 0))));
    for (int off = top; off > 0; off >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, off);
    return dot;
}

// v = (the current, non-updated) A(i, col) - sum_{c < kc} L(i, k0 + c) Wp(rrow, c) for
// rows i in [k, N), one warp per row; the result goes to Wp[i][dst].  src(i) gives
// the element's address (row or column of A, whichever the lower triangle holds).
template <class Src, class Keep>
__device__ __forceinline__ void panel_column(const BkPanelArgs &a, int k, int kc, const double *rrow,
                                             int dst, Src src, Keep keep)
{
    const int lane = threadIdx.x & 31;
    const unsigned warp_g = (unsigned)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const unsigned nwarps = (unsigned)((int64_t)gridDim.x * blockDim.x >> 5);
    const double r0 = lane < kc ? ld_l2(rrow + lane) : 0.0;
    const double r1 = lane + 32 < kc ? ld_l2(rrow + lane + 32) : 0.0;
    for (int i = k + (int)warp_g; i < a.N; i += (int)nwarps) {
        const double *row = a.W + (int64_t)i * a.ld + a.k0;
        const double l0 = lane < kc ? ld_l2(row + lane) : 0.0;
        const double l1 = lane + 32 < kc ? ld_l2(row + lane + 32) : 0.0;
        const double own = lane == 0 ? ld_l2(src(i)) : 0.0;
        const double dot = row_dot(l0, r0, l1, r1, kc);
        if (lane == 0) {
            const double v = own - dot;
            a.Wp[(int64_t)i * BK_NB + dst] = v;
            keep(v, i);
        }
    }
}

// The position-to-original-index map through the step's interchange (kk <-> kp,
// kk < 0 for none).  One thread.
__device__ __forceinline__ void mark_coupling(const BkPanelArgs &a, int k, int kstep, int kk, int kp)
{
    if (a.perm == nullptr || kk < 0) return;
    const int t = a.perm[kk];
    a.perm[kk] = a.perm[kp];
    a.perm[kp] = t;
}

// Every CTA reduces the partials (value, first index) itself, in warp 0, and hands
// the result to its threads through res (one block barrier).
__device__ void reduce_partials(const double *pv, const int *pi, double &v, int &idx, double *res_v,
                                int *res_i)
{
    if (threadIdx.x < 32) {
        unsigned long long key = 0ull;
        idx = 0x7fffffff;
        // the loads of a lane all issued before the first compare (a loop of load and
        // compare would wait out one L2 round trip per partial)
        constexpr int U = 8;
        for (int b0 = threadIdx.x; b0 < (int)gridDim.x; b0 += 32 * U) {
            double xv[U];
            int iv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int b = b0 + 32 * u;
                xv[u] = b < (int)gridDim.x ? ld_l2(pv + b) : 0.0;
                iv[u] = (b < (int)gridDim.x && pi != nullptr) ? ld_l2(pi + b) : 0x7fffffff;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const unsigned long long x = (unsigned long long)__double_as_longlong(xv[u]);
                if (x > key || (x == key && iv[u] < idx)) {
                    key = x;
                    idx = iv[u];
                }
            }
        }
        warp_argmax_key(key, idx);
        if (threadIdx.x == 0) {
            *res_v = __longlong_as_double((long long)key);
            *res_i = idx;
        }
    }
    __syncthreads();
    v = *res_v;
    idx = *res_i;
}

__global__ void __launch_bounds__(BK_THREADS) bk_panel_kernel(BkPanelArgs a)
{
    cg::grid_group g = cg::this_grid();
    __shared__ unsigned long long sk[BK_THREADS / 32];
    __shared__ int si[BK_THREADS / 32];
    __shared__ double res_v[2];
    __shared__ int res_i[2];
    const double alpha = (1.0 + sqrt(17.0)) / 8.0;
    double *W = a.W, *Wp = a.Wp;
    const int64_t ld = a.ld;
    const int N = a.N, ns = a.nsearch, k0 = a.k0;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t gt = (int64_t)blockIdx.x * blockDim.x + tid, gsz = (int64_t)gridDim.x * blockDim.x;
    auto wrow = [&](int i) { return Wp + (int64_t)i * BK_NB; };
    // the interchange of the previous column whose W rows are still in the stage
    int pend = 0, pkk = 0, pkp = 0, pcols = 0;
    const unsigned warp_g = (unsigned)(gt >> 5), nwarps = (unsigned)(gsz >> 5);
    int k = k0;
    bool have_col = false;  // column k already brought up to date by the previous phase
    while (k < ns && k - k0 < BK_NB - 1) {
        const int kc = k - k0;
        // ---- column k brought up to date: Wp[:, kc], partial max over rows (k, ns)
        if (!have_col) {
            const double *rrow = (pend && k == pkp) ? a.stage + BK_NB : wrow(k);
            unsigned long long bv = 0ull;
            int bi = 0x7fffffff;
            panel_column(a, k, kc, rrow, kc, [&](int i) { return W + (int64_t)i * ld + k; },
                         [&](double v, int i) {
                             if (i > k && i < ns) key_step(v, i, bv, bi);
                         });
            if (pend && blockIdx.x == 0 && warp == 0) {
                for (int c = lane; c < pcols; c += 32) {
                    wrow(pkk)[c] = ld_l2(a.stage + c);
                    wrow(pkp)[c] = ld_l2(a.stage + BK_NB + c);
                }
            }
            pend = 0;
            publish_partial_key(a.pv, a.pi, bv, bi, sk, si);
            bk_sync(g);
        }
        have_col = false;
        // ---- the pivot decision, taken by every CTA
        const double wkk = ld_l2(wrow(k) + kc);
        double colmax;
        int imax;
        reduce_partials(a.pv, a.pi, colmax, imax, res_v, res_i);
        const double absakk = fabs(wkk);
        int kp = k, kstep = 1, zero = 0, copy = 0;
        // row imax's updated entries in columns kc and kc+1 (the row-max search):
        // with wkk they are the whole pivot block, after any interchange
        double wimk = 0.0, wimim = 0.0;
        if (fmax(absakk, colmax) == 0.0) {
            zero = 1;
        } else if (!(absakk >= alpha * colmax)) {
            // column imax brought up to date into Wp[:, kc+1]; row max over it
            // without its diagonal, within the search rows
            unsigned long long rv = 0ull;
            int rdummy = 0;
            const int im = imax;
            panel_column(a, k, kc, wrow(im), kc + 1,
                         [&](int i) { return i < im ? W + (int64_t)im * ld + i : W + (int64_t)i * ld + im; },
                         [&](double v, int i) {
                             if (i != im && i < ns) {
                                 const unsigned long long kv = abs_key(v);
                                 rv = kv > rv ? kv : rv;
                             }
                         });
            publish_partial_key(a.pv2, nullptr, rv, rdummy, sk, si);
            bk_sync(g);
            wimim = ld_l2(wrow(im) + kc + 1);  // issued before the reduction's loads
            wimk = ld_l2(wrow(im) + kc);
            double rowmax;
            reduce_partials(a.pv2, nullptr, rowmax, rdummy, res_v + 1, res_i + 1);
            if (absakk >= alpha * colmax * (colmax / rowmax)) {
                kp = k;
            } else if (fabs(wimim) >= alpha * rowmax) {
                kp = im;
                copy = 1;  // W column kc takes the updated column imax
            } else {
                kp = im;
                kstep = 2;
            }
        }
        const int kk = k + kstep - 1;
        const bool swap = !zero && kp != kk;
        const int src = copy ? kc + 1 : kc;
        const int kn = k + kstep;
        if (!zero && !swap && kn < ns && kn - k0 < BK_NB - 1) {
            // ---- no interchange: the L column(s) and D of this step and the next
            // column brought up to date in one phase, each row by one warp (lane 0
            // forms the row's new L values and hands them to the lanes of the dot
            // product); the arithmetic is that of the separate phases
            const int kcn = kn - k0;
            const double *rrow = wrow(kn);
            const double r0 = lane < kcn ? ld_l2(rrow + lane) : 0.0;
            const double r1 = lane + 32 < kcn ? ld_l2(rrow + lane + 32) : 0.0;
            double d = 0.0, rcp = 0.0, d21 = 0.0, d11 = 0.0, d22 = 0.0, e21 = 0.0, wk1 = 0.0, wk11 = 0.0;
            if (kstep == 1) {
                d = wkk;
                rcp = 1.0 / d;
            } else {
                wk1 = wimk;  // no interchange: imax == k + 1
                wk11 = wimim;
                d21 = wk1;
                d11 = wk11 / d21;
                d22 = wkk / d21;
                const double t = 1.0 / (d11 * d22 - 1.0);
                e21 = t / d21;
            }
            unsigned long long bv = 0ull;
            int bi = 0x7fffffff;
            for (int i = k + (int)warp_g; i < N; i += (int)nwarps) {
                double *wrowi = W + (int64_t)i * ld;
                const double *wi = wrow(i);
                const double l0m = lane < kc ? ld_l2(wrowi + k0 + lane) : 0.0;
                const double l1m = lane + 32 < kc ? ld_l2(wrowi + k0 + lane + 32) : 0.0;
                const double own = (lane == 0 && i >= kn) ? ld_l2(wrowi + kn) : 0.0;
                double la = 0.0, lb = 0.0;
                if (lane == 0) {
                    if (kstep == 1) {
                        if (i == k) {
                            wrowi[k] = d;
                        } else {
                            la = ld_l2(wi + kc) * rcp;
                            wrowi[k] = la;
                        }
                    } else if (i == k) {
                        wrowi[k] = wkk;
                    } else if (i == k + 1) {
                        wrowi[k] = wk1;
                        wrowi[k + 1] = wk11;
                    } else {
                        const double u = ld_l2(wi + kc), w = ld_l2(wi + kc + 1);
                        la = e21 * (d11 * u - w);
                        lb = e21 * (d22 * w - u);
                        wrowi[k] = la;
                        wrowi[k + 1] = lb;
                    }
                }
                if (i >= kn) {
                    la = __shfl_sync(0xffffffffu, la, 0);
                    lb = __shfl_sync(0xffffffffu, lb, 0);
                    double l0 = l0m, l1 = l1m;
                    if (kc < 32) {
                        if (lane == kc) l0 = la;
                    } else if (lane == kc - 32) {
                        l1 = la;
                    }
                    if (kstep == 2) {
                        if (kc + 1 < 32) {
                            if (lane == kc + 1) l0 = lb;
                        } else if (lane == kc + 1 - 32) {
                            l1 = lb;
                        }
                    }
                    const double dot = row_dot(l0, r0, l1, r1, kcn);
                    if (lane == 0) {
                        const double v = own - dot;
                        Wp[(int64_t)i * BK_NB + kcn] = v;
                        if (i > kn && i < ns) key_step(v, i, bv, bi);
                    }
                }
            }
            publish_partial_key(a.pv, a.pi, bv, bi, sk, si);
            if (gt == 0) {
                if (kstep == 1) {
                    a.ipiv[k] = kp + 1;
                } else {
                    a.ipiv[k] = -(kp + 1);
                    a.ipiv[k + 1] = -(kp + 1);
                }
                mark_coupling(a, k, kstep, -1, kp);
            }
            bk_sync(g);
            k = kn;
            have_col = true;
            continue;
        }
        // ---- the interchange, the L columns and D
        if (zero) {
            // dsytf2 leaves the (current) column and takes no update from it
            for (int64_t i = k + gt; i < N; i += gsz) {
                double *w = wrow((int)i) + kc;
                W[i * ld + k] = ld_l2(w);
                *w = 0.0;
            }
        } else if (kstep == 1) {
            const double d = kp == k ? wkk : wimim;  // W(sig k, src): row k, or imax's copied column
            const double r = 1.0 / d;
            for (int64_t ii = k + gt; ii < N; ii += gsz) {
                const int i = (int)ii;
                if (swap && (i == kk || i == kp)) continue;
                double *wi = wrow(i);
                const double oldkk = (swap && i > kk) ? ld_l2(W + ii * ld + kk) : 0.0;
                const double v = ld_l2(wi + src);
                if (copy) wi[kc] = v;
                if (i == k) W[ii * ld + k] = d;
                else W[ii * ld + k] = v * r;
                if (swap && i > kk) {
                    if (i < kp) W[(int64_t)kp * ld + i] = oldkk;
                    else W[ii * ld + kp] = oldkk;
                }
            }
            if (swap && gt == 0) {
                const double dkk = ld_l2(W + (int64_t)kk * ld + kk), vkp = ld_l2(wrow(kk) + src);
                W[(int64_t)kp * ld + kp] = dkk;
                W[(int64_t)k * ld + k] = d;
                W[(int64_t)kp * ld + k] = vkp * r;
            }
        } else {
            const double d21 = wimk;  // sig(k + 1) == imax
            const double d11 = wimim / d21;
            const double d22 = wkk / d21;
            const double t = 1.0 / (d11 * d22 - 1.0);
            const double e21 = t / d21;
            for (int64_t ii = k + gt; ii < N; ii += gsz) {
                const int i = (int)ii;
                if (swap && (i == kk || i == kp)) continue;
                const double *wi = wrow(i);
                const double oldkk = (swap && i > kk) ? ld_l2(W + ii * ld + kk) : 0.0;
                if (i == k) {
                    W[ii * ld + k] = ld_l2(wi + kc);
                } else if (i == k + 1) {
                    W[ii * ld + k] = ld_l2(wi + kc);
                    W[ii * ld + k + 1] = ld_l2(wi + kc + 1);
                } else {
                    const double u = ld_l2(wi + kc), w = ld_l2(wi + kc + 1);
                    W[ii * ld + k] = e21 * (d11 * u - w);
                    W[ii * ld + k + 1] = e21 * (d22 * w - u);
                }
                if (swap && i > kk) {
                    if (i < kp) W[(int64_t)kp * ld + i] = oldkk;
                    else W[ii * ld + kp] = oldkk;
                }
            }
            if (swap && gt == 0) {
                const double *wkk = wrow(kk), *wkp = wrow(kp);
                const double dkk = ld_l2(W + (int64_t)kk * ld + kk);
                const double p0 = ld_l2(wkp + kc), p1 = ld_l2(wkp + kc + 1);
                const double u = ld_l2(wkk + kc), w = ld_l2(wkk + kc + 1);
                W[(int64_t)kp * ld + kp] = dkk;
                W[(int64_t)(k + 1) * ld + k] = p0;
                W[(int64_t)(k + 1) * ld + k + 1] = p1;
                W[(int64_t)kp * ld + k] = e21 * (d11 * u - w);
                W[(int64_t)kp * ld + k + 1] = e21 * (d22 * w - u);
            }
        }
        if (swap && blockIdx.x == 0 && warp == 0) {
            // rows kk and kp of the panel's L columns before k trade places, and
            // their W rows (after the copy) go to the stage; every load is issued
            // before the first store (columns < BK_NB: two per lane)
            double lx[2], ly[2], sa[2], sb[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = k0 + lane + 32 * h;
                lx[h] = c < k ? ld_l2(W + (int64_t)kk * ld + c) : 0.0;
                ly[h] = c < k ? ld_l2(W + (int64_t)kp * ld + c) : 0.0;
                const int cw = lane + 32 * h;
                const int cs = (copy && cw == kc) ? kc + 1 : cw;
                sa[h] = cw <= kk - k0 ? ld_l2(wrow(kp) + cs) : 0.0;
                sb[h] = cw <= kk - k0 ? ld_l2(wrow(kk) + cs) : 0.0;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = k0 + lane + 32 * h;
                if (c < k) {
                    W[(int64_t)kk * ld + c] = ly[h];
                    W[(int64_t)kp * ld + c] = lx[h];
                }
                const int cw = lane + 32 * h;
                if (cw <= kk - k0) {
                    a.stage[cw] = sa[h];
                    a.stage[BK_NB + cw] = sb[h];
                }
            }
        }
        if (swap) {
            pend = 1;
            pkk = kk;
            pkp = kp;
            pcols = kk - k0 + 1;
        }
        if (gt == 0) {
            if (kstep == 1) {
                a.ipiv[k] = kp + 1;
            } else {
                a.ipiv[k] = -(kp + 1);
                a.ipiv[k + 1] = -(kp + 1);
            }
            if (zero && *a.info == 0) *a.info = k + 1;
            mark_coupling(a, k, kstep, swap ? kk : -1, kp);
        }
        bk_sync(g);
        k += kstep;
    }
    if (pend && blockIdx.x == 0 && warp == 0) {
        for (int c = lane; c < pcols; c += 32) {
            wrow(pkk)[c] = ld_l2(a.stage + c);
            wrow(pkp)[c] = ld_l2(a.stage + BK_NB + c);
        }
    }
    if (gt == 0) *a.kb_out = k - k0;
}

// W[i][j] -= sum_{c < kb} L(i, k0 + c) Wp(j, c) over the trailing lower triangle
// i >= j >= k1, FP64, 64 x 64 tiles (the FP64 form of the panel's trailing update).
__device__ __forceinline__ void bk_tri_index(int64_t t, int &bi, int &bj)
{
    int64_t r = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = (int)r;
    bj = (int)(t - r * (r + 1) / 2);
}

__global__ void __launch_bounds__(256)
bk_update_fp64_kernel(double *__restrict__ W, int64_t ld, int N, int k0, int k1, int kb,
                      const double *__restrict__ Wp)
{
    __shared__ double Ls[16][64 + 1];
    __shared__ double Ws[16][64 + 1];
    int bi, bj;
    bk_tri_index(blockIdx.x, bi, bj);
    const int i0 = k1 + bi * 64, j0 = k1 + bj * 64;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;  // tx -> j, ty -> i
    double acc[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
    for (int t0 = 0; t0 < kb; t0 += 16) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * 256;
            const int r = e >> 4, c = e & 15;
            const int ri = i0 + r, rj = j0 + r;
            const bool in = t0 + c < kb;
            Ls[c][r] = (ri < N && in) ? W[(int64_t)ri * ld + k0 + t0 + c] : 0.0;
            Ws[c][r] = (rj < N && in) ? Wp[(int64_t)rj * BK_NB + t0 + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            double lv[4], wv[4];
#pragma unroll
            for (int v = 0; v < 4; ++v) lv[v] = Ls[c][ty + 16 * v];
#pragma unroll
            for (int u = 0; u < 4; ++u) wv[u] = Ws[c][tx + 16 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(lv[v], wv[u], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const int i = i0 + ty + 16 * v;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = j0 + tx + 16 * u;
            if (i < N && j <= i) W[(int64_t)i * ld + j] -= acc[u][v];
        }
    }
}

// ---- the inverse's coupling rows
// In [[A, I], [I, 0]] the coupling row of original index j is zero in every column
// until the column holding its 1 becomes a pivot, and each pivot brings one such row
// to life.  After every panel the coupling block is permuted (rows and columns
// together) so that coupling position p holds the row of the original index pivoted
// at position p: the live coupling rows are then [n, n + k1), and the trailing
// update only covers [k1, n + k1).  cpos/corig map original indices to coupling
// positions and back; srcmap (identity between panels) gives, for a position, the
// position its data comes from.

__global__ void bk_coupling_init_kernel(int *__restrict__ perm, int *__restrict__ cpos,
                                        int *__restrict__ corig, int *__restrict__ srcmap, int n,
                                        int *__restrict__ naff)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) perm[i] = cpos[i] = corig[i] = srcmap[i] = i;
    if (i == 0) *naff = 0;
}

// One thread: the transpositions that bring the originals pivoted at positions
// [k0, k1) to coupling positions [k0, k1), and the list of positions whose data moves.
__global__ void bk_compact_plan_kernel(const int *__restrict__ perm, int k0, int k1, int *__restrict__ cpos,
                                       int *__restrict__ corig, int *__restrict__ srcmap,
                                       int *__restrict__ aff, int *__restrict__ naff)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int m = *naff;
    for (int u = 0; u < m; ++u) srcmap[aff[u]] = aff[u];  // the last panel's moves are done
    m = 0;
    auto note = [&](int x) {
        for (int u = 0; u < m; ++u)
            if (aff[u] == x) return;
        aff[m++] = x;
    };
    for (int p = k0; p < k1; ++p) {
        const int j = perm[p], q = cpos[j];
        if (q == p) continue;
        const int jp = corig[p];
        corig[p] = j;
        cpos[j] = p;
        corig[q] = jp;
        cpos[jp] = q;
        const int sp = srcmap[p];
        srcmap[p] = srcmap[q];
        srcmap[q] = sp;
        note(p);
        note(q);
    }
    *naff = m;
}

__device__ __forceinline__ double& wsym(double *W, int64_t ld, int r, int c)
{
    return r >= c ? W[(int64_t)r * ld + c] : W[(int64_t)c * ld + r];
}

// The old full (symmetric) rows of the positions that move, and their W rows, into
// tmp (grid.y = row of the list).
__global__ void bk_compact_gather_kernel(const double *__restrict__ W, int64_t ld, int N, int n,
                                         const double *__restrict__ Wp, const int *__restrict__ aff,
                                         const int *__restrict__ naff, const int *__restrict__ srcmap,
                                         double *__restrict__ tmp, double *__restrict__ tmpw)
{
    const int u = blockIdx.y;
    if (u >= *naff) return;
    const int src = n + srcmap[aff[u]];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        tmp[(int64_t)u * N + c] = src >= c ? W[(int64_t)src * ld + c] : W[(int64_t)c * ld + src];
        if (c < BK_NB) tmpw[u * BK_NB + c] = Wp[(int64_t)src * BK_NB + c];
    }
}

// new(r, c) = old(srcmap r, srcmap c) on the moved positions' rows (and so columns).
// Where both r and c move, two threads write the same value.
__global__ void bk_compact_scatter_kernel(double *__restrict__ W, int64_t ld, int N, int n,
                                          double *__restrict__ Wp, const int *__restrict__ aff,
                                          const int *__restrict__ naff, const int *__restrict__ srcmap,
                                          const double *__restrict__ tmp, const double *__restrict__ tmpw)
{
    const int u = blockIdx.y;
    if (u >= *naff) return;
    const int r = n + aff[u];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x) {
        const int cs = c >= n ? n + srcmap[c - n] : c;
        wsym(W, ld, r, c) = tmp[(int64_t)u * N + cs];
        if (c < BK_NB) Wp[(int64_t)r * BK_NB + c] = tmpw[u * BK_NB + c];
    }
}

// Puts the panel's L columns in dsytf2's form: the interchange of each step is
// undone on the panel's columns before that step, last step first (one thread per
// column; a column's swaps run in order).
__global__ void bk_panel_undo_kernel(double *__restrict__ W, int64_t ld, int k0, const int *__restrict__ kb_in,
                                     const int *__restrict__ ipiv)
{
    const int kb = *kb_in;
    const int c = k0 + (int)threadIdx.x;
    if ((int)threadIdx.x >= kb) return;
    int j = k0 + kb - 1;
    while (j >= k0) {
        int jp = ipiv[j];
        const int jj = j;
        if (jp < 0) {
            jp = -jp;
            --j;
        }
        --j;
        jp -= 1;
        // the step's first column is j + 1; its interchange swapped rows jj and jp
        // on the columns before it
        if (jp != jj && c <= j) {
            double *x = W + (int64_t)jj * ld + c, *y = W + (int64_t)jp * ld + c;
            const double t = *x;
            *x = *y;
            *y = t;
        }
    }
}

// W[j][i] = W[i][j] for i > j: the strict lower triangle copied into the (unused)
// upper one, 32 x 32 tiles through shared memory.
__global__ void __launch_bounds__(256) bk_transpose_kernel(double *__restrict__ W, int64_t ld, int n)
{
    __shared__ double t[32][33];
    int bi, bj;
    bk_tri_index(blockIdx.x, bi, bj);
    const int i0 = bi * 32, j0 = bj * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int i = i0 + r, j = j0 + tx;
        t[r][tx] = (i < n && j < i) ? W[(int64_t)i * ld + j] : 0.0;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int j = j0 + r, i = i0 + tx;  // writes row j, column i of the upper triangle
        if (i < n && j < i) W[(int64_t)j * ld + i] = t[tx][r];
    }
}

// dsytrs (lower, one right-hand side) with the factor above, in one CTA.  L's
// column c is read as row c of the upper triangle, where bk_transpose_kernel has put
// L^T, so every load of a step is coalesced.  SH: the right-hand side is kept in
// shared memory for the whole solve (n <= BK_SOLVE_SMEM).  As in the ring kernel
// below, the D solves wait for one parallel pass and the backward sums are reduced
// through shared memory, since FP64 issue is what one SM has least of.
constexpr int BK_SOLVE_SMEM = 26112;

template <bool SH>
__global__ void __launch_bounds__(1024)
bk_solve_kernel(const double *__restrict__ W, int64_t ld, int n, const int *__restrict__ ipiv,
                double *__restrict__ bg, int *__restrict__ steps)
{
    __shared__ double red0[1024], red1[1024], q0[4], q1[4];
    extern __shared__ double sb[];
    double *b = SH ? sb : bg;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    if (SH) {
        for (int i = tid; i < n; i += nt) sb[i] = bg[i];
        __syncthreads();
    }
    // ---- L x = P b (the D solves follow in one pass)
    int k = 0;
    while (k < n) {
        const int p = ipiv[k];
        const bool two = p < 0;
        const int kp = two ? -p - 1 : p - 1, kk = two ? k + 1 : k;
        if (tid == 0) {
            steps[k] = two ? 2 : 1;
            if (two) steps[k + 1] = 0;
            if (kp != kk) {
                const double t = b[kk];
                b[kk] = b[kp];
                b[kp] = t;
            }
        }
        __syncthreads();
        const double *ck = W + (int64_t)k * ld, *ck1 = ck + ld;
        const double b0 = b[k], b1 = two ? b[k + 1] : 0.0;
        for (int i = kk + 1 + tid; i < n; i += nt) {
            if (two) b[i] -= ck[i] * b0 + ck1[i] * b1;
            else b[i] -= ck[i] * b0;
        }
        __syncthreads();
        k = kk + 1;
    }
    // ---- D x = b, every pivot block at once
    for (int c = tid; c < n; c += nt) {
        const int t = steps[c];
        if (t == 1) {
            b[c] = b[c] / W[(int64_t)c * ld + c];
        } else if (t == 2) {
            const double akm1k = W[(int64_t)(c + 1) * ld + c];
            const double akm1 = W[(int64_t)c * ld + c] / akm1k;
            const double ak = W[(int64_t)(c + 1) * ld + c + 1] / akm1k;
            const double denom = akm1 * ak - 1.0;
            const double bkm1 = b[c] / akm1k, bk = b[c + 1] / akm1k;
            b[c] = (ak * bkm1 - bk) / denom;
            b[c + 1] = (akm1 * bk - bkm1) / denom;
        }
    }
    __syncthreads();
    // ---- L^T x = b, from the last step back
    k = n - 1;
    while (k >= 0) {
        const bool two = ipiv[k] < 0;
        const int c = two ? k - 1 : k;
        const int kp = (two ? -ipiv[k] : ipiv[k]) - 1;
        const double *ck = W + (int64_t)k * ld, *cc = W + (int64_t)c * ld;
        double s0 = 0.0, s1 = 0.0;
        for (int i = k + 1 + tid; i < n; i += nt) {
            const double bi = b[i];
            s1 += ck[i] * bi;
            if (two) s0 += cc[i] * bi;
        }
        red1[tid] = s1;
        if (two) red0[tid] = s0;
        __syncthreads();
        if (warp < 4) {  // four warps reduce a quarter each (as in the ring kernel)
            double a0 = 0.0, a1 = 0.0;
            for (int j = warp * (nt >> 2) + lane; j < (warp + 1) * (nt >> 2); j += 32) {
                a1 += red1[j];
                if (two) a0 += red0[j];
            }
            for (int off = 16; off > 0; off >>= 1) {
                a1 += __shfl_xor_sync(0xffffffffu, a1, off);
                if (two) a0 += __shfl_xor_sync(0xffffffffu, a0, off);
            }
            if (lane == 0) {
                q1[warp] = a1;
                q0[warp] = a0;
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (tid == 0) {
                b[k] -= (q1[0] + q1[1]) + (q1[2] + q1[3]);
                if (two) b[k - 1] -= (q0[0] + q0[1]) + (q0[2] + q0[3]);
                if (kp != k) {
                    const double t = b[k];
                    b[k] = b[kp];
                    b[kp] = t;
                }
            }
        }
        __syncthreads();
        k = c - 1;
    }
    if (SH) {
        for (int i = tid; i < n; i += nt) bg[i] = sb[i];
    }
}

// dsytrs as above with the L columns streamed into a shared-memory ring by cp.async,
// DEPTH columns ahead of the step that uses them (column c's row of L^T, diagonal
// included, in slot c mod (DEPTH + 2)), so that no step waits on a global load.
// Needs (DEPTH + 3) n doubles of shared memory.
__device__ __forceinline__ void cp_async8(double *smem, const double *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// waits until at most `pending` (0 .. 7) of this thread's groups are in flight
__device__ __forceinline__ void cp_async_wait_pending(int pending)
{
    switch (pending) {
    case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
    case 3: asm volatile("cp.async.wait_group 3;" ::: "memory"); break;
    case 4: asm volatile("cp.async.wait_group 4;" ::: "memory"); break;
    case 5: asm volatile("cp.async.wait_group 5;" ::: "memory"); break;
    case 6: asm volatile("cp.async.wait_group 6;" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 7;" ::: "memory"); break;
    }
}

// GB300 runs FP64 at about two operations per clock per SM, so in this one-CTA
// kernel the FP64 work per step is kept to the update itself: the D solves wait
// for one parallel pass after the forward substitution (the forward steps only
// need the values before them), and the backward sums are reduced through shared
// memory by one warp (32 additions a lane) instead of a shuffle tree in every warp.
template <int DEPTH>
__global__ void __launch_bounds__(1024)
bk_solve_ring_kernel(const double *__restrict__ W, int64_t ld, int n, const int *__restrict__ ipiv,
                     double *__restrict__ bg, int *__restrict__ steps)
{
    constexpr int NS = DEPTH + 2;
    __shared__ double red0[1024], red1[1024], q0[4], q1[4];
    extern __shared__ double sm[];
    double *b = sm, *ring = sm + n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
    for (int i = tid; i < n; i += nt) b[i] = bg[i];
    auto slot = [&](int c) { return ring + (int64_t)(c % NS) * n; };
    auto issue = [&](int c) {
        double *dst = slot(c);
        const double *src = W + (int64_t)c * ld;
        for (int i = c + tid; i < n; i += nt) cp_async8(dst + i, src + i);
        cp_async_commit();
    };
    // ---- L x = P b (the D solves follow in one pass)
    int issued = 0;  // columns [0, issued) are in flight or arrived
    int k = 0;
    while (k < n) {
        const int p = ipiv[k];
        const bool two = p < 0;
        const int kp = two ? -p - 1 : p - 1, kk = two ? k + 1 : k;
        // keep DEPTH columns ahead of this step and wait for its own: the slots
        // refilled belong to columns before k, done with by the last barrier
        while (issued < n && issued <= kk + DEPTH) issue(issued++);
        cp_async_wait_pending(issued - 1 - kk);
        if (tid == 0) {
            steps[k] = two ? 2 : 1;
            if (two) steps[k + 1] = 0;
            if (kp != kk) {
                const double t = b[kk];
                b[kk] = b[kp];
                b[kp] = t;
            }
        }
        __syncthreads();
        const double *ck = slot(k), *ck1 = slot(k + 1);
        const double b0 = b[k], b1 = two ? b[k + 1] : 0.0;
        for (int i = kk + 1 + tid; i < n; i += nt) {
            if (two) b[i] -= ck[i] * b0 + ck1[i] * b1;
            else b[i] -= ck[i] * b0;
        }
        __syncthreads();
        k = kk + 1;
    }
    // ---- D x = b, every pivot block at once
    for (int c = tid; c < n; c += nt) {
        const int t = steps[c];
        if (t == 1) {
            b[c] = b[c] / W[(int64_t)c * ld + c];
        } else if (t == 2) {
            const double akm1k = W[(int64_t)(c + 1) * ld + c];
            const double akm1 = W[(int64_t)c * ld + c] / akm1k;
            const double ak = W[(int64_t)(c + 1) * ld + c + 1] / akm1k;
            const double denom = akm1 * ak - 1.0;
            const double bkm1 = b[c] / akm1k, bk = b[c + 1] / akm1k;
            b[c] = (ak * bkm1 - bk) / denom;
            b[c + 1] = (akm1 * bk - bkm1) / denom;
        }
    }
    // ---- L^T x = b, from the last step back
    cp_async_wait_pending(0);
    __syncthreads();
    auto first_col = [&](int k) { return ipiv[k] < 0 ? k - 1 : k; };
    int low = n;  // columns [low, n) issued for this pass
    if (n > 0) {
        const int c0 = first_col(n - 1);
        while (low > 0 && low > c0 - DEPTH) issue(--low);
        cp_async_wait_pending(c0 - low);
        __syncthreads();
    }
    k = n - 1;
    while (k >= 0) {
        const bool two = ipiv[k] < 0;
        const int c = two ? k - 1 : k;
        const int kp = (two ? -ipiv[k] : ipiv[k]) - 1;
        const double *ck = slot(k), *cc = slot(c);
        double s0 = 0.0, s1 = 0.0;
        for (int i = k + 1 + tid; i < n; i += nt) {
            const double bi = b[i];
            s1 += ck[i] * bi;
            if (two) s0 += cc[i] * bi;
        }
        red1[tid] = s1;
        if (two) red0[tid] = s0;
        __syncthreads();  // also: every thread is done with this step's slots
        const int kn = c - 1;
        if (warp < 4) {
            // four warps (one per scheduler's FP64 pipe) reduce a quarter each,
            // then the first of them the four sums
            double a0 = 0.0, a1 = 0.0;
            for (int j = warp * (nt >> 2) + lane; j < (warp + 1) * (nt >> 2); j += 32) {
                a1 += red1[j];
                if (two) a0 += red0[j];
            }
            for (int off = 16; off > 0; off >>= 1) {
                a1 += __shfl_xor_sync(0xffffffffu, a1, off);
                if (two) a0 += __shfl_xor_sync(0xffffffffu, a0, off);
            }
            if (lane == 0) {
                q1[warp] = a1;
                q0[warp] = a0;
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (tid == 0) {
                b[k] -= (q1[0] + q1[1]) + (q1[2] + q1[3]);
                if (two) b[k - 1] -= (q0[0] + q0[1]) + (q0[2] + q0[3]);
                if (kp != k) {
                    const double t = b[k];
                    b[k] = b[kp];
                    b[kp] = t;
                }
            }
        }
        if (kn >= 0) {
            const int cn = first_col(kn);
            while (low > 0 && low > cn - DEPTH) issue(--low);
            cp_async_wait_pending(cn - low);
        }
        __syncthreads();
        k = kn;
    }
    cp_async_wait_pending(0);
    __syncthreads();
    for (int i = tid; i < n; i += nt) bg[i] = b[i];
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

__global__ void bk_extract_kernel(const double *__restrict__ W, int n, const int *__restrict__ cpos,
                                  double *__restrict__ Ainv,
                                  int64_t ldi)
{
    const int N = 2 * n;
    const int64_t total = (int64_t)n * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const int pi = cpos[i], pj = cpos[j];  // the coupling positions of i and j
        const int hi = pi > pj ? pi : pj, lo = pi > pj ? pj : pi;
        Ainv[(int64_t)i + (int64_t)j * ldi] = -W[(int64_t)(n + hi) * N + (n + lo)];
    }
}

// r = y - A x in FP64 for the refinement step of the blocked solve, A the caller's
// column-major lower triangle (lda).  Lower part with the diagonal: 256-row blocks
// against 256-column chunks (column loads coalesced across the rows), partial sums
// per chunk in P[chunk][row]; strictly upper part: one warp per column j dotting
// column j below the diagonal with x.  The order of summation is fixed.
constexpr int BK_RES_T = 256;

__global__ void __launch_bounds__(BK_RES_T)
bk_resid_lower_kernel(const double *__restrict__ A, int64_t lda, int n, const double *__restrict__ x,
                      double *__restrict__ P)
{
    __shared__ double xs[BK_RES_T];
    const int rb = blockIdx.x, cb = blockIdx.y;
    if (cb > rb) return;
    const int i = rb * BK_RES_T + threadIdx.x, j0 = cb * BK_RES_T;
    const int j1 = min(n, j0 + BK_RES_T);
    if (j0 + (int)threadIdx.x < n) xs[threadIdx.x] = x[j0 + threadIdx.x];
    __syncthreads();
    if (i >= n) return;
    const int je = min(j1, i + 1);
    double s = 0.0;
    for (int j = j0; j < je; ++j) s = fma(A[(int64_t)i + (int64_t)j * lda], xs[j - j0], s);
    P[(int64_t)cb * n + i] = s;
}

__global__ void bk_resid_upper_kernel(const double *__restrict__ A, int64_t lda, int n,
                                      const double *__restrict__ x, double *__restrict__ U)
{
    const int lane = threadIdx.x & 31;
    const int j = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    if (j >= n) return;
    const double *col = A + (int64_t)j * lda;
    double s = 0.0;
    for (int i = j + 1 + lane; i < n; i += 32) s = fma(col[i], x[i], s);
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) U[j] = s;
}

// r = y - (sum of the chunks in order + the upper part)
__global__ void bk_resid_finish_kernel(int n, const double *__restrict__ y, const double *__restrict__ P,
                                       const double *__restrict__ U, double *__restrict__ r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = 0.0;
    for (int cb = 0; cb <= i / BK_RES_T; ++cb) s += P[(int64_t)cb * n + i];
    r[i] = y[i] - (s + U[i]);
}

__global__ void bk_axpy_kernel(int n, const double *__restrict__ d, double *__restrict__ x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += d[i];
}

constexpr int BK_MAX_GRID = 1024;

struct BkBufs {
    int *info, *dec, *ipiv, *pi, *kb, *err, *expo, *perm, *cpos, *corig, *srcmap, *aff, *naff;
    double *W, *col, *ci, *p0, *p1, *w0, *w1, *sc, *pv, *pv2, *Wp, *stage, *ctmp, *ctmpw, *rP, *rU, *rr;
    bool blocked = false;
    __nv_bfloat16 *dig;
};

constexpr int BK_SLICES = 8;

// Digit-plane rows: the L21 rows at 0, the W21 rows at plane_rows(N).
int bk_plane_rows(int N) { return 2 * qmlg::plane_rows(N); }

size_t bk_ws(int n, int N)
{
    qmlg::WorkspacePlan p;
    p.add<int>(4);
    p.add<int>(4);
    p.add<int>((size_t)std::max(n, 1));
    p.add<double>((size_t)N * N);
    p.add<double>((size_t)4 * N);
    for (int v = 0; v < 5; ++v) p.add<double>((size_t)N);
    p.add<double>(4);
    p.add<double>(BK_MAX_GRID);
    p.add<int>(BK_MAX_GRID);
    // the blocked form
    p.add<double>(BK_MAX_GRID);
    p.add<double>((size_t)N * BK_NB);
    p.add<double>(2 * BK_NB);
    p.add<int>(4);
    p.add<int>(4);
    p.add<int>((size_t)bk_plane_rows(N));
    p.add<__nv_bfloat16>((size_t)BK_SLICES * bk_plane_rows(N) * BK_NB);
    for (int v = 0; v < 5; ++v) p.add<int>((size_t)std::max(n, 1));  // perm, cpos, corig, srcmap, aff
    p.add<int>(4);
    p.add<double>((size_t)2 * BK_NB * N);
    p.add<double>((size_t)2 * BK_NB * BK_NB);
    // the solve's refinement: chunk partials, upper part, residual
    p.add<double>((size_t)qmlg::ceil_div(std::max(n, 1), BK_RES_T) * std::max(n, 1));
    p.add<double>((size_t)std::max(n, 1));
    p.add<double>((size_t)std::max(n, 1));
    return p.total();
}

// The blocked factorisation (N > 256, cooperative launches allowed): per panel the
// panel kernel, the trailing update, and (undo) the L columns put in dsytf2's form.
// exact: the trailing update in FP64, else as an emulated-FP64 product.  The
// emulated product is fixed point per row (each row scaled to its largest entry),
// which is as accurate as FP64 where the rows are bounded, as the pivoting bounds
// L for the solve.  The rows of the inverse's coupling block are not bounded (they
// become rows of -A^-1): on the reference's 200 x 200 fixture (condition 4.4e9) the
// emulated update gave max|A A^-1 - I| = 4.9e-2 against LAPACK's 1.4e-8, the FP64
// update 2.4e-8, so the inverse takes the FP64 update.
int bk_factor_blocked(BkBufs &b, int n, int N, int grid, bool undo, bool exact, cudaStream_t s)
{
    BkPanelArgs pa{b.W, (int64_t)N, N, n, 0, b.Wp, b.stage, b.ipiv, b.info, b.pv, b.pv2, b.pi, b.kb,
                   nullptr};
    const int rpad = bk_plane_rows(N), roff = qmlg::plane_rows(N);
    cudaError_t e = cudaMemsetAsync(b.err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const bool coupled = N > n;  // the maps were set to the identity by bk_factor
    if (coupled) pa.perm = b.perm;
    int st = QMLG_OK;
    for (int k0 = 0; k0 < n;) {
        pa.k0 = k0;
        void *args[] = {(void *)&pa};
        st = qmlg::launch_cooperative_serialised((const void *)bk_panel_kernel, grid, BK_THREADS, args, s);
        if (st != QMLG_OK) return st;
        int kb = 0;
        if ((st = qmlg::read_back(&kb, b.kb, sizeof(int), s)) != QMLG_OK) return st;
        if (kb < 1 || kb > BK_NB || k0 + kb > n) return QMLG_E_CUDA;
        const int k1 = k0 + kb;
        if (coupled) {
            // the coupling rows pivoted in this panel to positions [k0, k1)
            bk_compact_plan_kernel<<<1, 32, 0, s>>>(b.perm, k0, k1, b.cpos, b.corig, b.srcmap, b.aff, b.naff);
            const dim3 cg((unsigned)std::min<int64_t>(qmlg::ceil_div(N, 256), 64), 2 * BK_NB);
            bk_compact_gather_kernel<<<cg, 256, 0, s>>>(b.W, N, N, n, b.Wp, b.aff, b.naff, b.srcmap, b.ctmp,
                                                        b.ctmpw);
            bk_compact_scatter_kernel<<<cg, 256, 0, s>>>(b.W, N, N, n, b.Wp, b.aff, b.naff, b.srcmap, b.ctmp,
                                                         b.ctmpw);
            qmlg::count_launches(3);
            if ((st = qmlg::check_launch()) != QMLG_OK) return st;
        }
        // the live rows end at n + k1 (the coupling rows not yet pivoted are zero)
        const int ne = coupled ? std::min(N, n + k1) : N;
        if (k1 < ne && exact) {
            const int64_t t = qmlg::ceil_div(ne - k1, 64);
            bk_update_fp64_kernel<<<(unsigned)(t * (t + 1) / 2), 256, 0, s>>>(b.W, N, ne, k0, k1, kb, b.Wp);
            qmlg::count_launches(1);
            if ((st = qmlg::check_launch()) != QMLG_OK) return st;
        } else if (k1 < N) {
            st = qmlg::slice_rows(b.W, N, k1, N - k1, k0, kb, BK_NB, rpad, BK_SLICES, b.dig, b.expo,
                                  nullptr, s);
            if (st == QMLG_OK)
                st = qmlg::slice_rows(b.Wp, BK_NB, k1, N - k1, 0, kb, BK_NB, rpad, BK_SLICES,
                                      b.dig + (size_t)roff * BK_NB, b.expo + roff, nullptr, s);
            if (st == QMLG_OK)
                st = qmlg::emu_tc_update(b.W, N, k1, N, k1, N, b.dig, b.expo, BK_NB, rpad, BK_SLICES,
                                         roff, 0, 1, b.err, s);
            if (st != QMLG_OK) return st;
        }
        if (undo) {
            bk_panel_undo_kernel<<<1, BK_NB, 0, s>>>(b.W, N, k0, b.kb, b.ipiv);
            qmlg::count_launches(1);
            if ((st = qmlg::check_launch()) != QMLG_OK) return st;
        }
        k0 = k1;
    }
    return qmlg::read_device_flag(b.err, s);
}

int bk_factor(const double *A, int64_t lda, int n, int N, void *workspace, size_t ws_bytes,
              BkBufs &b, bool undo, bool exact, cudaStream_t s)
{
    if (ws_bytes < bk_ws(n, N)) return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    b.info = ws.take<int>(4);
    b.dec = ws.take<int>(4);
    b.ipiv = ws.take<int>((size_t)std::max(n, 1));
    b.W = ws.take<double>((size_t)N * N);
    b.col = ws.take<double>((size_t)4 * N);
    b.ci = ws.take<double>((size_t)N);
    b.p0 = ws.take<double>((size_t)N);
    b.p1 = ws.take<double>((size_t)N);
    b.w0 = ws.take<double>((size_t)N);
    b.w1 = ws.take<double>((size_t)N);
    b.sc = ws.take<double>(4);
    b.pv = ws.take<double>(BK_MAX_GRID);
    b.pi = ws.take<int>(BK_MAX_GRID);
    b.pv2 = ws.take<double>(BK_MAX_GRID);
    b.Wp = ws.take<double>((size_t)N * BK_NB);
    b.stage = ws.take<double>(2 * BK_NB);
    b.kb = ws.take<int>(4);
    b.err = ws.take<int>(4);
    b.expo = ws.take<int>((size_t)bk_plane_rows(N));
    b.dig = ws.take<__nv_bfloat16>((size_t)BK_SLICES * bk_plane_rows(N) * BK_NB);
    b.perm = ws.take<int>((size_t)std::max(n, 1));
    b.cpos = ws.take<int>((size_t)std::max(n, 1));
    b.corig = ws.take<int>((size_t)std::max(n, 1));
    b.srcmap = ws.take<int>((size_t)std::max(n, 1));
    b.aff = ws.take<int>((size_t)std::max(n, 1));
    b.naff = ws.take<int>(4);
    b.ctmp = ws.take<double>((size_t)2 * BK_NB * N);
    b.ctmpw = ws.take<double>((size_t)2 * BK_NB * BK_NB);
    b.rP = ws.take<double>((size_t)qmlg::ceil_div(std::max(n, 1), BK_RES_T) * std::max(n, 1));
    b.rU = ws.take<double>((size_t)std::max(n, 1));
    b.rr = ws.take<double>((size_t)std::max(n, 1));
    cudaError_t e = cudaMemsetAsync(b.info, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const int blocks = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)N * N, 256), 152 * 64);
    { bk_build_kernel<<<blocks, 256, 0, s>>>(A, lda, n, N, b.W); qmlg::count_launches(1); }
    if (N > n) {  // the inverse: coupling positions start as the identity
        bk_coupling_init_kernel<<<(unsigned)qmlg::ceil_div(n, 256), 256, 0, s>>>(b.perm, b.cpos, b.corig,
                                                                                 b.srcmap, n, b.naff);
        qmlg::count_launches(1);
    }
    int grid = 1;
    if (N > 256 && qmlg::cooperative_allowed_on(s)) {
        int dev = 0, sms = 0, per = 0, per2 = 0;
        if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, bk_factor_kernel, BK_THREADS, 0)) !=
                cudaSuccess ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per2, bk_panel_kernel, BK_THREADS, 0)) !=
                cudaSuccess)
            return qmlg::set_cuda_error(e);
        const int lim = qmlg::sm_limit(sms);
        grid = std::max(1, std::min({lim, sms * std::max(std::min(per, per2), 1), BK_MAX_GRID}));
    }
    b.blocked = grid > 1;
    if (grid > 1) return bk_factor_blocked(b, n, N, grid, undo, exact, s);
    BkArgs a{b.W, (int64_t)N, N, n, b.ipiv, b.info, b.col, b.ci, b.p0, b.p1, b.w0, b.w1, b.sc, b.pv, b.pi, b.dec};
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
    int st = bk_factor(A, lda, n, n, workspace, ws_bytes, b, true, false, s);
    if (st != QMLG_OK) return st;
    cudaError_t e = cudaMemcpyAsync(x, y, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    if (n > 1) {
        const int64_t t = qmlg::ceil_div(n, 32);
        bk_transpose_kernel<<<(unsigned)(t * (t + 1) / 2), 256, 0, s>>>(b.W, n, n);
        qmlg::count_launches(1);
    }
    // dsytrs on v in place with the factor (and L^T above its diagonal)
    auto dsytrs = [&](double *v) -> int {
        const size_t ring2 = sizeof(double) * 5 * (size_t)n;
        // the kernel's 16 KB of static shared memory counts too
        if (ring2 + 18 * 1024 <= (size_t)227 * 1024) {
            if ((e = cudaFuncSetAttribute(bk_solve_ring_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)ring2)) != cudaSuccess)
                return qmlg::set_cuda_error(e);
            bk_solve_ring_kernel<2><<<1, 1024, ring2, s>>>(b.W, n, n, b.ipiv, v, reinterpret_cast<int *>(b.col));
        } else if (n <= BK_SOLVE_SMEM) {
            const size_t smem = sizeof(double) * (size_t)n;
            if ((e = cudaFuncSetAttribute(bk_solve_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)std::max<size_t>(smem, 1))) != cudaSuccess)
                return qmlg::set_cuda_error(e);
            bk_solve_kernel<true><<<1, 1024, smem, s>>>(b.W, n, n, b.ipiv, v, reinterpret_cast<int *>(b.col));
        } else {
            bk_solve_kernel<false><<<1, 1024, 0, s>>>(b.W, n, n, b.ipiv, v, reinterpret_cast<int *>(b.col));
        }
        qmlg::count_launches(1);
        return qmlg::check_launch();
    };
    if ((st = dsytrs(x)) != QMLG_OK) return st;
    int info = 0;
    if ((st = qmlg::read_back(&info, b.info, sizeof(int), s)) != QMLG_OK) return st;
    if (info == 0 && b.blocked) {
        // The blocked factor's trailing updates are emulated-FP64 products (fixed
        // point per row), whose error can exceed FP64's where a row's entries spread
        // widely (2x2 pivots everywhere: a residual 19x LAPACK's at n = 600).  One
        // step of refinement on the FP64 residual of the caller's A brings x back to
        // FP64 accuracy.
        const unsigned rb = (unsigned)qmlg::ceil_div(n, BK_RES_T);
        bk_resid_lower_kernel<<<dim3(rb, rb), BK_RES_T, 0, s>>>(A, lda, n, x, b.rP);
        bk_resid_upper_kernel<<<(unsigned)qmlg::ceil_div((int64_t)n * 32, 256), 256, 0, s>>>(A, lda, n, x, b.rU);
        bk_resid_finish_kernel<<<(unsigned)qmlg::ceil_div(n, 256), 256, 0, s>>>(n, y, b.rP, b.rU, b.rr);
        qmlg::count_launches(3);
        if ((st = qmlg::check_launch()) != QMLG_OK) return st;
        if ((st = dsytrs(b.rr)) != QMLG_OK) return st;
        bk_axpy_kernel<<<(unsigned)qmlg::ceil_div(n, 256), 256, 0, s>>>(n, b.rr, x);
        qmlg::count_launches(1);
        if ((st = qmlg::check_launch()) != QMLG_OK) return st;
        if ((st = qmlg::read_back(&info, b.info, sizeof(int), s)) != QMLG_OK) return st;
    }
    return info;
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
    int st = bk_factor(A, lda, n, 2 * n, workspace, ws_bytes, b, false, true, s);
    if (st != QMLG_OK) return st;
    const int eb = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)n * n, 256), 152 * 64);
    { bk_extract_kernel<<<eb, 256, 0, s>>>(b.W, n, b.cpos, Ainv, ldi); qmlg::count_launches(1); }
    if ((st = qmlg::check_launch()) != QMLG_OK) return st;
    int info = 0;
    st = qmlg::read_back(&info, b.info, sizeof(int), s);
    return st != QMLG_OK ? st : info;
}
